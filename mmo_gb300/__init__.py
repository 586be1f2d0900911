"""GB300-native (sm_103a) UFF ligand/protein scoring: the force-field hot path of
UnixJunkie/MMO (src/mol.ml:794-903) behind a C ABI (include/mmo_gpu.h)."""

from .topology import Mol, read_pqrs, write_pqrs  # noqa: F401

__all__ = ["Mol", "read_pqrs", "write_pqrs"]
