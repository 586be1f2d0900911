"""The C-ABI library builds, loads and exports every symbol include/*.h
declares; argument errors come back as status codes (CPU only: no compute)."""
import ctypes as C
import glob
import os
import re

import numpy as np

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"\b(mmo_[a-z_0-9]+)\s*\(", src)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("mmo_ctx_create", "mmo_set_protein", "mmo_set_ligand", "mmo_ene_inter",
              "mmo_ene_intra", "mmo_score_poses", "mmo_score_poses_device"):
        assert n in names


def test_library_exports_every_declared_symbol(gpu_lib):
    for n in declared_functions():
        assert hasattr(gpu_lib, n), n


def test_python_binding_covers_header(gpu_lib):
    from mmo_gb300 import lib

    assert set(declared_functions()) == set(lib.SIGNATURES)


def test_null_context_is_rejected(gpu_lib):
    from mmo_gb300 import lib

    assert gpu_lib.mmo_ctx_destroy(None) == lib.EINVAL
    assert gpu_lib.mmo_set_physics(None, 0, 0, 0, 0) == lib.EINVAL
    assert gpu_lib.mmo_score_poses(None, 1, None, 0, None, None, None) == lib.EINVAL
    assert gpu_lib.mmo_sync(None, None) == lib.EINVAL
    assert gpu_lib.mmo_ctx_create(0, None) == lib.EINVAL
    assert gpu_lib.mmo_mc_run(None, 1, 1, None, None, None, 1) == lib.EINVAL
    assert gpu_lib.mmo_tune(None, 1, None, 0, None, None, None, None, None) == lib.EINVAL
    assert gpu_lib.mmo_build_grids(None, None, None) == lib.EINVAL
    assert gpu_lib.mmo_load_grids(None, None, None) == lib.EINVAL
    assert gpu_lib.mmo_set_grid_build(None, 1) == lib.EINVAL
    assert gpu_lib.mmo_build_masks(None, None, 1.4) == lib.EINVAL
    assert gpu_lib.mmo_clash_poses(None, 1, None, 0, 7, None) == lib.EINVAL
    assert gpu_lib.mmo_dock_exhaustive(None, None, None, None, None) == lib.EINVAL
    assert gpu_lib.mmo_place_in_roi(None, None, 1.0, 1, 0, None, None) == lib.EINVAL
    assert gpu_lib.mmo_protein_desolv(None, None, 1.0, None) == lib.EINVAL
    assert gpu_lib.mmo_so3_rotations(-1, None) == lib.EINVAL
    assert gpu_lib.mmo_grid_values(None, None) == lib.EINVAL
    assert gpu_lib.mmo_grid_dims(None, None, None, None, None) == lib.EINVAL
    assert gpu_lib.mmo_grid_device(None, None) == lib.EINVAL
    assert gpu_lib.mmo_grid_atom_types(None, None) == lib.EINVAL


def test_create_without_gpu_fails_cleanly(gpu_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from mmo_gb300 import lib

    h = C.c_void_p()
    rc = gpu_lib.mmo_ctx_create(0, C.byref(h))
    assert rc in (lib.ECUDA, lib.EINVAL)
    assert not h.value
    assert gpu_lib.mmo_last_error(None)


def test_no_cpu_fallback_when_library_missing(tmp_path):
    from mmo_gb300 import lib

    saved = lib._lib
    try:
        lib._lib = None
        with pytest.raises(RuntimeError, match="not built"):
            lib.load(str(tmp_path / "absent.so"))
    finally:
        lib._lib = saved


def test_so3_rotations_need_no_gpu(gpu_lib):
    """mmo_so3_rotations is host arithmetic: proper rotations, the paper's
    first sample."""
    from mmo_gb300.ff import so3_rotations

    R = so3_rotations(16)
    for M in R:
        assert np.allclose(M @ M.T, np.eye(3), atol=1e-12) and np.linalg.det(M) > 0
    assert not np.allclose(R[0], R[1])
