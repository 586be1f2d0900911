"""The allocation-free entry point mmo_score_poses_noalloc, through the C ABI.

Some callers of the scorer cannot allocate device memory while they score (a
CUDA stream capture in progress, a real-time loop that may not stall on the
allocator, a host whose device memory belongs to another allocator).  This
entry point takes the same device inputs and outputs as
mmo_score_poses_device but keeps its work buffers in a static device array.
Two calls in a row must each match the allocating entry point within the
parity tolerances (energies 1e-5 relative, gradients 1e-4 of the largest
component), and a batch too large for the static array must be refused.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E_TOL = 1e-5
G_TOL = 1e-4


@pytest.fixture(scope="module")
def setup():
    import torch

    from mmo_gb300 import lib as L
    from mmo_gb300 import synth
    from mmo_gb300.ff import UFFScorer

    s = synth.pose_batch(n_poses=1000, seed=17)
    sc = UFFScorer(0)
    sc.set_protein(s.pocket)
    sc.set_ligand(s.ligand)
    dev = torch.device("cuda", 0)
    yield sc, L, torch, dev, s
    sc.close()


def _buffers(torch, dev, B, nd):
    return (torch.empty(B, dtype=torch.float64, device=dev),
            torch.empty((B, nd), dtype=torch.float32, device=dev),
            torch.empty(B, dtype=torch.int32, device=dev))


def _reference(sc, L, torch, dev, dofs, flags):
    B, nd = dofs.shape
    E, G, st = _buffers(torch, dev, B, nd)
    rc = sc._lib.mmo_score_poses_device(sc.handle, B, dofs.data_ptr(), flags, E.data_ptr(),
                                        G.data_ptr(), st.data_ptr(), None)
    assert rc == L.OK
    assert sc._lib.mmo_sync(sc.handle, None) == L.OK
    return E.cpu().numpy(), G.cpu().numpy(), st.cpu().numpy()


@pytest.mark.parametrize("grad", [True, False])
def test_noalloc_matches_allocating_entry_point_twice(setup, grad):
    sc, L, torch, dev, s = setup
    flags = L.F_INTER | L.F_INTRA | (L.F_GRAD if grad else 0)
    dofs = torch.from_numpy(s.poses).to(dev)
    B, nd = dofs.shape
    E0, G0, st0 = _reference(sc, L, torch, dev, dofs, flags)
    for _ in range(2):  # the second call reuses the static scratch left by the first
        E, G, st = _buffers(torch, dev, B, nd)
        E.fill_(np.nan)
        G.fill_(np.nan)
        rc = sc._lib.mmo_score_poses_noalloc(sc.handle, B, dofs.data_ptr(), flags, E.data_ptr(),
                                             G.data_ptr(), st.data_ptr(), None)
        assert rc == L.OK, sc._lib.mmo_last_error(sc.handle)
        assert sc._lib.mmo_sync(sc.handle, None) == L.OK
        E, G, st = E.cpu().numpy(), G.cpu().numpy(), st.cpu().numpy()
        assert np.array_equal(st, st0)
        assert (np.abs(E - E0) / np.abs(E0)).max() <= E_TOL
        if grad:
            err = np.abs(G - G0).max(axis=1) / np.abs(G0).max(axis=1)
            assert err.max() <= G_TOL


def test_noalloc_rejects_batch_beyond_static_scratch(setup):
    sc, L, torch, dev, s = setup
    dofs = torch.from_numpy(s.poses[:1]).to(dev)
    E, G, st = _buffers(torch, dev, 1, dofs.shape[1])
    # 200,000 poses of 48 atoms need far more than the 32 MiB static array; the
    # size check refuses the call before any launch touches the buffers
    rc = sc._lib.mmo_score_poses_noalloc(sc.handle, 200000, dofs.data_ptr(),
                                         L.F_INTER | L.F_INTRA | L.F_GRAD, E.data_ptr(),
                                         G.data_ptr(), st.data_ptr(), None)
    assert rc == L.EINVAL
    msg = sc._lib.mmo_last_error(sc.handle).decode()
    assert "static scratch" in msg and "200000" in msg
