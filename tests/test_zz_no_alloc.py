"""The allocation-free entry point mmo_score_poses_noalloc, through the C ABI.

Some callers of the scorer cannot allocate device memory while they score: a
real-time loop that may not stall on the allocator, or a host whose device
memory belongs to another allocator (a framework's caching allocator, a fixed
arena reserved up front).  This entry point takes the same device inputs and
outputs as mmo_score_poses_device but keeps its work buffers in a static
device array.  Two calls in a row must each match the allocating entry point
within the parity tolerances (energies 1e-5 relative, gradient components
1e-4 relative with the floor at 1% of each component's sum of |terms|), over
one pose, a batch, energy only, intra only, the grid lookup and a batch near
the array's limit (where the call uses fewer protein chunks than the
allocating path); one batch is also checked against the FP64 oracle, and a
batch too large for the static array must be refused.
"""
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

    s = synth.pose_batch(n_poses=4096, seed=17)
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


def _call(sc, L, torch, dev, dofs, flags, noalloc):
    B, nd = dofs.shape
    E, G, st = _buffers(torch, dev, B, nd)
    E.fill_(np.nan)
    G.fill_(np.nan)
    fn = sc._lib.mmo_score_poses_noalloc if noalloc else sc._lib.mmo_score_poses_device
    rc = fn(sc.handle, B, dofs.data_ptr(), flags, E.data_ptr(), G.data_ptr(), st.data_ptr(), None)
    assert rc == L.OK, sc._lib.mmo_last_error(sc.handle)
    assert sc._lib.mmo_sync(sc.handle, None) == L.OK
    return E.cpu().numpy(), G.cpu().numpy(), st.cpu().numpy()


def _grad_scale(s, dofs, flags):
    """Per-component condition scales of the gradient (the oracle's
    orc_grad_scale): the floor of the gradient comparison, as in the parity
    tests, is 1% of each component's own sum of |terms|."""
    from oracle import oracle as O

    fl = (O.F_INTER if flags & 1 else 0) | (O.F_INTRA if flags & 2 else 0)
    _, GA, _ = O.score_batch(s.pocket, s.ligand, dofs.cpu().numpy(), flags=fl, mode=3,
                             nthreads=16)
    return GA


def _check(sc, L, torch, dev, dofs, flags, s):
    grad = bool(flags & L.F_GRAD)
    E0, G0, st0 = _call(sc, L, torch, dev, dofs, flags, False)
    GA = _grad_scale(s, dofs, flags) if grad else None
    for _ in range(2):  # the second call reuses the static scratch left by the first
        E, G, st = _call(sc, L, torch, dev, dofs, flags, True)
        assert np.array_equal(st, st0)
        with np.errstate(divide="ignore", invalid="ignore"):
            rel = np.where(E == E0, 0.0, np.abs(E - E0) / np.abs(E0))
        assert rel.max() <= E_TOL
        if grad:
            d = np.abs(G.astype(np.float64) - G0)
            den = np.maximum(np.abs(G0.astype(np.float64)), 0.01 * GA)
            with np.errstate(divide="ignore", invalid="ignore"):
                assert np.where(d == 0, 0.0, d / den).max() <= G_TOL
    return E, G, st


@pytest.mark.parametrize("B", [1, 1000])
@pytest.mark.parametrize("terms", ["inter+intra+grad", "inter+intra", "intra+grad"])
def test_noalloc_matches_allocating_entry_point_twice(setup, B, terms):
    sc, L, torch, dev, s = setup
    flags = {"inter+intra+grad": L.F_INTER | L.F_INTRA | L.F_GRAD,
             "inter+intra": L.F_INTER | L.F_INTRA,
             "intra+grad": L.F_INTRA | L.F_GRAD}[terms]
    dofs = torch.from_numpy(s.poses[:B]).to(dev)
    _check(sc, L, torch, dev, dofs, flags, s)


def test_noalloc_near_the_limit_with_fewer_chunks(setup):
    """4,096 poses of the 48-atom ligand with the gradient: the static array
    holds fewer protein chunks than the allocating path's plan, so the call
    runs the full sweep with its chunk count reduced."""
    sc, L, torch, dev, s = setup
    dofs = torch.from_numpy(s.poses).to(dev)
    _check(sc, L, torch, dev, dofs, L.F_INTER | L.F_INTRA | L.F_GRAD, s)


def test_noalloc_grid_lookup(setup):
    """MMO_F_GRID: the inter energy from per-type grids built for this ligand."""
    sc, L, torch, dev, s = setup
    from mmo_gb300 import grids as GR

    origin, dims = GR.lattice_from_box(0.5, (-17.0, -17.0, -17.0), (17.0, 17.0, 17.0))
    types, _ = GR.type2id([s.ligand])
    sc.build_grids(0.5, dims, origin, types)
    dofs = torch.from_numpy(s.poses[:512]).to(dev)
    _check(sc, L, torch, dev, dofs, L.F_INTER | L.F_INTRA | L.F_GRAD | L.F_GRID, s)


def test_noalloc_against_the_oracle(setup, oracle):
    """One batch of the allocation-free path against the FP64 oracle under
    the scoring contract (tests/contract.py)."""
    from contract import assert_ref, ref_batch

    sc, L, torch, dev, s = setup
    dofs = torch.from_numpy(s.poses[:1000]).to(dev)
    E, G, st = _call(sc, L, torch, dev, dofs, L.F_INTER | L.F_INTRA | L.F_GRAD, True)
    assert_ref(E, G, ref_batch(oracle, s, s.poses[:1000], grad=True), st)


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
