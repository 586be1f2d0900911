"""Monte Carlo chains (mmo_mc_run) on the GPU, through the C ABI.

The chains' generator against the oracle's Philox4x32-10; final energies
against an FP64 re-score of the final poses; a CUDA-graph run against the
same sequence launched directly; chains that do not depend on how many run
beside them; no uphill move at kT -> 0; the move laws' step statistics."""
import ctypes as C

import numpy as np
import pytest

from mmo_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def system():
    return synth.pose_batch(n_poses=256, seed=9, n_atoms=32, n_rot=5, n_pocket=3000,
                            radius=15.0, half_box=3.0)


def _params(L, **kw):
    p = dict(kT=0.593, rot_step=np.radians(5.0), trans_step=0.3, tors_step=np.radians(30.0),
             move_law=L.MC_GAUSSIAN, adapt=0, flip_every=0, minimize_every=0, minimize_iters=0,
             gd_step=0.1, seed=1234)
    p.update(kw)
    return p


def _run(torch, sc, L, dofs0, steps, graph=True, **kw):
    dev = torch.device("cuda", 0)
    B, nd = dofs0.shape
    d = torch.from_numpy(np.ascontiguousarray(dofs0)).to(dev)
    E = torch.empty(B, dtype=torch.float64, device=dev)
    bd = torch.empty_like(d)
    bE = torch.empty_like(E)
    acc = torch.empty(B, dtype=torch.int32, device=dev)
    st = torch.empty(B, dtype=torch.int32, device=dev)
    sc.mc_run_device(B, steps, _params(L, **kw), d.data_ptr(), E.data_ptr(), bd.data_ptr(),
                     bE.data_ptr(), acc.data_ptr(), st.data_ptr(), None, graph)
    torch.cuda.synchronize()
    return tuple(x.cpu().numpy() for x in (d, E, bd, bE, acc, st))


def test_philox_matches_oracle(oracle, scorer_factory, system):
    torch = pytest.importorskip("torch")
    sc = scorer_factory(system.pocket, system.ligand)
    n = 1000
    out = torch.empty(4 * n, dtype=torch.int32, device="cuda")
    assert sc._lib.mmo_philox4x32(sc.handle, 0x1234567, 0x89ABCDEF, 77, 3, n, out.data_ptr(),
                                  None) == 0
    got = out.cpu().numpy().view(np.uint32).reshape(n, 4)
    f = oracle.lib().orc_philox4x32_10
    for i in range(0, n, 37):
        c = (C.c_uint32 * 4)(i, 77, 3, 0)
        k = (C.c_uint32 * 2)(0x1234567, 0x89ABCDEF)
        o = (C.c_uint32 * 4)()
        f(c, k, o)
        assert list(o) == list(got[i])


def test_final_energies_match_fp64_rescore(oracle, scorer_factory, system):
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L

    from contract import assert_ref, ref_batch

    sc = scorer_factory(system.pocket, system.ligand)
    d0 = system.poses[:64]
    E_start, _, _ = sc.score_poses(d0, recenter=True)
    d, E, bd, bE, acc, st = _run(torch, sc, L, d0, 120, minimize_every=40, minimize_iters=8)
    assert np.all(acc > 0) and np.all(np.isfinite(E))
    assert np.all(bE <= E_start) and np.all(bE <= E)
    # the returned energies are the scorer's energies of the returned poses
    Er, _, _ = sc.score_poses(d, recenter=True)
    assert np.array_equal(Er, E)
    Eb, _, _ = sc.score_poses(bd, recenter=True)
    assert np.array_equal(Eb, bE)
    assert_ref(E, None, ref_batch(oracle, system, d, recenter=True))


def test_graph_equals_direct_launches(scorer_factory, system):
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L

    sc = scorer_factory(system.pocket, system.ligand)
    d0 = system.poses[:48]
    a = _run(torch, sc, L, d0, 110, graph=True, minimize_every=50, minimize_iters=4, adapt=1,
             move_law=L.MC_UNIFORM, flip_every=7)
    b = _run(torch, sc, L, d0, 110, graph=False, minimize_every=50, minimize_iters=4, adapt=1,
             move_law=L.MC_UNIFORM, flip_every=7)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    c = _run(torch, sc, L, d0, 110, graph=True, minimize_every=50, minimize_iters=4, adapt=1,
             move_law=L.MC_UNIFORM, flip_every=7)  # the cached graph again
    for x, y in zip(a, c):
        assert np.array_equal(x, y)


def test_chains_independent_of_batch(scorer_factory, system):
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L

    sc = scorer_factory(system.pocket, system.ligand)
    big = _run(torch, sc, L, system.poses[:96], 60)
    small = _run(torch, sc, L, system.poses[:40], 60)
    for x, y in zip(big, small):
        assert np.array_equal(x[:40], y)


def test_cold_chains_never_go_uphill(scorer_factory, system):
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L

    sc = scorer_factory(system.pocket, system.ligand)
    d = system.poses[:64].copy()
    E_prev, _, _ = sc.score_poses(d, recenter=True)
    for k in range(4):
        d, E, bd, bE, acc, st = _run(torch, sc, L, d, 25, kT=1e-12, seed=99 + k)
        assert np.all(E <= E_prev)
        E_prev = E
    assert acc.sum() > 0


@pytest.mark.parametrize("law", ["gaussian", "uniform"])
def test_move_step_statistics(scorer_factory, system, law):
    """kT -> infinity: every clean move is accepted; after one rigid step the
    translation changes follow the move law, after the torsion step exactly
    one torsion has changed."""
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L

    sc = scorer_factory(system.pocket, system.ligand)
    rng = np.random.default_rng(3)
    d0 = np.repeat(system.poses[:1], 2048, axis=0).copy()
    d0[:, 6:] = rng.uniform(-0.2, 0.2, size=(2048, d0.shape[1] - 6)).astype(np.float32)
    mode = L.MC_GAUSSIAN if law == "gaussian" else L.MC_UNIFORM
    d1, _, _, _, acc1, st1 = _run(torch, sc, L, d0, 1, kT=1e30, move_law=mode, trans_step=0.3)
    ok = (acc1 == 1)
    assert ok.mean() > 0.95
    dt = (d1[ok, :3] - d0[ok, :3]).ravel()
    want = 0.3 if law == "gaussian" else 0.3 / np.sqrt(3.0)
    assert abs(dt.std() / want - 1.0) < 0.05
    assert np.all(d1[ok, 6:] == d0[ok, 6:])
    d2, _, _, _, acc2, _ = _run(torch, sc, L, d0, 2, kT=1e30, move_law=mode, trans_step=0.3)
    both = acc2 == 2
    changed = (d2[both, 6:] != d1[both, 6:]).sum(axis=1)
    assert np.all(changed == 1)
