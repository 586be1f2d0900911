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


# -- step by step against the oracle ------------------------------------------------

def _run_trace(torch, sc, L, dofs0, steps, **kw):
    """A run with its trace: (final dofs, E, resets, trial [steps, B, nd],
    E_trial [steps, B], event [steps, B])."""
    dev = torch.device("cuda", 0)
    B, nd = dofs0.shape
    d = torch.from_numpy(np.ascontiguousarray(dofs0)).to(dev)
    E = torch.empty(B, dtype=torch.float64, device=dev)
    res = torch.zeros(B, dtype=torch.int32, device=dev)
    tr = torch.zeros((steps, B, nd), dtype=torch.float32, device=dev)
    tE = torch.zeros((steps, B), dtype=torch.float64, device=dev)
    tev = torch.zeros((steps, B), dtype=torch.int32, device=dev)
    sc.mc_run_device(B, steps, _params(L, **kw), d.data_ptr(), E.data_ptr(), graph=True,
                     d_resets=res.data_ptr(), d_trace_dofs=tr.data_ptr(),
                     d_trace_E=tE.data_ptr(), d_trace_event=tev.data_ptr())
    torch.cuda.synchronize()
    return tuple(x.cpu().numpy() for x in (d, E, res, tr, tE, tev))


def _oracle_params(kw):
    return dict(kT=kw["kT"], rot=kw["rot_step"], trans=kw["trans_step"], tors=kw["tors_step"],
                law=kw["move_law"], adapt=kw["adapt"], flip_every=kw["flip_every"],
                seed=kw["seed"], roi_c=kw.get("roi_center", (0.0, 0.0, 0.0)),
                roi_r=kw.get("roi_radius", 0.0), reset_zero=kw.get("reset_on_zero_inter", 0),
                too_long_ends=kw.get("too_long_ends_chain", 0))


@pytest.mark.parametrize("law", ["uniform", "gaussian"])
def test_every_step_replays_in_the_oracle(oracle, scorer_factory, system, law):
    """900 frames of 24 chains, traced: every trial pose equals the oracle's
    proposal from the chain's state bit for bit (Philox draws, move laws, the
    flip cadence, step sizes adapted from the sliding windows); every outcome
    (accepted, rejected, reset to the start) equals the oracle's FP64 outcome
    except where the energies' tolerance straddles the Metropolis threshold;
    hard-ROI and E_inter = 0 resets and the step-size adaptation all occur.
    Four of the chains start 60 A from the pocket (E_inter = 0, a reset every
    frame)."""
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L

    sc = scorer_factory(system.pocket, system.ligand)
    d0 = system.poses[:24].copy()
    d0[20:, :3] += 60.0
    kw = _params(L, move_law=L.MC_UNIFORM if law == "uniform" else L.MC_GAUSSIAN, adapt=1,
                 flip_every=100, rot_step=np.radians(15.0), trans_step=0.15,
                 tors_step=np.radians(5.0), roi_center=(0.0, 0.0, 0.0), roi_radius=4.2,
                 reset_on_zero_inter=1, seed=4321)
    steps = 900
    d, E, res, tr, tE, tev = _run_trace(torch, sc, L, d0, steps, **kw)
    r = oracle.mc_replay(system.pocket, system.ligand, _oracle_params(kw), d0, tr, tE, tev,
                         e_tol=1e-5, nthreads=16)
    n = steps * len(d0)
    assert r["proposals"] == r["decisions"] == n
    assert r["proposal_mismatch"] == 0, r
    assert r["decision_mismatch"] == 0, r
    assert r["ambiguous"] <= 0.02 * n, r
    assert r["max_rel_err_E"] <= 1e-5, r
    assert np.all(tev[:, 20:] == L.MC_RESET)  # far chains: E_inter = 0 every frame
    assert res[:20].sum() > 0  # hard-ROI resets among the pocket chains
    assert r["resets"] == res.sum()
    assert r["adapt_events"] > 0
    assert ((tev[:, :20] & L.MC_ACCEPTED) > 0).mean() > 0.05


def test_over_long_conformer_ends_the_chain(oracle, scorer_factory):
    """too_long_ends_chain: the first over-long trial conformer ends a chain
    (the reference's Mol.Too_long leaves its frame loop), later frames keep
    its pose; without it the trial is rejected and the chain goes on."""
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L
    from mmo_gb300.topology import build_ligand

    n = 22
    xyz = np.array([[i * 1.22, 0.8 * (i % 2), 0.0] for i in range(n)])
    lig = build_ligand("chain", xyz - xyz.mean(0), np.zeros(n), np.full(n, 6, np.int32),
                       [(i, i + 1) for i in range(n - 1)])
    pocket = synth.random_pocket(np.random.default_rng(2), 600, 12.0)
    sc = scorer_factory(pocket, lig)
    d0 = np.zeros((16, 6 + lig.nrb), np.float32)
    d0[:, 6 + 9] = 1.85  # one fold: 11.9 A from the centroid, a random flip often unfolds it
    d0[:, :3] = 30.0     # away from the pocket atoms
    kw = _params(L, move_law=L.MC_UNIFORM, flip_every=1, kT=1e30, too_long_ends_chain=1,
                 seed=77)
    steps = 60
    d, E, res, tr, tE, tev = _run_trace(torch, sc, L, d0, steps, **kw)
    ended = (tev & L.MC_STOPPED) > 0
    assert ended.any(axis=0).sum() >= 8
    for b in range(16):
        if ended[:, b].any():
            k = int(np.argmax(ended[:, b]))
            assert np.all(ended[k:, b])
            assert np.array_equal(d[b], tr[-1, b])  # the pose stays from then on
    r = oracle.mc_replay(pocket, lig, _oracle_params(kw), d0, tr, tE, tev, nthreads=16)
    assert r["proposal_mismatch"] == 0 and r["decision_mismatch"] == 0, r
    kw2 = dict(kw, too_long_ends_chain=0)
    _, _, _, tr2, tE2, tev2 = _run_trace(torch, sc, L, d0, steps, **kw2)
    assert not np.any(tev2 & L.MC_STOPPED) and np.any(tev2 & L.MC_BLOCKED)
    r = oracle.mc_replay(pocket, lig, _oracle_params(kw2), d0, tr2, tE2, tev2, nthreads=16)
    assert r["proposal_mismatch"] == 0 and r["decision_mismatch"] == 0, r
