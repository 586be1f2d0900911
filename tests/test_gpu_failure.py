"""The bounded device-side waits give up cleanly.

The pair sweeps copy protein atoms into shared memory with the TMA bulk
engine and wait on an mbarrier with a bounded number of polls.  Here the
first wait's bound is set to 0 (mmo_diag_set_wait_polls), so every CTA gives
up at once: it sets the device-side error flag, waits once more with the
default bound for its copy in flight (which lands), and returns.  Nothing is
left waiting, nothing faults; mmo_sync reports MMO_ETIMEOUT, and once the
bound is restored the next call is clean and equals the FP64 oracle.  This
covers the cut-off sweep, the full sweep and the ragged systems sweep."""
import numpy as np
import pytest

from contract import assert_ref, ref_batch
from mmo_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def system():
    return synth.pose_batch(n_poses=256, seed=1)


def _score_device(sc, L, torch, d, flags):
    dev = torch.device("cuda", 0)
    B, nd = d.shape
    dofs = torch.from_numpy(d).to(dev)
    E = torch.zeros(B, dtype=torch.float64, device=dev)
    G = torch.zeros((B, nd), dtype=torch.float32, device=dev)
    st = torch.zeros(B, dtype=torch.int32, device=dev)
    rc = sc._lib.mmo_score_poses_device(sc.handle, B, dofs.data_ptr(), flags, E.data_ptr(),
                                        G.data_ptr(), st.data_ptr(), None)
    assert rc == L.OK, sc._lib.mmo_last_error(sc.handle)
    return sc._lib.mmo_sync(sc.handle, None), E.cpu().numpy(), G.cpu().numpy(), \
        st.cpu().numpy()


@pytest.mark.parametrize("sweep", ["cut-off", "full"])
def test_wait_that_gives_up_reports_timeout(oracle, scorer_factory, system, sweep):
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L

    sc = scorer_factory(system.pocket, system.ligand)
    if sweep == "full":
        sc.set_cull(mode=1)
    flags = L.F_INTER | L.F_INTRA | L.F_GRAD
    d = system.poses
    rc, E0, G0, st0 = _score_device(sc, L, torch, d, flags)
    assert rc == L.OK
    assert sc._lib.mmo_diag_set_wait_polls(sc.handle, 0) == L.OK
    try:
        rc, _, _, _ = _score_device(sc, L, torch, d, flags)
        assert rc == L.ETIMEOUT
        assert b"gave up" in sc._lib.mmo_last_error(sc.handle)
    finally:
        assert sc._lib.mmo_diag_set_wait_polls(sc.handle, -1) == L.OK
    # the flag was cleared by the report; the context scores as before
    rc, E, G, st = _score_device(sc, L, torch, d, flags)
    assert rc == L.OK
    assert np.array_equal(E, E0) and np.array_equal(G, G0) and np.array_equal(st, st0)
    assert_ref(E, G, ref_batch(oracle, system, d, grad=True), st)


def test_systems_sweep_wait_that_gives_up(oracle, scorer_factory):
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L

    systems = [synth.ragged_system(i, seed=3, poses_per=16) for i in range(3)]
    sc = scorer_factory()
    sc.set_systems([(s.pocket, s.ligand, len(s.poses)) for s in systems])
    packed = np.concatenate([s.poses.ravel() for s in systems]).astype(np.float32)
    E0, G0, _ = sc.score_systems(packed, grad=True)
    assert sc._lib.mmo_diag_set_wait_polls(sc.handle, 0) == L.OK
    try:
        dev = torch.device("cuda", 0)
        B = sum(len(s.poses) for s in systems)
        d_dofs = torch.from_numpy(packed).to(dev)
        d_E = torch.zeros(B, dtype=torch.float64, device=dev)
        d_G = torch.zeros(len(packed), dtype=torch.float32, device=dev)
        d_st = torch.zeros(B, dtype=torch.int32, device=dev)
        sc.score_systems_device(d_dofs.data_ptr(), d_E.data_ptr(), d_G.data_ptr(),
                                d_st.data_ptr(), L.F_INTER | L.F_INTRA | L.F_GRAD, None)
        assert sc._lib.mmo_sync(sc.handle, None) == L.ETIMEOUT
    finally:
        assert sc._lib.mmo_diag_set_wait_polls(sc.handle, -1) == L.OK
    E, G, _ = sc.score_systems(packed, grad=True)
    assert np.array_equal(E, E0) and np.array_equal(G, G0)
    po, do = sc.systems_layout()
    for k, s in enumerate(systems):
        g = G[do[k]:do[k + 1]].reshape(len(s.poses), -1)
        assert_ref(E[po[k]:po[k + 1]], g, ref_batch(oracle, s, s.poses, grad=True))
