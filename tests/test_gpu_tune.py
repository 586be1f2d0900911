"""The autotuner (mmo_tune) of the batched pair sweep, through the C ABI.

It times launch plans on a batch, keeps the fastest and leaves the outputs
as that plan computes them; a cache file replays a plan without timing."""
import numpy as np
import pytest

from mmo_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def system():
    return synth.pose_batch(n_poses=512, seed=4)


def _device(torch, s):
    dev = torch.device("cuda", 0)
    B, nd = s.poses.shape
    return (torch.from_numpy(s.poses).to(dev), torch.empty(B, dtype=torch.float64, device=dev),
            torch.empty((B, nd), dtype=torch.float32, device=dev),
            torch.empty(B, dtype=torch.int32, device=dev))


def test_tune_picks_plan_and_keeps_results(scorer_factory, system, tmp_path):
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L

    sc = scorer_factory(system.pocket, system.ligand)
    E0, G0, st0 = sc.score_poses(system.poses, grad=True)
    d, E, G, st = _device(torch, system)
    flags = L.F_INTER | L.F_INTRA | L.F_GRAD
    cache = str(tmp_path / "plans.txt")
    sc.set_tune_cache(cache)
    ms = sc.tune_device(d.data_ptr(), len(d), E.data_ptr(), G.data_ptr(), st.data_ptr(), flags)
    assert ms > 0
    plan = sc.plan()
    assert plan["sweep"] in ("cut-off", "full")
    # the outputs left by mmo_tune, and a call after it, are the chosen plan's
    E1, G1, st1 = E.cpu().numpy(), G.cpu().numpy(), st.cpu().numpy()
    E2, G2, _ = sc.score_poses(system.poses, grad=True)
    assert np.array_equal(E1, E2) and np.array_equal(G1, G2)
    assert np.array_equal(st1, st0)
    assert np.abs(E2 - E0).max() <= 1e-6 * np.abs(E0).max()
    assert (np.abs(G2 - G0).max(axis=1) / np.abs(G0).max(axis=1)).max() <= 1e-5
    lines = [x for x in open(cache) if not x.startswith("#")]
    assert len(lines) == 1

    # a fresh context replays the recorded plan without timing
    sc2 = scorer_factory(system.pocket, system.ligand)
    sc2.set_tune_cache(cache)
    ms2 = sc2.tune_device(d.data_ptr(), len(d), E.data_ptr(), G.data_ptr(), st.data_ptr(), flags)
    assert ms2 == -1.0
    assert sc2.plan() == plan
    E3, G3, _ = sc2.score_poses(system.poses, grad=True)
    assert np.array_equal(E3, E2) and np.array_equal(G3, G2)


def test_tune_global_form(scorer_factory, system):
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L
    from mmo_gb300.ff import Physics

    sc = scorer_factory(system.pocket, system.ligand, Physics(0, 0, 1, 0))
    E0, _, _ = sc.score_poses(system.poses[:256])
    s256 = synth.System("s", system.pocket, system.ligand, system.poses[:256])
    d, E, G, st = _device(torch, s256)
    sc.tune_device(d.data_ptr(), 256, E.data_ptr(), None, st.data_ptr(), L.F_INTER | L.F_INTRA)
    assert sc.plan()["sweep"] == "full"
    assert np.abs(E.cpu().numpy() - E0).max() <= 1e-6 * np.abs(E0).max()
