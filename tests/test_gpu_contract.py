"""The scoring contract (tests/contract.py) on the benchmark workloads, every
pose: 4,096 poses of energy + gradient (the 48-atom, 8-torsion ligand against
the 6,000-atom pocket), the same poses one per call, the gradient against FP64
central differences, and 8,192 of the 65,536 energy-only poses."""
import numpy as np
import pytest

from contract import (E_TOL, G_FLOOR, G_TOL, assert_energy, assert_grad, assert_ref,
                      energy_errors, fd_check, grad_errors, ref_batch)
from mmo_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg2():
    return synth.pose_batch(n_poses=4096, seed=1)


@pytest.fixture(scope="module")
def cfg2_ref(oracle, cfg2):
    return ref_batch(oracle, cfg2, cfg2.poses, grad=True)


@pytest.mark.parametrize("recenter", [False, True])
def test_every_pose_energy_and_gradient(oracle, scorer_factory, cfg2, cfg2_ref, recenter):
    s = scorer_factory(cfg2.pocket, cfg2.ligand)
    E, G, st = s.score_poses(cfg2.poses, grad=True, recenter=recenter)
    ref = cfg2_ref if not recenter else ref_batch(oracle, cfg2, cfg2.poses, grad=True,
                                                  recenter=True)
    assert_ref(E, G, ref, st)
    e, g = energy_errors(E, ref.E, ref.S), grad_errors(G, ref.G, ref.GA)
    print("4096 poses: max |E-E64|/|E64| %.2e (%d cancellation cases), gradient components "
          "%.2e of max(|G64|, %.2f GA) at most, %.4f%% of them within %.0e plain relative"
          % (e["max_rel"], e["n_cancel"], g["max_comp"], G_FLOOR, 100 * g["frac_plain_ok"], G_TOL))


def test_every_pose_one_per_call(oracle, scorer_factory, cfg2, cfg2_ref):
    """The plain path (B = 1, the drop-in) on 256 of the poses."""
    s = scorer_factory(cfg2.pocket, cfg2.ligand)
    n = 256
    E = np.zeros(n)
    G = np.zeros((n, cfg2.poses.shape[1]), np.float32)
    st = np.zeros(n, np.int32)
    for b in range(n):
        e, g, t = s.score_poses(cfg2.poses[b:b + 1], grad=True)
        E[b], G[b], st[b] = e[0], g[0], t[0]
    assert_energy(E, cfg2_ref.E[:n], cfg2_ref.S[:n])
    assert_grad(G, cfg2_ref.G[:n], cfg2_ref.GA[:n])
    assert np.array_equal(st, cfg2_ref.st[:n])


def test_gradient_against_central_differences(oracle, scorer_factory, cfg2, cfg2_ref):
    """The GPU gradient against FP64 central differences (h = 1e-4 A / rad,
    and h / 2), Richardson-extrapolated, on the components where the
    differences themselves are accurate: their truncation error (estimated by
    the change from h to h / 2) and their FP64 rounding (about 1e-16 S / h,
    which makes them meaningless where the energy is 1e20 and a step moves it
    by less than its last bit) are both under 1e-5 of the component."""
    n = 512
    s = scorer_factory(cfg2.pocket, cfg2.ligand)
    _, G, _ = s.score_poses(cfg2.poses[:n], grad=True)
    h = 1e-4
    _, F1, _ = oracle.score_batch(cfg2.pocket, cfg2.ligand, cfg2.poses[:n], mode=2, eps=h,
                                  nthreads=16)
    _, F2, _ = oracle.score_batch(cfg2.pocket, cfg2.ligand, cfg2.poses[:n], mode=2, eps=h / 2,
                                  nthreads=16)
    err, trusted = fd_check(G, F1, F2, cfg2_ref.S[:n], cfg2_ref.GA[:n], h)
    assert trusted.mean() >= 0.5, trusted.mean()
    assert err.max() <= G_TOL, err.max()
    # and the oracle's analytic gradient agrees with them as well
    err64, _ = fd_check(cfg2_ref.G[:n], F1, F2, cfg2_ref.S[:n], cfg2_ref.GA[:n], h)
    assert err64.max() <= 1e-6, err64.max()


def test_energy_only_large_sample(oracle, scorer_factory):
    """65,536 poses of energy only (inter + intra): 8,192 of them against the
    oracle under the energy contract."""
    big = synth.pose_batch(n_poses=65536, seed=1)
    s = scorer_factory(big.pocket, big.ligand)
    E, _, st = s.score_poses(big.poses)
    idx = np.random.default_rng(7).choice(len(E), 8192, replace=False)
    ref = ref_batch(oracle, big, big.poses[idx])
    r = assert_energy(E[idx], ref.E, ref.S, tol=E_TOL)
    assert np.array_equal(st[idx], ref.st)
    print("8192 of 65536 poses: max |E-E64|/|E64| %.2e" % r["max_rel"])
