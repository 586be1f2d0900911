"""Ragged batches of systems (mmo_set_systems / mmo_score_systems*) on the GPU.

Systems of uneven size (ligands of 12-80 atoms with 0-15 torsions, pockets of
2,000-9,000 atoms, 0-40 poses each) in one pass: every pose's energy and
gradient against the same pose scored through the one-system entry points,
the FP64 oracle on a sample, the global form, a CUDA-graph replay and the
host-buffer entry point."""
import numpy as np
import pytest

from mmo_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def systems():
    ss = synth.ragged_systems(n_systems=9, poses_per=24, seed=11)
    rng = np.random.default_rng(2)
    out = []
    for k, s in enumerate(ss):
        n = [24, 0, 40, 7, 24, 1, 33, 24, 16][k]
        poses = synth.random_poses(rng, n, s.ligand.nrb, 4.0) if n else s.poses[:0]
        out.append(synth.System(s.name, s.pocket, s.ligand, poses))
    # one pocket too large for the one-system cut-off sweep's shared memory
    big = synth.pose_batch(n_poses=20, seed=4, n_atoms=40, n_rot=6, n_pocket=9000, radius=20.5)
    out.append(big)
    return out


def _packed(systems):
    return np.concatenate([s.poses.reshape(-1) for s in systems]).astype(np.float32)


def _split(v, off):
    return [v[off[k]:off[k + 1]] for k in range(len(off) - 1)]


@pytest.mark.parametrize("recenter", [False, True])
def test_systems_match_one_system_path(scorer_factory, systems, recenter):
    sc = scorer_factory()
    sc.set_systems([(s.pocket, s.ligand, len(s.poses)) for s in systems])
    po, do = sc.systems_layout()
    E, G, st = sc.score_systems(_packed(systems), grad=True, recenter=recenter)
    Es, Gs, sts = _split(E, po), _split(G, do), _split(st, po)
    for k, s in enumerate(systems):
        if not len(s.poses):
            continue
        one = scorer_factory(s.pocket, s.ligand)
        E1, G1, st1 = one.score_poses(s.poses, grad=True, recenter=recenter)
        assert np.array_equal(sts[k], st1)
        if s.pocket.n <= 6000 and not recenter and len(s.poses) >= 2:
            # same row index, pieces and arithmetic as the one-system cut-off sweep
            # (a single pose takes the one-pose kernel there)
            assert np.array_equal(Es[k], E1), k
            g = Gs[k].reshape(G1.shape)
            bad = ~((g == G1) | (np.isnan(g) & np.isnan(G1)))
            assert not bad.any(), (k, np.argwhere(bad)[:5], g[bad][:5], G1[bad][:5])
        else:
            assert np.abs(Es[k] - E1).max() <= 1e-6 * np.abs(E1).max(), k
            g = Gs[k].reshape(G1.shape)
            assert (np.abs(g - G1).max(axis=1) / np.abs(G1).max(axis=1)).max() <= 1e-5, k


def test_systems_against_oracle(oracle, scorer_factory, systems):
    from contract import assert_ref, ref_batch

    sc = scorer_factory()
    sc.set_systems([(s.pocket, s.ligand, len(s.poses)) for s in systems])
    po, do = sc.systems_layout()
    E, G, _ = sc.score_systems(_packed(systems), grad=True)
    Es, Gs = _split(E, po), _split(G, do)
    for k in (0, 3, 5, 9):
        s = systems[k]
        assert_ref(Es[k], Gs[k].reshape(len(s.poses), -1), ref_batch(oracle, s, s.poses,
                                                                     grad=True))


def test_systems_global_form(oracle, scorer_factory, systems):
    """The global form has no cut-off: every protein atom counts, also the
    ones beyond 12 A of a pose (every pose against the FP64 oracle under the
    scoring contract)."""
    from mmo_gb300.ff import Physics
    from contract import assert_ref, ref_batch

    sub = [systems[0], systems[3], systems[6]]
    sc = scorer_factory(physics=Physics(1, 0, 1, 0))
    sc.set_systems([(s.pocket, s.ligand, len(s.poses)) for s in sub])
    po, do = sc.systems_layout()
    E, G, _ = sc.score_systems(_packed(sub), grad=True)
    for k, s in enumerate(sub):
        one = scorer_factory(s.pocket, s.ligand, Physics(1, 0, 1, 0))
        E1, G1, _ = one.score_poses(s.poses, grad=True)
        e = E[po[k]:po[k + 1]]
        g = G[do[k]:do[k + 1]].reshape(G1.shape)
        assert np.abs(e - E1).max() <= 1e-6 * np.abs(E1).max()
        assert (np.abs(g - G1).max(axis=1) / np.abs(G1).max(axis=1)).max() <= 1e-5
        assert_ref(e, g, ref_batch(oracle, s, s.poses, grad=True, ph=oracle.physics(1, 0, 1, 0)))


def test_systems_graph_replay_and_device_entry(scorer_factory, systems):
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L

    sc = scorer_factory()
    sc.set_systems([(s.pocket, s.ligand, len(s.poses)) for s in systems])
    po, do = sc.systems_layout()
    h = _packed(systems)
    E0, G0, st0 = sc.score_systems(h, grad=True)
    dev = torch.device("cuda", 0)
    d = torch.from_numpy(h).to(dev)
    E = torch.empty(int(po[-1]), dtype=torch.float64, device=dev)
    G = torch.empty_like(d)
    st = torch.empty(int(po[-1]), dtype=torch.int32, device=dev)
    flags = L.F_INTER | L.F_INTRA | L.F_GRAD
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        sc.score_systems_device(d.data_ptr(), E.data_ptr(), G.data_ptr(), st.data_ptr(), flags,
                                s.cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(E.cpu().numpy(), E0) and np.array_equal(G.cpu().numpy(), G0)
    g = torch.cuda.CUDAGraph()
    E.zero_()
    G.zero_()
    with torch.cuda.graph(g, stream=s):
        sc.score_systems_device(d.data_ptr(), E.data_ptr(), G.data_ptr(), st.data_ptr(), flags,
                                s.cuda_stream)
    for _ in range(2):
        E.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(E.cpu().numpy(), E0) and np.array_equal(G.cpu().numpy(), G0)
        assert np.array_equal(st.cpu().numpy(), st0)


def test_systems_page_locked_buffers_give_the_same_results(scorer_factory, systems):
    torch = pytest.importorskip("torch")
    sc = scorer_factory()
    sc.set_systems([(s.pocket, s.ligand, len(s.poses)) for s in systems])
    po, do = sc.systems_layout()
    h = _packed(systems)
    E0, G0, st0 = sc.score_systems(h, grad=True)
    B = int(po[-1])
    out = (torch.zeros(B, dtype=torch.float64).pin_memory().numpy(),
           torch.zeros(h.size, dtype=torch.float32).pin_memory().numpy(),
           torch.zeros(B, dtype=torch.int32).pin_memory().numpy())
    E, G, st = sc.score_systems(torch.from_numpy(h).pin_memory().numpy(), grad=True, out=out)
    assert E is out[0] and G is out[1] and st is out[2]
    assert np.array_equal(E, E0) and np.array_equal(st, st0)
    assert not (~((G == G0) | (np.isnan(G) & np.isnan(G0)))).any()
