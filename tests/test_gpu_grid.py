"""Precomputed interaction grids on the GPU (include/mmo_grid.h) against the oracle.

Grid values: Lds.pre_calculate_FF_components_grid (src/lds.ml:452-469) at
lattice points, the oracle's orc_grid_point in FP64; within 1e-5 of it,
relative to max(|E|, sum of |pair terms| at the point), the scoring contract's
energy tolerance; capped points equal max_E exactly; masked-out points 0.
Interpolated energies: Mol.ene_inter_UFF_interp (src/mol.ml:1010-1020) on the
same float32 grids, the oracle's orc_ene_inter_interp (FP64); within 1e-6
relative to the sum over the atoms of sum |corner value| x weight (the GPU
interpolates the float32 values in FP32 from a float-pair lattice coordinate).
Gradients: the derivative of the trilinear form chained through the pose,
within 1e-4 (relative to the largest component) of central differences of the
oracle's interpolated energy."""
import numpy as np
import pytest

from mmo_gb300 import grids as GR
from mmo_gb300 import synth

pytestmark = pytest.mark.gpu

E_TOL = 1e-5
I_TOL = 1e-6
G_TOL = 1e-4
STEP = 0.5


@pytest.fixture(scope="module")
def system():
    # 32-atom ligand, 1,500-atom pocket in a 14 A sphere; poses within 3 A of the centre
    s = synth.pose_batch(n_poses=64, seed=5, n_atoms=32, n_rot=5, n_pocket=1500, radius=14.0,
                         half_box=3.0)
    return s


@pytest.fixture(scope="module")
def lattice():
    origin, dims = GR.lattice_from_box(STEP, (-17.0, -17.0, -17.0), (17.0, 17.0, 17.0))
    return origin, dims


def _types(lig):
    types, per = GR.type2id([lig])
    return types, per[0]


def _built(scorer_factory, system, lattice, physics=None, **kw):
    s = scorer_factory(system.pocket, system.ligand, physics)
    types, lt = _types(system.ligand)
    origin, dims = lattice
    ms = s.build_grids(STEP, dims, origin, types, **kw)
    assert ms > 0
    return s, types, lt


def _point_scale(T, pocket, p, anum, q, diel=0, mixing=0):
    return T.ene_inter(pocket.xyz(), pocket.q, pocket.anum, np.asarray(p)[None, :],
                       np.array([q]), np.array([anum]), mixing=mixing, dielectric=diel,
                       absolute=True)


# (dielectric, mixing): the reference's eps = 4 with geometric means (the
# factorised build), eps = 4 r, Lorentz-Berthelot (the per-element build)
@pytest.mark.parametrize("diel,mixing", [(0, 0), (1, 0), (0, 1)])
def test_grid_values_match_oracle(oracle, scorer_factory, system, lattice, diel, mixing):
    from mmo_gb300.ff import Physics
    from oracle import np_twin as T

    ph = oracle.physics(diel, mixing, 0, 0)
    s, types, _ = _built(scorer_factory, system, lattice, Physics(diel, mixing, 0, 0))
    g = s.grid_values()
    origin, (nx, ny, nz) = lattice
    assert g.shape == (len(types), nz, ny, nx)
    rng = np.random.default_rng(7)
    ijk = np.stack([rng.integers(0, n, 48) for n in (nx, ny, nz)], axis=1)
    # points close to protein atoms (large values, the cap) and the lattice corners
    near = np.rint((system.pocket.xyz()[:16] - origin) / STEP).astype(int)
    corners = np.array([[i, j, k] for i in (0, nx - 1) for j in (0, ny - 1) for k in (0, nz - 1)])
    ta = np.array([t[0] for t in types])
    tq = np.array([t[1] for t in types])
    capped = 0
    for i, j, k in np.concatenate([ijk, near, corners]):
        p = origin + STEP * np.array([i, j, k], np.float64)
        ref = oracle.grid_point(system.pocket, p, ta, tq, ph=ph)
        got = g[:, k, j, i].astype(np.float64)
        for l in range(len(types)):
            if ref[l] >= GR.MAX_E:
                assert got[l] == GR.MAX_E
                capped += 1
                continue
            sc = _point_scale(T, system.pocket, p, ta[l], tq[l], diel, mixing)
            err = abs(got[l] - ref[l]) / max(abs(ref[l]), sc, 1e-300)
            assert err <= E_TOL, (i, j, k, l, got[l], ref[l], err)
    assert capped > 0  # the near-atom points reach the cap


def test_mask_sphere_zeroes_outside(oracle, scorer_factory, system, lattice):
    c = np.array([1.5, -2.0, 0.5])
    R = 9.0
    s, types, _ = _built(scorer_factory, system, lattice, mask_center=c, mask_radius=R)
    g = s.grid_values()
    origin, (nx, ny, nz) = lattice
    zz, yy, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    pts = np.stack([xx, yy, zz], axis=-1) * STEP + origin
    inside = ((pts - c) ** 2).sum(axis=-1) < R * R
    assert np.all(g[:, ~inside] == 0.0)
    # inside the mask the values equal the unmasked build's
    s2, _, _ = _built(scorer_factory, system, lattice)
    g2 = s2.grid_values()
    assert np.array_equal(g[:, inside], g2[:, inside])


def test_values_independent_of_launch_shape(scorer_factory, system, lattice):
    s, types, _ = _built(scorer_factory, system, lattice)
    origin, dims = lattice
    out = []
    for kp, prof in ((1, False), (2, False), (4, False), (2, True)):
        s.set_grid_build(kp)
        s.set_profiling(prof)  # the pair-counting variant of the kernel
        s.build_grids(STEP, dims, origin, types, mask_center=(0.5, 0.0, -1.0), mask_radius=15.0)
        out.append(s.grid_values())
    s.set_profiling(False)
    assert all(np.array_equal(out[0], o) for o in out[1:])
    st = s.grid_build_stats()
    assert st["pairs_evaluated"] >= st["pairs_within_cutoff"] > 0


def _corner_scale(grids, lt, uvw):
    """sum over the atoms of sum |corner value| x trilinear weight (uvw: lattice
    coordinates in steps)."""
    tot = 0.0
    for t, (u, v, w) in zip(lt, uvw):
        i, j, k = int(u), int(v), int(w)
        fx, fy, fz = u - i, v - j, w - k
        for c in range(8):
            di, dj, dk = c & 1, (c >> 1) & 1, c >> 2
            wt = (fx if di else 1 - fx) * (fy if dj else 1 - fy) * (fz if dk else 1 - fz)
            tot += abs(float(grids[t, k + dk, j + dj, i + di])) * wt
    return tot


def _interp_ref(oracle, system, grids, lattice, lt, conf, recenter=False):
    origin, dims = lattice
    xyz, _ = oracle.apply_config(system.ligand, np.asarray(conf, np.float64),
                                 oracle.F_RECENTER if recenter else 0)
    e, off = oracle.ene_inter_interp(STEP, dims, grids, xyz - origin, lt)
    return e, off, xyz


@pytest.mark.parametrize("recenter", [False, True])
def test_interpolated_energy_matches_oracle(oracle, scorer_factory, system, lattice, recenter):
    s, types, lt = _built(scorer_factory, system, lattice)
    assert np.array_equal(s.grid_atom_types(), lt)
    g = s.grid_values()
    d = system.poses[:32]
    E, _, st = s.score_poses(d, intra=False, grid=True, recenter=recenter)
    assert np.all(st & 4 == 0)
    origin, dims = lattice
    for b in range(len(d)):
        e, off, xyz = _interp_ref(oracle, system, g, lattice, lt, d[b], recenter)
        assert not off
        sc = _corner_scale(g, lt, (xyz - origin) / STEP)
        assert abs(E[b] - e) <= I_TOL * max(sc, 1e-300), (b, E[b], e)
    # with the intra term: the sum of both, as the pair path adds them
    Ei, _, _ = s.score_poses(d, inter=False, recenter=recenter)
    Et, _, _ = s.score_poses(d, grid=True, recenter=recenter)
    assert np.allclose(Et, E + Ei, rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("recenter", [False, True])
def test_one_pose_on_grids_is_one_launch(oracle, scorer_factory, system, lattice, recenter):
    """One pose per call with MMO_F_GRID runs the one-pose kernel (a lookup CTA
    beside the intra CTA): one launch, the energy against the oracle's
    interpolation plus intra term, the gradient as the batched grid path's, and
    the off-lattice bit."""
    s, types, lt = _built(scorer_factory, system, lattice)
    g = s.grid_values()
    d = system.poses[:8]
    Eb, Gb, stb = s.score_poses(d, grad=True, grid=True, recenter=recenter)
    Ei, _, _ = s.score_poses(d, inter=False, recenter=recenter)
    origin, dims = lattice
    for b in range(len(d)):
        E1, G1, st1 = s.score_poses(d[b:b + 1], grad=True, grid=True, recenter=recenter)
        assert s.last_launches() == 1
        assert st1[0] == stb[b]
        e, off, xyz = _interp_ref(oracle, system, g, lattice, lt, d[b], recenter)
        sc = _corner_scale(g, lt, (xyz - origin) / STEP)
        # (E1 - Ei: the inter part, up to the intra sums' FP32 rounding)
        assert abs((E1[0] - Ei[b]) - e) <= I_TOL * max(sc, 1e-300) + 1e-6 * abs(Ei[b])
        # the intra sums round differently (FP32 terms in another order)
        assert abs(E1[0] - Eb[b]) <= 1e-7 * max(abs(Eb[b]), sc, abs(Ei[b]))
        assert np.abs(G1[0] - Gb[b]).max() <= 1e-5 * np.abs(Gb[b]).max()
    far = d[:1].copy()
    far[0, 0] = 16.0  # the ligand's far side leaves the lattice
    _, _, stf = s.score_poses(far, grad=True, grid=True, recenter=recenter)
    assert stf[0] & 4


def test_interpolated_gradient_matches_differences(oracle, scorer_factory, system, lattice):
    s, types, lt = _built(scorer_factory, system, lattice)
    g = s.grid_values()
    d = system.poses[:8]
    E, G, st = s.score_poses(d, intra=False, grad=True, grid=True)
    E0, _, _ = s.score_poses(d, intra=False, grid=True)
    assert np.array_equal(E, E0)  # the energy does not depend on the gradient flag
    h = 1e-5
    for b in range(len(d)):
        conf = d[b].astype(np.float64)
        fd = np.zeros(len(conf))
        for k in range(len(conf)):
            cp, cm = conf.copy(), conf.copy()
            cp[k] += h
            cm[k] -= h
            fd[k] = (_interp_ref(oracle, system, g, lattice, lt, cp)[0] -
                     _interp_ref(oracle, system, g, lattice, lt, cm)[0]) / (2 * h)
        err = np.abs(G[b].astype(np.float64) - fd).max() / np.abs(fd).max()
        assert err <= G_TOL, (b, err)


def test_off_lattice_atoms_flagged_and_skipped(oracle, scorer_factory, system, lattice):
    s, types, lt = _built(scorer_factory, system, lattice)
    g = s.grid_values()
    d = system.poses[:4].copy()
    d[:, 0] = 16.0  # the ligand's far side leaves the lattice (points up to x = 17 A)
    E, _, st = s.score_poses(d, intra=False, grid=True)
    for b in range(len(d)):
        e, off, _ = _interp_ref(oracle, system, g, lattice, lt, d[b])
        assert off and (st[b] & 4)
        assert abs(E[b] - e) <= I_TOL * max(abs(e), 100.0)
        # the closure (one launch) flags it the same way
        xyz, _ = oracle.apply_config(system.ligand, d[b].astype(np.float64), 0)
        e1, st1 = s.ene_inter_grid(system.ligand.with_xyz(xyz))
        assert st1 & 4
        assert abs(e1 - e) <= I_TOL * max(abs(e), 100.0)


def test_loaded_grids_score_like_built(scorer_factory, system, lattice, tmp_path):
    s, types, lt = _built(scorer_factory, system, lattice)
    g = s.grid_values()
    origin, dims = lattice
    files = GR.write_ba1(str(tmp_path / "lig"), STEP, dims, g)
    assert len(files) == len(types)
    step, dims2, g2 = GR.read_ba1(str(tmp_path / "lig"), len(types))
    assert step == STEP and tuple(dims2) == tuple(dims) and np.array_equal(g, g2)
    s2 = scorer_factory(system.pocket, system.ligand)
    s2.load_grids(STEP, dims, origin, types, g2)
    d = system.poses[:16]
    a = s.score_poses(d, grad=True, grid=True)
    b = s2.score_poses(d, grad=True, grid=True)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    # no protein is needed to score from grids; the device frame is then the
    # protein's frame (origin 0), so the values agree to rounding
    s3 = scorer_factory(None, system.ligand)
    s3.load_grids(STEP, dims, origin, types, g2)
    e2, _, _ = s2.score_poses(d, intra=False, grid=True)
    e3, _, st3 = s3.score_poses(d, intra=False, grid=True)
    assert np.all(st3 == 0)
    assert np.allclose(e3, e2, rtol=1e-6, atol=1e-6)


def test_ligand_type_missing_from_grids(gpu_lib, scorer_factory, system, lattice):
    from mmo_gb300 import lib as L

    s = scorer_factory(system.pocket, system.ligand)
    types, _ = _types(system.ligand)
    origin, dims = lattice
    s.build_grids(STEP, dims, origin, types[:-1])  # the last type is left out
    with pytest.raises(L.MMOError) as ei:
        s.score_poses(system.poses[:2], grid=True)
    assert ei.value.code == L.ESTATE
    with pytest.raises(L.MMOError):
        s.grid_atom_types()
    s.score_poses(system.poses[:2])  # the pair path is unaffected


def test_mc_chains_on_grids(scorer_factory, system, lattice):
    torch = pytest.importorskip("torch")
    from mmo_gb300 import lib as L

    s, types, lt = _built(scorer_factory, system, lattice)
    dev = torch.device("cuda", 0)
    B = 32
    d0 = system.poses[:B]
    d = torch.from_numpy(np.ascontiguousarray(d0)).to(dev)
    E = torch.empty(B, dtype=torch.float64, device=dev)
    bd, bE = torch.empty_like(d), torch.empty_like(E)
    acc = torch.empty(B, dtype=torch.int32, device=dev)
    st = torch.empty(B, dtype=torch.int32, device=dev)
    prm = dict(kT=0.593, rot_step=np.radians(5.0), trans_step=0.3, tors_step=np.radians(30.0),
               move_law=L.MC_GAUSSIAN, adapt=0, flip_every=0, minimize_every=30,
               minimize_iters=4, gd_step=0.1, seed=77, use_grid=1)
    s.mc_run_device(B, 60, prm, d.data_ptr(), E.data_ptr(), bd.data_ptr(), bE.data_ptr(),
                    acc.data_ptr(), st.data_ptr(), None, True)
    torch.cuda.synchronize()
    dn, En, an = d.cpu().numpy(), E.cpu().numpy(), acc.cpu().numpy()
    assert np.all(an > 0)
    Er, _, _ = s.score_poses(dn, recenter=True, grid=True)
    assert np.array_equal(Er, En)
    # the grid energies differ from the pair sums (an interpolation), not wildly
    Ep, _, _ = s.score_poses(dn, recenter=True)
    assert np.all(np.isfinite(Ep))


def test_plain_interp_closure_matches_oracle(oracle, gpu_lib, system, lattice):
    """ene_inter_interp_builder: the closure of src/lds.ml:1975 on posed ligands."""
    from mmo_gb300.ff import ene_inter_interp_builder

    origin, dims = lattice
    f = ene_inter_interp_builder(system.pocket, [system.ligand], step=STEP, margin=3.0)
    s = f.scorer
    g = s.grid_values()
    nt, nx, ny, nz = g.shape
    _, lt = _types(system.ligand)
    p = system.pocket.xyz()
    o2, d2 = GR.lattice_from_box(STEP, p.min(axis=0) - 3.0, p.max(axis=0) + 3.0)
    for conf in system.poses[:6]:
        xyz, _ = oracle.apply_config(system.ligand, conf.astype(np.float64), 0)
        e = f(system.ligand.with_xyz(xyz))
        assert s.last_launches() == 1  # lookup and sum in one block
        e64, off = oracle.ene_inter_interp(STEP, d2, g, xyz - o2, lt)
        assert not off
        assert abs(e - e64) <= I_TOL * _corner_scale(g, lt, (xyz - o2) / STEP)
    f.scorer.close()
