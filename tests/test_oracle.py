"""The FP64 oracle against known answers, the reference's own test vectors and
an independent NumPy restatement (CPU only)."""
import math

import numpy as np
import pytest

from mmo_gb300 import synth
from mmo_gb300.topology import Mol, build_ligand

K = 332.0637 / 4.0


def two_atoms(a1, q1, a2, q2, r):
    prot = Mol("p", np.array([0.0]), np.array([0.0]), np.array([0.0]), np.array([q1]),
               np.array([a1], np.int32))
    lig = Mol("l", np.array([r]), np.array([0.0]), np.array([0.0]), np.array([q2]),
              np.array([a2], np.int32))
    return prot, lig


def chain(n, bond=1.5):
    """zig-zag chain of n carbons with all internal bonds rotatable"""
    xyz = []
    for i in range(n):
        xyz.append([i * bond * math.sin(math.radians(54.75)), 0.8 * (i % 2), 0.0])
    bonds = [(i, i + 1) for i in range(n - 1)]
    return build_ligand("chain%d" % n, np.array(xyz), np.zeros(n), np.full(n, 6, np.int32), bonds)


# -- known answers from the formulas -------------------------------------------

def test_elec_weight(oracle):
    assert oracle.elec_weight() == pytest.approx(83.015925, abs=1e-12)


def test_shift_values(oracle):
    # FF.ml:17-20
    assert oracle.shift_12A(0.0) == 1.0
    assert oracle.shift_12A(6.0) == pytest.approx(0.5625, abs=1e-15)
    assert oracle.shift_12A(12.0) == 0.0
    assert oracle.shift_12A(13.0) == 0.0
    assert oracle.non_zero_dist(0.001) == 0.01
    assert oracle.non_zero_dist(0.5) == 0.5


def test_pair_table(oracle):
    # UFF.ml:43-51: geometric means; unsupported elements give NaN
    x, d = oracle.pair_params(6, 8)
    assert x == pytest.approx(math.sqrt(3.851 * 3.500), rel=1e-15)
    assert d == pytest.approx(math.sqrt(0.105 * 0.060), rel=1e-15)
    x, d = oracle.pair_params(6, 8, oracle.physics(mixing=1))
    assert x == pytest.approx(0.5 * (3.851 + 3.500), rel=1e-15)
    x, d = oracle.pair_params(6, 2)
    assert math.isnan(x) and math.isnan(d)


@pytest.mark.parametrize("anum,xi,di", [(1, 2.886, 0.044), (6, 3.851, 0.105), (7, 3.660, 0.069),
                                        (8, 3.500, 0.060), (16, 4.035, 0.274), (53, 4.5, 0.339)])
def test_lj_minimum(oracle, anum, xi, di):
    # at r = x_ij the LJ 12-6 term is -D_ij; global form has no switch
    prot, lig = two_atoms(anum, 0.0, anum, 0.0, xi)
    g = oracle.physics(inter_form=1)
    assert oracle.ene_inter(prot, lig, ph=g) == pytest.approx(-di, rel=1e-12)
    w = (1.0 - (xi / 12.0) ** 2) ** 2
    assert oracle.ene_inter(prot, lig) == pytest.approx(-di * w, rel=1e-12)


def test_coulomb_pair(oracle):
    # virtual element 0 has no vdW: only K q1 q2 / r (times the switch)
    prot, lig = two_atoms(0, 0.5, 0, -0.3, 5.0)
    w = (1.0 - (5.0 / 12.0) ** 2) ** 2
    assert oracle.ene_inter(prot, lig) == pytest.approx(K * -0.15 / 5.0 * w, rel=1e-13)
    assert oracle.ene_inter(prot, lig, ph=oracle.physics(inter_form=1)) == pytest.approx(
        K * -0.15 / 5.0, rel=1e-13)
    assert oracle.ene_inter(prot, lig, ph=oracle.physics(dielectric=1, inter_form=1)) == \
        pytest.approx(K * -0.15 / 25.0, rel=1e-13)


def test_cutoff_and_clamp(oracle):
    prot, lig = two_atoms(6, 0.5, 6, 0.5, 12.0)
    assert oracle.ene_inter(prot, lig) == 0.0
    prot, lig = two_atoms(0, 1.0, 0, 1.0, 0.001)  # clamped to 0.01 A
    assert oracle.ene_inter(prot, lig, ph=oracle.physics(inter_form=1)) == pytest.approx(
        K / 0.01, rel=1e-13)


def test_intra_exclusions(oracle):
    # 1-2 and 1-3 pairs are excluded; 1-4 counts fully (mol.ml:203-208, 891-894)
    lig3 = chain(3)
    assert lig3.interacting.sum() == 0
    assert oracle.ene_intra(lig3) == 0.0
    lig4 = chain(4)
    assert lig4.interacting[0, 3] == 1 and lig4.interacting.sum() == 2
    r = np.linalg.norm(lig4.xyz()[0] - lig4.xyz()[3])
    p6 = (3.851 / r) ** 6
    assert oracle.ene_intra(lig4) == pytest.approx(0.105 * (p6 * p6 - 2 * p6), rel=1e-12)


# -- the reference's own numeric test vectors (src/tests.ml:10-54) --------------

def test_dihedral_vectors_from_reference(oracle):
    c = math.cos(0.25 * math.pi)
    i, j, k = [0., 0., 0.], [0., 1., 0.], [1., 1., 0.]
    ls = [[1, 2, 0], [1, 1 + c, c], [1, 1, 1], [1, 1 - c, c], [1, 0, 0], [1, 1 - c, -c],
          [1, 1, -1], [1, 1 + c, -c]]
    want = [1.0, -0.75, -0.5, -0.25, 0.0, 0.25, 0.5, 0.75]
    for l, w in zip(ls, want):
        assert abs(oracle.dihedral(i, j, k, l) - w * math.pi) <= 0.001


def test_rotate_bond_turns_dihedral(oracle, rng):
    # rotate_bond (mol.ml:610-631) about (j, k) by theta moves dihedral i-j-k-l by +theta,
    # pinned through the dihedral function of the reference's test above
    xyz = np.array([[0, 0, 0], [0, 1, 0], [1, 1, 0], [1, 2, 0.]])
    d0 = oracle.dihedral(*xyz)
    for th in rng.uniform(-math.pi, math.pi, 8):
        x2 = oracle.rotate_bond(xyz, 1, 2, [3], th)
        d1 = oracle.dihedral(*x2)
        assert abs((d1 - d0 - th + math.pi) % (2 * math.pi) - math.pi) < 1e-12
        back = oracle.rotate_bond(x2, 1, 2, [3], -th)
        assert np.abs(back - xyz).max() < 1e-14


# -- C oracle vs the independent NumPy twin --------------------------------------

@pytest.mark.parametrize("ph", [dict(), dict(inter_form=1), dict(dielectric=1), dict(mixing=1)])
def test_c_vs_numpy_inter(oracle, ph):
    from oracle import np_twin as T

    s = synth.single_pose(seed=7)
    conf = s.poses[0].astype(np.float64)
    xyz, st = oracle.apply_config(s.ligand, conf)
    p, l = s.pocket, s.ligand
    e_c = oracle.ene_inter(p, l, xyz, ph=oracle.physics(**ph))
    e_n = T.ene_inter(p.xyz(), p.q, p.anum, xyz, l.q, l.anum, shifted=ph.get("inter_form", 0) == 0,
                      mixing=ph.get("mixing", 0), dielectric=ph.get("dielectric", 0))
    assert e_c == pytest.approx(e_n, rel=1e-12)
    if ph.get("inter_form", 0) == 0:
        assert oracle.ene_inter_cells(p, l, xyz, ph=oracle.physics(**ph)) == pytest.approx(
            e_c, rel=1e-12)


@pytest.mark.parametrize("ph", [dict(), dict(inter_form=1), dict(dielectric=1)])
def test_c_vs_numpy_inter_parts(oracle, ph):
    """orc_ene_inter_parts (the electrostatic and van der Waals parts of
    Mol.ene_inter_UFF_shifted_bst_components, mol.ml:920-957) against the same
    parts summed in NumPy; their sum is the oracle's ene_inter."""
    from oracle import np_twin as T

    s = synth.single_pose(seed=7)
    xyz, _ = oracle.apply_config(s.ligand, s.poses[0].astype(np.float64))
    p, l = s.pocket, s.ligand
    el, lj = oracle.ene_inter_parts(p, l, xyz, ph=oracle.physics(**ph))
    xp, dp = T.params(p.anum)
    xl, dl = T.params(l.anum)
    d = np.linalg.norm(p.xyz()[:, None, :] - xyz[None, :, :], axis=2)
    r = np.maximum(d, 0.01)
    if ph.get("inter_form", 0) == 0:
        w = np.where(d * d < 144.0, (1.0 - (r / 12.0) ** 2) ** 2, 0.0)
    else:
        w = np.ones_like(r)
    qq = p.q[:, None] * l.q[None, :]
    el_n = (w * T.ELEC * (qq / r if ph.get("dielectric", 0) == 0 else qq / (r * r))).sum()
    p6 = (np.sqrt(xp[:, None] * xl[None, :]) / r) ** 6
    lj_n = (w * np.sqrt(dp[:, None] * dl[None, :]) * (p6 * p6 - 2.0 * p6)).sum()
    assert el == pytest.approx(el_n, rel=1e-12, abs=1e-12)
    assert lj == pytest.approx(lj_n, rel=1e-12, abs=1e-12)
    assert el + lj == pytest.approx(oracle.ene_inter(p, l, xyz, ph=oracle.physics(**ph)),
                                    rel=1e-12)


def test_c_vs_numpy_intra_and_pose(oracle, rng):
    from oracle import np_twin as T

    for seed in range(4):
        r = np.random.default_rng(seed)
        lig = synth.random_ligand(r, int(r.integers(8, 60)), int(r.integers(0, 12)))
        conf = np.concatenate([r.uniform(-3, 3, 3), r.uniform(-np.pi, np.pi, 3 + lig.nrb)])
        for flags in (0, oracle.F_RECENTER):
            x_c, _ = oracle.apply_config(lig, conf, flags)
            x_n = T.apply_config(lig.xyz(), lig.rbonds, lig.rgroups, conf, recenter=bool(flags))
            assert np.abs(x_c - x_n).max() < 1e-12
        assert oracle.ene_intra(lig, x_c) == pytest.approx(
            T.ene_intra(x_c, lig.q, lig.anum, lig.interacting), rel=1e-12, abs=1e-12)


# -- analytic FP64 gradient vs central differences (h = 1e-4) --------------------

@pytest.mark.parametrize("flags", [3, 3 | 8, 1, 2])
def test_gradient_vs_fd(oracle, flags):
    # dense pocket: clash energies up to 1e16, so a small step (1e-6) keeps the
    # central-difference truncation error below the check
    s = synth.pose_batch(n_poses=4, seed=5, n_atoms=20, n_rot=4, n_pocket=400, radius=10.0,
                         half_box=6.0)
    for conf in s.poses.astype(np.float64):
        E, g, st = oracle.grad_analytic(s.pocket, s.ligand, conf, flags)
        Es, _ = oracle.score_conf(s.pocket, s.ligand, conf, flags)
        assert E == pytest.approx(Es, rel=1e-12)
        gf = oracle.grad_fd(s.pocket, s.ligand, conf, 1e-6, flags)
        scale = np.abs(g).max()
        assert np.abs(g - gf).max() <= 1e-6 * scale + 1e-9


def test_gradient_vs_fd_h1e4(oracle):
    # sparse pocket (moderate energies): central differences with h = 1e-4 A/rad
    s = synth.pose_batch(n_poses=4, seed=8, n_atoms=24, n_rot=5, n_pocket=150, radius=14.0,
                         half_box=3.0)
    for conf in s.poses.astype(np.float64):
        E, g, _ = oracle.grad_analytic(s.pocket, s.ligand, conf)
        gf = oracle.grad_fd(s.pocket, s.ligand, conf, 1e-4)
        assert np.abs(g - gf).max() <= 1e-4 * np.abs(g).max()


@pytest.mark.parametrize("flags", [3, 1, 2, 11])
def test_condition_scales(oracle, flags):
    """orc_grad_scale: S is the sum over pairs of w (|elec| + D p12 + 2 D p6)
    (the NumPy twin's absolute sum), S >= |E|, each GA_k bounds |G_k|, and the batch mode
    returns the same numbers."""
    from oracle import np_twin as T

    s = synth.pose_batch(n_poses=6, seed=12, n_atoms=20, n_rot=4, n_pocket=400, radius=10.0)
    S, GA, _ = oracle.score_batch(s.pocket, s.ligand, s.poses, flags=flags, mode=3, nthreads=2)
    _, G, _ = oracle.score_batch(s.pocket, s.ligand, s.poses, flags=flags, mode=1, nthreads=2)
    for b, conf in enumerate(s.poses.astype(np.float64)):
        Sb, gb = oracle.grad_scale(s.pocket, s.ligand, conf, flags=flags)
        assert Sb == S[b] and np.array_equal(gb, GA[b])
        xyz, _ = oracle.apply_config(s.ligand, conf, flags & oracle.F_RECENTER)
        want = 0.0
        if flags & oracle.F_INTER:
            p = s.pocket
            want += T.ene_inter(p.xyz(), p.q, p.anum, xyz, s.ligand.q, s.ligand.anum,
                                absolute=True)
        if flags & oracle.F_INTRA:
            want += T.ene_intra(xyz, s.ligand.q, s.ligand.anum, s.ligand.interacting,
                                absolute=True)
        assert Sb == pytest.approx(want, rel=1e-10)
    E, _, _ = oracle.score_batch(s.pocket, s.ligand, s.poses, flags=flags, mode=0)
    assert np.all(S >= np.abs(E) * (1 - 1e-12))
    assert np.all(GA >= np.abs(G) * (1 - 1e-12))
    if flags == oracle.F_INTRA:  # intra energy is rigid-invariant: G_0..2 = 0, their scale not
        assert np.all(np.abs(G[:, :3]) <= 1e-9 * GA[:, :3])


def test_gradient_physics_variants(oracle):
    s = synth.pose_batch(n_poses=2, seed=9, n_atoms=16, n_rot=3, n_pocket=300, radius=9.0)
    for ph in (oracle.physics(1, 1, 1, 1), oracle.physics(0, 0, 1, 0), oracle.physics(1, 0, 0, 1)):
        for conf in s.poses.astype(np.float64):
            E, g, _ = oracle.grad_analytic(s.pocket, s.ligand, conf, ph=ph)
            gf = oracle.grad_fd(s.pocket, s.ligand, conf, 1e-4, ph=ph)
            assert np.abs(g - gf).max() <= 1e-5 * np.abs(g).max() + 1e-9


# -- invariances and statuses ---------------------------------------------------

def test_invariances(oracle, rng):
    s = synth.single_pose(seed=3)
    xyz, _ = oracle.apply_config(s.ligand, s.poses[0].astype(np.float64))
    e0 = oracle.ene_inter(s.pocket, s.ligand, xyz)
    perm = rng.permutation(s.pocket.n)
    p = s.pocket
    pp = Mol("pp", p.x[perm], p.y[perm], p.z[perm], p.q[perm], p.anum[perm])
    assert oracle.ene_inter(pp, s.ligand, xyz) == pytest.approx(e0, rel=1e-12)
    t = np.array([3.0, -7.0, 11.0])
    pt = Mol("pt", p.x + t[0], p.y + t[1], p.z + t[2], p.q, p.anum)
    assert oracle.ene_inter(pt, s.ligand, xyz + t) == pytest.approx(e0, rel=1e-11)


def test_too_long_status(oracle):
    lig = chain(22)  # about 29 A end to end
    lig = lig.centered()
    _, st = oracle.apply_config(lig, np.zeros(6 + lig.nrb))
    assert st == oracle.S_TOO_LONG
    short = chain(6).centered()
    _, st = oracle.apply_config(short, np.zeros(6 + short.nrb))
    assert st == 0


def test_batch_matches_single(oracle):
    s = synth.pose_batch(n_poses=6, seed=2, n_atoms=12, n_rot=3, n_pocket=200, radius=8.0)
    E, G, st = oracle.score_batch(s.pocket, s.ligand, s.poses, mode=1, nthreads=3)
    Ec, _, _ = oracle.score_batch(s.pocket, s.ligand, s.poses, mode=0, use_cells=True)
    for b, conf in enumerate(s.poses.astype(np.float64)):
        e, g, _ = oracle.grad_analytic(s.pocket, s.ligand, conf)
        assert E[b] == e and np.array_equal(G[b], g)
        assert Ec[b] == pytest.approx(e, rel=1e-12)


def test_philox_known_answers(oracle):
    """Philox4x32-10 against the known-answer vectors published with the
    algorithm (Random123 kat_vectors: zero, all-ones and the pi digits)."""
    import ctypes as C

    f = oracle.lib().orc_philox4x32_10

    def ph(ctr, key):
        c, k, o = (C.c_uint32 * 4)(*ctr), (C.c_uint32 * 2)(*key), (C.c_uint32 * 4)()
        f(c, k, o)
        return list(o)

    assert ph([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert ph([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6,
                                                      0x6D5451FD]
    assert ph([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_grid_point_is_single_atom_inter_energy(oracle):
    """A grid value is the shifted inter energy of a one-atom ligand of that
    type at the point (Mol.ene_inter_UFF_shifted_grid == _shifted_brute on a
    one-atom ligand), capped at max_E."""
    from mmo_gb300 import synth

    rng = np.random.default_rng(0)
    prot = synth.random_pocket(rng, 300, 9.0)
    types_a, types_q = [6, 7, 8, 16, 1], [0.1, -0.3, -0.5, 0.0, 0.2]
    for _ in range(5):
        p = rng.uniform(-6, 6, 3)
        g = oracle.grid_point(prot, p, types_a, types_q, max_E=1e30)
        for l, (a, q) in enumerate(zip(types_a, types_q)):
            one = Mol("one", np.array([p[0]]), np.array([p[1]]), np.array([p[2]]),
                      np.array([q]), np.array([a], np.int32), None, np.zeros((1, 1), np.int32))
            e = oracle.ene_inter(prot, one)
            assert abs(g[l] - e) <= 1e-12 * max(1.0, abs(e))
    capped = oracle.grid_point(prot, prot.xyz()[0] + 0.05, [6], [0.0], max_E=100000.0)
    assert capped[0] == 100000.0


def test_trilin_reproduces_linear_functions(oracle):
    step, dims = 0.5, (7, 6, 5)
    k, j, i = np.meshgrid(np.arange(dims[2]), np.arange(dims[1]), np.arange(dims[0]),
                          indexing="ij")
    v = (1.5 + 0.25 * i * step - 0.5 * j * step + 2.0 * k * step).astype(np.float32)
    rng = np.random.default_rng(1)
    for _ in range(20):
        p = rng.uniform(0, [(d - 1.01) * step for d in dims])
        e, off = oracle.trilin(step, dims, v, p)
        assert not off
        assert abs(e - (1.5 + 0.25 * p[0] - 0.5 * p[1] + 2.0 * p[2])) < 1e-5
    assert oracle.trilin(step, dims, v, [-0.1, 0.0, 0.0])[1]
    assert oracle.trilin(step, dims, v, [0.0, 0.0, (dims[2] - 1) * step])[1]


def test_grid_points_cells_equal_brute_grid_point(oracle):
    """The threaded cell-list sum (the CPU baseline of the grid build) against
    the brute per-point sum, at points inside, at the edge of and outside the
    protein's box."""
    from mmo_gb300 import synth

    rng = np.random.default_rng(4)
    prot = synth.random_pocket(rng, 800, 12.0)
    ta = np.array([6, 8, 7, 1], np.int32)
    tq = np.array([0.1, -0.4, 0.0, 0.25])
    pts = rng.uniform(-25.0, 25.0, size=(40, 3))
    pts[:5] = prot.xyz()[:5] + 0.05  # near atoms: capped values
    got = oracle.grid_points(prot, pts, ta, tq, nthreads=3)
    for k, p in enumerate(pts):
        ref = oracle.grid_point(prot, p, ta, tq)
        assert np.allclose(got[k], ref, rtol=1e-12, atol=1e-10)
    assert np.any(got == 100000.0) and np.any(got == 0.0)


# ---- masks, clash tests, SO(3) samples, docking, desolvation ----------------

def _small_lattice(oracle, lo=-6.0, n=25, step=0.5):
    return oracle.lattice(step, (n, n, n), (lo, lo, lo))


def test_masks_are_the_sphere_predicates(oracle):
    """Lds.vdW_volume / first_solvent_shell: the cube walk of atom_bitmask_set
    equals the plain predicates over every lattice point."""
    rng = np.random.default_rng(1)
    g = _small_lattice(oracle)
    xyz = rng.uniform(-4.0, 4.0, size=(12, 3))
    r = rng.choice([1.2, 1.55, 1.7, 1.8], size=12)
    vdw, shell = oracle.masks(g, xyz, r, 1.4)
    ax = -6.0 + 0.5 * np.arange(25)
    zz, yy, xx = np.meshgrid(ax, ax, ax, indexing="ij")
    pts = np.stack([xx, yy, zz], axis=-1)
    d2 = ((pts[..., None, :] - xyz) ** 2).sum(axis=-1)
    inside = (d2 < r * r).any(axis=-1)
    outer = (d2 < (r + 1.4) ** 2).any(axis=-1)
    assert np.array_equal(vdw.astype(bool), inside)
    assert np.array_equal(shell.astype(bool), outer & ~inside)


def test_clash_params_and_corner_tests(oracle):
    # Ptable.vdW_clash_params2: (0.8 (r_i + r_j))^2
    assert oracle.clash2(6, 8) == pytest.approx((0.8 * (1.7 + 1.55)) ** 2, rel=1e-15)
    assert oracle.clash2(1, 1) == pytest.approx((0.8 * 2.4) ** 2, rel=1e-15)
    g = _small_lattice(oracle)
    m = np.zeros((25, 25, 25), np.uint8)
    m[10, 10, 10] = 1  # one set point at (-1, -1, -1)
    assert oracle.protein_ligand_clash(g, m, [[-1.2, -1.2, -1.2]])   # cell (9, 9, 9) touches it
    assert not oracle.protein_ligand_clash(g, m, [[-1.7, -1.7, -1.7]])
    assert not oracle.clash_and(g, m, [-1.2, -1.2, -1.2])
    m[10:12, 10:12, 10:12] = 1
    assert oracle.clash_and(g, m, [-0.8, -0.8, -0.8])


def test_super_fibonacci_rotations_match_the_paper_formula(oracle):
    """SO3.super_fibonacci (Alexa 2022, Algorithm 1) restated in NumPy,
    through the quaternion's rotation matrix; proper rotations."""
    n = 50
    psi = 1.533751168755204288118041
    for i in (0, 1, 7, 49):
        s = i + 0.5
        t = s / n
        d = 2.0 * np.pi * s
        w, x = np.sqrt(t) * np.sin(d / np.sqrt(2.0)), np.sqrt(t) * np.cos(d / np.sqrt(2.0))
        y, z = np.sqrt(1 - t) * np.sin(d / psi), np.sqrt(1 - t) * np.cos(d / psi)
        Rq = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                       [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                       [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
        R = oracle.so3_rotation(n, i)
        assert np.allclose(R, Rq, atol=1e-12)
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-12) and np.linalg.det(R) > 0


def test_heavy_and_intra_clash(oracle):
    from mmo_gb300 import synth
    from mmo_gb300.topology import Mol

    rad = {1: 1.2, 6: 1.7, 7: 1.6, 8: 1.55, 16: 1.8}
    for seed in range(6):
        lig = synth.random_ligand(np.random.default_rng(seed), 10, 2)
        it = lig.interacting
        for scale in (1.0, 1.3, 2.0):
            xyz = lig.xyz() * scale
            r = np.array([rad[int(a)] for a in lig.anum])
            d2 = ((xyz[:, None] - xyz[None]) ** 2).sum(axis=-1)
            want = bool(np.any(np.triu(it.astype(bool), 1) &
                               (d2 < (0.8 * (r[:, None] + r[None])) ** 2)))
            assert oracle.intra_clash(xyz, lig.anum, it) == want
        assert not oracle.intra_clash(lig.xyz() * 2.0, lig.anum, it)
    z = np.zeros(1)
    prot = Mol("p", np.array([0.0]), z.copy(), z.copy(), z.copy(), np.array([6], np.int32), None)
    near = np.array([[2.0, 0.0, 0.0]])
    assert oracle.heavy_atom_clash(prot, near, [8])            # 2.0 < 0.8 (1.7 + 1.55) = 2.6
    assert not oracle.heavy_atom_clash(prot, near, [1])        # hydrogens are not tested
    assert not oracle.heavy_atom_clash(prot, [[2.7, 0.0, 0.0]], [8])


def test_dock_scores_are_interpolated_energies(oracle):
    """Every unskipped exhaustive-docking score is const + the interpolated
    energy of its pose (the grid oracle), skipped ones are the clashing poses."""
    from mmo_gb300 import grids as GR
    from mmo_gb300 import synth

    s = synth.docking_site(seed=3, n_pocket=600, n_atoms=8, n_rot=1)
    types, (lt,) = GR.type2id([s.ligand])
    g = oracle.lattice(0.5, (41, 41, 41), (-10.0, -10.0, -10.0))
    rng = np.random.default_rng(0)
    grids = rng.normal(size=(len(types), 41, 41, 41)).astype(np.float32)
    vdw, _ = oracle.masks(g, s.pocket.xyz(), s.pocket.radius)
    R = np.stack([oracle.so3_rotation(6, i) for i in range(6)])
    sc, dims = oracle.dock_scores(g, grids, vdw, s.ligand, lt, s.ligand.radius, [0.0, 0.0, 0.0],
                                  1.0, 0.5, R, const_intra=2.5)
    assert dims == (5, 5, 5)
    ok = np.isfinite(sc)
    assert ok.any() and not ok.all()
    for f in np.flatnonzero(ok)[:10]:
        p, r = divmod(int(f), 6)
        i, j, k = p % 5, (p // 5) % 5, p // 25
        pos = np.array([-1.0 + 0.5 * i, -1.0 + 0.5 * j, -1.0 + 0.5 * k])
        xyz = s.ligand.xyz() @ R[r].T + pos
        e, off = oracle.ene_inter_interp(0.5, (41, 41, 41), grids, xyz + 10.0, lt)
        assert sc[f] == pytest.approx(2.5 + e, rel=1e-12, abs=1e-12)
        assert not oracle.protein_ligand_clash(g, vdw, xyz)


def test_desolvation_is_the_sum_over_shell_points(oracle):
    from mmo_gb300 import synth

    s = synth.docking_site(seed=4, n_pocket=400, n_atoms=8, n_rot=1)
    g = oracle.lattice(0.5, (41, 41, 41), (-10.0, -10.0, -10.0))
    _, shell = oracle.masks(g, s.pocket.xyz(), s.pocket.radius)
    C_ = (1.0 / 4.0 - 1.0 / 78.5) / (8.0 * np.pi)
    contrib = oracle.protein_desolv(g, s.pocket, shell, [0.0, 0.0, 0.0], 8.0)
    k, j, i = np.argwhere(contrib > 0)[0]
    p = -10.0 + 0.5 * np.array([i, j, k])
    d2 = ((s.pocket.xyz() - p) ** 2).sum(axis=1)
    want = C_ * 0.125 * np.sum(np.where(d2 < 144.0, (s.pocket.q / d2) ** 2, 0.0))
    assert contrib[k, j, i] == pytest.approx(want, rel=1e-12)
    assert np.all(contrib[shell == 0] == 0.0)
    xyz = s.ligand.xyz() + np.array([0.5, 0.0, 0.0])
    prot, lig = oracle.desolvation_penalty(g, contrib, shell, xyz, s.ligand.q, s.ligand.radius)
    _, lshell = oracle.masks(g, xyz, s.ligand.radius)
    both = (lshell > 0) & (shell > 0)
    assert prot == pytest.approx(contrib[both].sum(), rel=1e-12)
    pts = np.argwhere(both)[:, ::-1] * 0.5 - 10.0
    d2 = ((pts[:, None, :] - xyz) ** 2).sum(axis=-1)
    want = C_ * 0.125 * np.sum(np.where(d2 < 144.0, (s.ligand.q / d2) ** 2, 0.0))
    assert lig == pytest.approx(want, rel=1e-10)


# -- Monte Carlo chains: the replay that checks GPU traces step by step ---------

def _mc_setup():
    s = synth.pose_batch(n_poses=8, seed=9, n_atoms=24, n_rot=4, n_pocket=1500, radius=14.0,
                         half_box=1.0)
    prm = dict(kT=0.593, rot=math.radians(15.0), trans=0.15, tors=math.radians(5.0), law=0,
               adapt=1, flip_every=100, seed=7, roi_c=(0.0, 0.0, 0.0), roi_r=0.0,
               reset_zero=1, too_long_ends=0)
    return s, prm


def test_mc_replay_of_its_own_trace_and_planted_mistakes(oracle):
    """orc_mc_run writes a trace; orc_mc_replay of it finds no mismatch; a
    flipped outcome and a trial pose moved by one float ulp, planted in the
    trace, are each found."""
    s, prm = _mc_setup()
    tr, E, ev, st = oracle.mc_run(s.pocket, s.ligand, prm, s.poses, 500, nthreads=4)
    assert st["adapt_events"] > 0 and (ev & 1).sum() > 0
    r = oracle.mc_replay(s.pocket, s.ligand, prm, s.poses, tr, E, ev, nthreads=4)
    assert r["proposal_mismatch"] == 0 and r["decision_mismatch"] == 0
    assert r["proposals"] == r["decisions"] == 500 * len(s.poses)
    ev2 = ev.copy()
    k = tuple(np.argwhere((ev2 & 1) == 1)[3])
    ev2[k] ^= 1
    r = oracle.mc_replay(s.pocket, s.ligand, prm, s.poses, tr, E, ev2, e_tol=0.0, nthreads=4)
    assert r["decision_mismatch"] == 1
    tr2 = tr.copy()
    tr2[201, 3, 7] = np.nextafter(tr2[201, 3, 7], np.float32(10.0))
    r = oracle.mc_replay(s.pocket, s.ligand, prm, s.poses, tr2, E, ev, nthreads=4)
    assert r["proposal_mismatch"] >= 1


def test_mc_resets_of_the_reference(oracle):
    """Far from the pocket E_inter is 0: with reset_zero every frame resets
    (lds.ml:918-927); a hard ROI of 0.05 A about the start resets every rigid
    frame whose translation leaves it (lds.ml:908-916) and never a conformer
    frame, which keeps the translation."""
    s, prm = _mc_setup()
    far = s.poses[:2].copy()
    far[:, :3] += 80.0
    _, _, ev, st = oracle.mc_run(s.pocket, s.ligand, prm, far, 40, nthreads=2)
    assert np.all(ev == 2) and st["resets"] == 80
    near = s.poses[:2].copy()
    roi = dict(prm, roi_c=tuple(float(v) for v in near[0, :3]), roi_r=0.05, reset_zero=0)
    _, _, ev, _ = oracle.mc_run(s.pocket, s.ligand, roi, near[:1], 40, nthreads=1)
    assert np.all(ev[0::2] == 2) and not np.any(ev[1::2] == 2)
