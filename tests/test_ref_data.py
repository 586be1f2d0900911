"""The reference's own molecules as fixtures (tests/golden/make_ref_data.py):
the 48-atom ligand of data/docked.mol2, data/minimized.mol2 and
data/ligdecs.mol2 (one molecule in three poses), converted by this
repository's .pqrs writer, and the 3A2J receptor of data/xtal.pdb.

On the CPU: the fixtures' topology, their regeneration from the reference's
files when those are at hand, and the oracle on a real complex (the C oracle
against its NumPy twin, the analytic gradient against central differences).
The GPU side is tests/test_gpu_ref_data.py."""
import os
import sys

import numpy as np
import pytest

from mmo_gb300.topology import read_pqrs

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def ref_molecules():
    ligs = read_pqrs(os.path.join(GOLD, "ref_ligands.pqrs"))
    (rec,) = read_pqrs(os.path.join(GOLD, "ref_receptor.pqrs"))
    return rec, ligs


def test_fixture_topology():
    rec, ligs = ref_molecules()
    assert [m.name.split("|")[0] for m in ligs] == ["docked", "minimized", "ligdecs"]
    for m in ligs:
        assert m.n == 48 and m.nrb == 9
        assert np.array_equal(m.dists, ligs[0].dists)
        assert np.array_equal(m.rbonds, ligs[0].rbonds)
        assert all(np.array_equal(a, b) for a, b in zip(m.rgroups, ligs[0].rgroups))
        assert abs(m.q.sum()) < 1e-9  # the mol2 charges of a neutral molecule
        assert (m.anum == 1).sum() == 20  # 20 hydrogens (data/docked.mol2)
        # the three poses are different conformers of the same molecule
    assert np.abs(ligs[0].xyz() - ligs[1].xyz()).max() > 0.1
    assert rec.n == 2015 and set(np.unique(rec.anum)) == {6, 7, 8, 16}
    assert rec.dists is None


def test_fixture_regenerates(tmp_path):
    sys.path.insert(0, GOLD)
    import make_ref_data as G

    root = G.reference_root()
    if not root or not os.path.isdir(os.path.join(root, "data")):
        pytest.skip("the reference's data directory is not on this machine")
    G.main(root, str(tmp_path))
    for fn in ("ref_ligands.pqrs", "ref_receptor.pqrs"):
        with open(os.path.join(GOLD, fn)) as a, open(os.path.join(tmp_path, fn)) as b:
            assert a.read() == b.read(), fn


def test_oracle_twin_on_the_real_complex(oracle):
    from oracle import np_twin as T

    rec, ligs = ref_molecules()
    for m in ligs:
        for diel in (0, 1):
            ph = oracle.physics(dielectric=diel)
            e = oracle.ene_inter(rec, m, ph=ph)
            t = T.ene_inter(rec.xyz(), rec.q, rec.anum, m.xyz(), m.q, m.anum, dielectric=diel)
            assert e == pytest.approx(t, rel=1e-12, abs=1e-12)
            ei = oracle.ene_intra(m, ph=ph)
            ti = T.ene_intra(m.xyz(), m.q, m.anum, m.interacting, dielectric=diel)
            assert ei == pytest.approx(ti, rel=1e-12, abs=1e-12)
    # the docked pose binds: a favourable inter energy without clashes
    assert oracle.ene_inter(rec, ligs[0]) < -5.0


def test_oracle_gradient_on_the_real_complex(oracle):
    rec, ligs = ref_molecules()
    lig = ligs[0]
    rng = np.random.default_rng(4)
    confs = np.zeros((4, 6 + lig.nrb))
    confs[1:, :3] = rng.uniform(-0.3, 0.3, size=(3, 3))
    confs[1:, 3:] = rng.uniform(-0.2, 0.2, size=(3, 3 + lig.nrb))
    _, G, _ = oracle.score_batch(rec, lig, confs, mode=1)
    for b in range(len(confs)):
        fd = oracle.grad_fd(rec, lig, confs[b], 1e-6)
        scale = np.abs(fd).max()
        assert np.abs(G[b] - fd).max() <= 1e-5 * scale, b


def test_reference_reader_reads_our_pqrs(tmp_path):
    """The reference's own .pqrs reader (bin/pqrs_center.py: the header and the
    atom lines, their geometric centre) on molecules written by this
    repository's .pqrs writer: the same header and centre as ours."""
    import subprocess

    from mmo_gb300.topology import write_pqrs

    sys.path.insert(0, GOLD)
    import make_ref_data as G

    root = G.reference_root()
    tool = os.path.join(root, "bin", "pqrs_center.py") if root else ""
    if not os.path.isfile(tool):
        pytest.skip("the reference's bin/pqrs_center.py is not on this machine")
    rec, ligs = ref_molecules()
    for k, (m, receptor) in enumerate([(rec, True)] + [(l, False) for l in ligs]):
        fn = os.path.join(tmp_path, "m%d.pqrs" % k)
        write_pqrs(fn, [m], receptor=receptor)
        out = subprocess.run([sys.executable, tool, fn], capture_output=True, text=True,
                             check=True).stdout.splitlines()
        head = "%d:%s" % (m.n, m.name) if receptor else "%d:%d:%s" % (m.n, m.nrb, m.name)
        assert out[0] == head
        got = np.array([float(v) for v in out[1].split()])
        assert np.allclose(got, m.xyz().mean(axis=0), rtol=1e-5, atol=1e-5)
