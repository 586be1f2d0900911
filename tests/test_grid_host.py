"""Host helpers of the grid path (mmo_gb300/grids.py) against the reference's
definitions: type numbering, charge rounding, lattice sizing, grid files."""
import numpy as np
import pytest

from mmo_gb300 import grids as GR
from mmo_gb300.topology import Mol


def _mol(anum, q):
    n = len(anum)
    z = np.zeros(n)
    return Mol("m", z, z.copy(), z.copy(), np.asarray(q, np.float64),
               np.asarray(anum, np.int32), None)


def test_type2id_first_appearance_over_ligands():
    a = _mol([6, 8, 6, 7], [0.1, -0.2, 0.1, 0.0])
    b = _mol([7, 6, 16], [0.0, 0.2, 0.1])
    types, per = GR.type2id([a, b])
    assert types == [(6, 0.1), (8, -0.2), (7, 0.0), (6, 0.2), (16, 0.1)]
    assert per[0].tolist() == [0, 1, 0, 2]
    assert per[1].tolist() == [2, 3, 4]


@pytest.mark.parametrize("x,want", [(0.123, 0.12), (0.125, 0.13), (-0.125, -0.13),
                                    (-0.124, -0.12), (0.0, 0.0), (1.005, 1.0), (-2.349, -2.35)])
def test_reduce_precision(x, want):
    # Utls.reduce_precision: float (int_of_float (x *. 100. +. (+-0.5))) /. 100.
    # (1.005 * 100 = 100.49999999999999 in binary, hence 1.0)
    assert GR.reduce_precision(x) == pytest.approx(want, abs=1e-15)


def test_lattice_from_box_counts_points_as_grid_from_box():
    origin, dims = GR.lattice_from_box(0.5, (0.0, 0.0, 0.0), (10.0, 10.2, 0.5))
    assert tuple(origin) == (0.0, 0.0, 0.0)
    # num_steps = ceil(length / step), points = num_steps + 1
    assert dims == (21, 22, 2)


def test_roi_mask_radius():
    assert GR.roi_mask_radius(8.0) == 32.0


def test_ba1_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    g = rng.normal(size=(3, 4, 5, 6)).astype(np.float32)
    files = GR.write_ba1(str(tmp_path / "lig.mol2"), 0.5, (6, 5, 4), g)
    assert [f.rsplit("/", 1)[1] for f in files] == ["lig.mol2.t%d.ba1" % i for i in range(3)]
    assert open(files[0] + ".dims").read() == "step: 0.5\nx_dim: 6\ny_dim: 5\nz_dim: 4\n"
    # raw float32, x fastest: value (i, j, k) at i + j nx + k nx ny
    raw = np.fromfile(files[1], np.float32)
    assert raw[2 + 3 * 6 + 1 * 30] == g[1, 1, 3, 2]
    step, dims, back = GR.read_ba1(str(tmp_path / "lig.mol2"), 3)
    assert step == 0.5 and dims == (6, 5, 4) and np.array_equal(back, g)
    with pytest.raises(ValueError):
        GR.write_ba1(str(tmp_path / "x"), 0.5, (5, 5, 4), g)
