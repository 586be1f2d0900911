"""Host helpers of the precomputed-grid path (include/mmo_grid.h).

The reference's default inter energy interpolates per-type grids
(src/lds.ml:1963-1975).  This module restates its set-up steps that are not
GPU work:

* :func:`type2id` -- the ligand atom types, unique (anum, charge) pairs in order
  of first appearance over the ligands (Mol.get_type2id_ht, src/mol.ml:280-293)
  and each atom's type (Mol.assign_FF_types, src/mol.ml:456-461);
* :func:`reduce_precision` -- the --less-charges rounding to 0.01 e
  (Utls.reduce_precision, src/utls.ml:129-132) that merges types;
* :func:`lattice_from_box` -- Grid.from_box (src/grid.ml:40-52):
  ceil(length / step) + 1 points per axis from the box's low corner;
* :func:`roi_mask_radius` -- the mask of Lds.bitmask_ROI_only
  (src/lds.ml:269-274): the ROI's outer radius plus twice the 12 A cut-off;
* :func:`write_ba1` / :func:`read_ba1` -- the grid files of
  G3D.to_ba1_file / of_ba1_file (src/G3D.ml:14-64): raw native float32 values
  (x fastest) and a text ``.dims`` file; files are named
  ``<prefix>.t<i>.ba1`` after the types' names ``t<i>``
  (Mol.get_all_vdW_elec_types, src/mol.ml:295-304).  The reference also
  reads zstd-compressed ``.ba1.zst`` files; zstd is not available here, so
  those are not read.
"""
from __future__ import annotations

import math

import numpy as np

CHARGED_CUTOFF = 12.0   # A (src/const.ml:12)
GRID_STEP = 0.5         # A (Params.grid_step, src/params.ml:22)
MAX_E = 100000.0        # Params.max_E (src/params.ml:26)


def reduce_precision(x: float) -> float:
    """Utls.reduce_precision: round to 0.01, halves away from zero (truncating
    x * 100 +- 0.5 toward zero)."""
    return float(int(x * 100.0 + (0.5 if x >= 0.0 else -0.5))) / 100.0


def type2id(ligands):
    """(types, per-ligand atom types): types a list of (anum, charge) in order
    of first appearance over the ligands' atoms; each ligand's int32 array of
    type ids."""
    ids = {}
    types = []
    per = []
    for lig in ligands:
        t = np.empty(lig.n, np.int32)
        for i in range(lig.n):
            key = (int(lig.anum[i]), float(lig.q[i]))
            if key not in ids:
                ids[key] = len(types)
                types.append(key)
            t[i] = ids[key]
        per.append(t)
    return types, per


def lattice_from_box(step: float, lo, hi):
    """(origin, dims) of Grid.from_box for the box [lo, hi]: the lowest point
    at lo and ceil((hi - lo) / step) + 1 points per axis."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    dims = tuple(int(math.ceil((h - l) / step)) + 1 for l, h in zip(lo, hi))
    return lo.copy(), dims


def roi_mask_radius(roi_out_radius: float) -> float:
    """Radius of the lattice mask of Lds.bitmask_ROI_only."""
    return roi_out_radius + 2.0 * CHARGED_CUTOFF


def ba1_name(prefix: str, i: int) -> str:
    return "%s.t%d.ba1" % (prefix, i)


def write_ba1(prefix: str, step: float, dims, grids) -> list:
    """One ``.ba1`` file (and its ``.dims``) per type of grids
    float32 [ntypes, nz, ny, nx]; returns the file names."""
    g = np.ascontiguousarray(grids, np.float32)
    nx, ny, nz = (int(d) for d in dims)
    if g.ndim != 4 or g.shape[1:] != (nz, ny, nx):
        raise ValueError("grids must be [ntypes, nz, ny, nx]")
    out = []
    for i in range(g.shape[0]):
        fn = ba1_name(prefix, i)
        g[i].tofile(fn)
        with open(fn + ".dims", "w") as f:
            f.write("step: %g\nx_dim: %d\ny_dim: %d\nz_dim: %d\n" % (step, nx, ny, nz))
        out.append(fn)
    return out


def parse_dims(fn: str):
    """G3D.parse_dims_file: (step, (x_dim, y_dim, z_dim))."""
    vals = {}
    with open(fn) as f:
        for line in f:
            if ":" in line:
                k, v = line.split(":", 1)
                vals[k.strip()] = v.strip()
    return float(vals["step"]), (int(vals["x_dim"]), int(vals["y_dim"]), int(vals["z_dim"]))


def read_ba1(prefix: str, ntypes: int):
    """(step, dims, grids float32 [ntypes, nz, ny, nx]) from the files of
    write_ba1 (or of the reference, uncompressed)."""
    step, dims = parse_dims(ba1_name(prefix, 0) + ".dims")
    nx, ny, nz = dims
    out = np.empty((ntypes, nz, ny, nx), np.float32)
    for i in range(ntypes):
        fn = ba1_name(prefix, i)
        s, d = parse_dims(fn + ".dims")
        if d != dims or s != step:
            raise ValueError("%s: dims differ from type 0" % fn)
        v = np.fromfile(fn, np.float32)
        if v.size != nx * ny * nz:
            raise ValueError("%s: %d values, expected %d" % (fn, v.size, nx * ny * nz))
        out[i] = v.reshape(nz, ny, nx)
    return step, dims, out
