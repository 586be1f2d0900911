"""Host-side mirror of MMO's force-field scoring interface over the CUDA library.

MMO (src/lds.ml) scores a ligand with two closures of type Mol.t -> float:

* ``ene_inter``: ``Mol.ene_inter_UFF_global_brute`` / ``_shifted_brute`` /
  ``_shifted_bst prot_bst`` applied to the protein (src/lds.ml:1952-1955,
  1965-1967, selected by ``-ff BrG|BrL|Bst``);
* ``ene_intra``: ``Mol.ene_intra_UFFNB_brute`` (src/lds.ml:702-712).

:func:`ene_inter_builder` and :func:`ene_intra_builder` return the same
closures backed by the GPU; :class:`UFFScorer` adds the batched pose scorer
with the analytic gradient that replaces ``approx_local_gradient``
(src/lds.ml:1118-1136).  Errors follow the reference: an enclosing radius
above 12 A raises :class:`TooLong` (Mol.Too_long, src/mol.ml:587-591) where the
reference raises it (Optim.apply_config, src/optim.ml:75).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import lib as _L
from .topology import Mol


class TooLong(Exception):
    """Mol.Too_long: the conformer's enclosing radius exceeds 12 A."""


@dataclass(frozen=True)
class Physics:
    """Physics switches; the defaults are the reference's behaviour."""

    dielectric: int = _L.DIEL_CONST
    mixing: int = _L.MIX_GEOMEAN
    inter_form: int = _L.INTER_SHIFTED
    intra_form: int = _L.INTRA_PLAIN


FF_STYLES = {"BrG": _L.INTER_GLOBAL, "BrL": _L.INTER_SHIFTED, "Bst": _L.INTER_SHIFTED}


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, np.float64)


class UFFScorer:
    """One GPU context holding a protein and a ligand (libmmo_gpu.so)."""

    def __init__(self, device: int = 0, physics: Physics = Physics()):
        self._lib = _L.load()
        h = C.c_void_p()
        _L.check(self._lib.mmo_ctx_create(device, C.byref(h)), None)
        self._h = h
        self.device = device
        self.physics = physics
        self.protein: Mol | None = None
        self.ligand: Mol | None = None
        self.systems: list = []
        if physics != Physics():
            self.set_physics(physics)

    # -- lifetime --------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.mmo_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def _check(self, code: int) -> None:
        _L.check(code, self._h)

    # -- set-up ----------------------------------------------------------
    def set_physics(self, ph: Physics) -> None:
        self._check(self._lib.mmo_set_physics(self._h, ph.dielectric, ph.mixing, ph.inter_form,
                                              ph.intra_form))
        self.physics = ph

    def set_tiles(self, poses_per_lane=0, threads=0, chunks=0) -> None:
        self._check(self._lib.mmo_set_tiles(self._h, poses_per_lane, threads, chunks))

    def set_cull(self, mode=0, row_spacing=0.0, piece_atoms=0, entries_per_lane=0) -> None:
        """Cut-off sweep of the shifted form: mode 0 automatic, 1 off, 2 the
        cut-off sweep reading the protein from global memory."""
        self._check(self._lib.mmo_set_cull(self._h, mode, float(row_spacing), piece_atoms,
                                           entries_per_lane))

    def tune_device(self, d_dofs: int, B: int, d_E: int, d_grad: int | None, d_status: int,
                    flags: int, stream: int | None = None) -> float:
        """Autotune the batched sweep on this device batch (mmo_tune); returns
        the chosen plan's device ms (-1 when taken from the cache file)."""
        ms = C.c_double()
        self._check(self._lib.mmo_tune(self._h, B, d_dofs, flags, d_E, d_grad or None, d_status,
                                       stream, C.byref(ms)))
        return ms.value

    def set_tune_cache(self, path: str | None) -> None:
        self._check(self._lib.mmo_set_tune_cache(self._h, (path or "").encode()))

    def plan(self) -> dict:
        """Launch plan of the last batched call."""
        v = [C.c_int() for _ in range(4)]
        h = C.c_double()
        self._check(self._lib.mmo_get_plan(self._h, *[C.byref(x) for x in v], C.byref(h)))
        path, lane, threads, pc = (x.value for x in v)
        if path in (1, 2):
            return {"sweep": "cut-off", "entries_per_lane": lane, "threads": threads,
                    "piece_atoms": pc, "row_spacing_A": h.value,
                    "protein": "shared memory" if path == 1 else "global memory"}
        return {"sweep": "full", "poses_per_lane": lane, "threads": threads,
                "protein_chunks": pc}

    def mc_run_device(self, chains: int, steps: int, params, d_dofs: int, d_E: int,
                      d_best_dofs: int | None = None, d_best_E: int | None = None,
                      d_accepted: int | None = None, d_status: int | None = None,
                      stream: int | None = None, graph: bool = True, d_resets: int | None = None,
                      d_trace_dofs: int | None = None, d_trace_E: int | None = None,
                      d_trace_event: int | None = None) -> None:
        """Monte Carlo chains (mmo_mc_run) on device buffers; params is a
        lib.MCParams or a dict of its fields."""
        if isinstance(params, dict):
            params = dict(params)
            roi = params.pop("roi_center", None)
            params = _L.MCParams(**params)
            if roi is not None:
                params.roi_center[:] = [float(v) for v in roi]
        st = _L.MCState(d_dofs, d_E, d_best_dofs, d_best_E, d_accepted, d_status, d_resets,
                        d_trace_dofs, d_trace_E, d_trace_event)
        self._check(self._lib.mmo_mc_run(self._h, chains, steps, C.byref(params), C.byref(st),
                                         stream, int(graph)))

    def sms(self) -> int:
        out = C.c_int()
        self._check(self._lib.mmo_device_sms(self._h, C.byref(out)))
        return out.value

    def set_protein(self, prot: Mol) -> None:
        x, y, z, q = (_f64(v) for v in (prot.x, prot.y, prot.z, prot.q))
        an = np.ascontiguousarray(prot.anum, np.int32)
        self._check(self._lib.mmo_set_protein(self._h, prot.n, _dp(x), _dp(y), _dp(z), _dp(q),
                                              _ip(an)))
        self.protein = prot

    def set_ligand(self, lig: Mol) -> None:
        """``lig`` is the centred reference conformer (the ``centered_lig`` of
        src/lds.ml), with its rotatable bonds and rotation groups."""
        x, y, z, q = (_f64(v) for v in (lig.x, lig.y, lig.z, lig.q))
        an = np.ascontiguousarray(lig.anum, np.int32)
        inter = np.ascontiguousarray(lig.interacting, np.uint8)
        bonds = np.ascontiguousarray(lig.rbonds.reshape(-1), np.int32)
        off, atoms = lig.group_arrays()
        off = np.ascontiguousarray(off, np.int32)
        atoms = np.ascontiguousarray(atoms if atoms.size else np.zeros(1, np.int32), np.int32)
        if not bonds.size:
            bonds = np.zeros(2, np.int32)
        self._check(self._lib.mmo_set_ligand(
            self._h, lig.n, _dp(x), _dp(y), _dp(z), _dp(q), _ip(an),
            inter.ctypes.data_as(C.POINTER(C.c_uint8)), lig.nrb, _ip(bonds), _ip(off),
            _ip(atoms)))
        self.ligand = lig

    # -- ragged batches of systems (include/mmo_systems.h) -----------------
    def set_systems(self, systems) -> None:
        """systems: a sequence of (pocket Mol, ligand Mol, poses) triples."""
        keep, arr = [], (_L.System * max(1, len(systems)))()
        for k, (prot, lig, poses) in enumerate(systems):
            px, py, pz, pq = (_f64(v) for v in (prot.x, prot.y, prot.z, prot.q))
            pa = np.ascontiguousarray(prot.anum, np.int32)
            lx, ly, lz, lq = (_f64(v) for v in (lig.x, lig.y, lig.z, lig.q))
            la = np.ascontiguousarray(lig.anum, np.int32)
            inter = np.ascontiguousarray(lig.interacting, np.uint8)
            bonds = np.ascontiguousarray(lig.rbonds.reshape(-1), np.int32)
            off, atoms = lig.group_arrays()
            off = np.ascontiguousarray(off, np.int32)
            atoms = np.ascontiguousarray(atoms if atoms.size else np.zeros(1, np.int32), np.int32)
            if not bonds.size:
                bonds = np.zeros(2, np.int32)
            bufs = (px, py, pz, pq, pa, lx, ly, lz, lq, la, inter, bonds, off, atoms)
            keep.append(bufs)
            arr[k] = _L.System(prot.n, *(b.ctypes.data for b in bufs[:5]), lig.n,
                               *(b.ctypes.data for b in bufs[5:11]), lig.nrb,
                               bonds.ctypes.data, off.ctypes.data, atoms.ctypes.data, int(poses))
        self._check(self._lib.mmo_set_systems(self._h, len(systems), arr))
        self.systems = [(p, l, int(n)) for p, l, n in systems]

    def systems_layout(self):
        """(pose_off [nsys + 1], dof_off [nsys + 1]) of the packed layout."""
        n = len(self.systems)
        B, D = C.c_int(), C.c_int()
        po, do = (C.c_int * (n + 1))(), (C.c_int * (n + 1))()
        self._check(self._lib.mmo_systems_layout(self._h, C.byref(B), C.byref(D), po, do))
        return np.array(po[:], np.int64), np.array(do[:], np.int64)

    def score_systems(self, dofs, inter=True, intra=True, grad=False, recenter=False, out=None):
        """Packed float32 DOFs of every system's poses (systems_layout) ->
        E [B] float64, grad (packed like dofs) or None, status [B]; out: those
        arrays to fill instead of new ones (as score_poses)."""
        po, do = self.systems_layout()
        dofs = np.ascontiguousarray(dofs, np.float32).reshape(-1)
        if dofs.size != do[-1]:
            raise ValueError("dofs must hold %d floats" % do[-1])
        B = int(po[-1])
        flags = ((_L.F_INTER if inter else 0) | (_L.F_INTRA if intra else 0) |
                 (_L.F_GRAD if grad else 0) | (_L.F_RECENTER if recenter else 0))
        if out is not None:
            E, G, st = out
            ok = (E.dtype == np.float64 and E.shape == (B,) and st.dtype == np.int32 and
                  st.shape == (B,) and E.flags.c_contiguous and st.flags.c_contiguous and
                  (not grad or (G is not None and G.dtype == np.float32 and
                                G.shape == (dofs.size,) and G.flags.c_contiguous)))
            if not ok:
                raise ValueError("out must be (float64 [B], float32 [DOFs] or None, int32 [B])")
            if not grad:
                G = None
        else:
            E = np.zeros(B, np.float64)
            G = np.zeros(dofs.size, np.float32) if grad else None
            st = np.zeros(B, np.int32)
        self._check(self._lib.mmo_score_systems(
            self._h, dofs.ctypes.data_as(C.POINTER(C.c_float)), flags, _dp(E),
            G.ctypes.data_as(C.POINTER(C.c_float)) if G is not None else None, _ip(st)))
        return E, G, st

    def score_systems_device(self, d_dofs: int, d_E: int, d_grad: int | None, d_status: int,
                             flags: int, stream: int | None = None) -> None:
        self._check(self._lib.mmo_score_systems_device(self._h, d_dofs, flags, d_E,
                                                       d_grad or None, d_status, stream))

    def tune_systems_device(self, d_dofs: int, d_E: int, d_grad: int | None, d_status: int,
                            flags: int, stream: int | None = None) -> float:
        ms = C.c_double()
        self._check(self._lib.mmo_tune_systems(self._h, d_dofs, flags, d_E, d_grad or None,
                                               d_status, stream, C.byref(ms)))
        return ms.value

    def systems_plan(self) -> dict:
        kp, th, pa = C.c_int(), C.c_int(), C.c_int()
        self._check(self._lib.mmo_systems_plan(self._h, C.byref(kp), C.byref(th), C.byref(pa)))
        return {"entries_per_lane": kp.value, "threads": th.value, "piece_atoms": pa.value}

    # -- plain drop-ins (one call per Mol.t, like the reference closures) --
    def ene_inter(self, lig: Mol) -> float:
        """Mol.ene_inter_UFF_shifted_bst prot_bst prot lig (src/mol.ml:958-960)."""
        x, y, z, q = (_f64(v) for v in (lig.x, lig.y, lig.z, lig.q))
        an = np.ascontiguousarray(lig.anum, np.int32)
        out = C.c_double()
        self._check(self._lib.mmo_ene_inter(self._h, lig.n, _dp(x), _dp(y), _dp(z), _dp(q),
                                            _ip(an), C.byref(out)))
        return out.value

    def ene_inter_parts(self, lig: Mol) -> tuple[float, float]:
        """Mol.ene_inter_UFF_shifted_bst_components prot_bst prot lig
        (src/mol.ml:920-957): (electrostatic, van der Waals)."""
        x, y, z, q = (_f64(v) for v in (lig.x, lig.y, lig.z, lig.q))
        an = np.ascontiguousarray(lig.anum, np.int32)
        el, lj = C.c_double(), C.c_double()
        self._check(self._lib.mmo_ene_inter_parts(self._h, lig.n, _dp(x), _dp(y), _dp(z), _dp(q),
                                                  _ip(an), C.byref(el), C.byref(lj)))
        return el.value, lj.value

    def ene_intra(self, lig: Mol) -> float:
        """Mol.ene_intra_UFFNB_brute lig (src/mol.ml:881-903) for the ligand of
        set_ligand at lig's coordinates."""
        x, y, z = (_f64(v) for v in (lig.x, lig.y, lig.z))
        out = C.c_double()
        self._check(self._lib.mmo_ene_intra(self._h, _dp(x), _dp(y), _dp(z), C.byref(out)))
        return out.value

    # -- precomputed interaction grids (include/mmo_grid.h) ----------------
    def _grid_spec(self, step, dims, origin, types, mask_center=None, mask_radius=0.0,
                   max_E=1e5):
        ta = np.ascontiguousarray([t[0] for t in types], np.int32)
        tq = np.ascontiguousarray([t[1] for t in types], np.float64)
        sp = _L.GridSpec()
        sp.step = float(step)
        sp.nx, sp.ny, sp.nz = (int(v) for v in dims)
        sp.origin[:] = [float(v) for v in origin]
        sp.mask_center[:] = [float(v) for v in (mask_center if mask_center is not None
                                                else (0.0, 0.0, 0.0))]
        sp.mask_radius = float(mask_radius)
        sp.max_E = float(max_E)
        sp.ntypes = len(ta)
        sp.type_anum = ta.ctypes.data
        sp.type_q = tq.ctypes.data
        return sp, (ta, tq)  # the arrays must outlive the call

    def build_grids(self, step, dims, origin, types, mask_center=None, mask_radius=0.0,
                    max_E=1e5) -> float:
        """Lds.pre_calculate_FF_components_grid (src/lds.ml:452-469) on the GPU
        for the protein of set_protein: types is a list of (anum, charge);
        returns the build kernel's milliseconds."""
        sp, keep = self._grid_spec(step, dims, origin, types, mask_center, mask_radius, max_E)
        ms = C.c_double()
        self._check(self._lib.mmo_build_grids(self._h, C.byref(sp), C.byref(ms)))
        del keep
        return ms.value

    def set_grid_build(self, points_per_lane: int = 0) -> None:
        """Launch shape of the grid build (1, 2 or, under geometric mixing, 4
        lattice points per lane; 0 automatic)."""
        self._check(self._lib.mmo_set_grid_build(self._h, points_per_lane))

    def load_grids(self, step, dims, origin, types, values) -> None:
        """Grids computed elsewhere: values float32 [ntypes, nz, ny, nx]."""
        v = np.ascontiguousarray(values, np.float32)
        nx, ny, nz = (int(d) for d in dims)
        if v.size != len(types) * nx * ny * nz:
            raise ValueError("values must hold ntypes * nz * ny * nx floats")
        sp, keep = self._grid_spec(step, dims, origin, types)
        self._check(self._lib.mmo_load_grids(self._h, C.byref(sp),
                                             v.ctypes.data_as(C.POINTER(C.c_float))))
        del keep

    def grid_values(self) -> np.ndarray:
        """The context's grids, float32 [ntypes, nz, ny, nx]."""
        nt, nx, ny, nz = (C.c_int() for _ in range(4))
        self._check(self._lib.mmo_grid_dims(self._h, C.byref(nt), C.byref(nx), C.byref(ny),
                                            C.byref(nz)))
        out = np.zeros((nt.value, nz.value, ny.value, nx.value), np.float32)
        self._check(self._lib.mmo_grid_values(self._h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def grid_build_stats(self) -> dict:
        """Masked points and (point, protein atom) pair counts of the last build."""
        v = [C.c_double() for _ in range(3)]
        self._check(self._lib.mmo_grid_build_stats(self._h, *(C.byref(x) for x in v)))
        return {"points": v[0].value, "pairs_evaluated": v[1].value,
                "pairs_within_cutoff": v[2].value}

    def ene_inter_grid(self, lig: Mol):
        """Mol.ene_inter_UFF_interp on the context's grids: (energy, status)."""
        x, y, z, q = (_f64(v) for v in (lig.x, lig.y, lig.z, lig.q))
        an = np.ascontiguousarray(lig.anum, np.int32)
        out, st = C.c_double(), C.c_int()
        self._check(self._lib.mmo_ene_inter_grid(self._h, lig.n, _dp(x), _dp(y), _dp(z), _dp(q),
                                                 _ip(an), C.byref(out), C.byref(st)))
        return out.value, st.value

    def grid_atom_types(self) -> np.ndarray:
        """Grid type of each ligand atom (Mol.get_typ)."""
        out = np.zeros(self.ligand.n, np.int32)
        self._check(self._lib.mmo_grid_atom_types(self._h, _ip(out)))
        return out

    # -- binding-site clients (include/mmo_dock.h) --------------------------
    def build_masks(self, radius, r_water: float = 1.4) -> None:
        """Lds.vdW_volume and Lds.first_solvent_shell on the grids' lattice;
        radius: one per protein atom (set_protein order)."""
        r = _f64(radius)
        if r.shape != (self.protein.n,):
            raise ValueError("one radius per protein atom")
        self._check(self._lib.mmo_build_masks(self._h, _dp(r), float(r_water)))

    def load_masks(self, vdw, shell) -> None:
        v = np.ascontiguousarray(vdw, np.uint8)
        sh = np.ascontiguousarray(shell, np.uint8)
        self._check(self._lib.mmo_load_masks(self._h, v.ctypes.data_as(C.POINTER(C.c_uint8)),
                                             sh.ctypes.data_as(C.POINTER(C.c_uint8))))

    def mask_values(self):
        """(vdW volume, solvent shell) as uint8 [nz, ny, nx]."""
        nt, nx, ny, nz = (C.c_int() for _ in range(4))
        self._check(self._lib.mmo_grid_dims(self._h, C.byref(nt), C.byref(nx), C.byref(ny),
                                            C.byref(nz)))
        v = np.zeros((nz.value, ny.value, nx.value), np.uint8)
        sh = np.zeros_like(v)
        self._check(self._lib.mmo_mask_values(self._h, v.ctypes.data_as(C.POINTER(C.c_uint8)),
                                              sh.ctypes.data_as(C.POINTER(C.c_uint8))))
        return v, sh

    def clash_poses(self, dofs, tests=7, recenter=False) -> np.ndarray:
        """MMO_CLASH_* bits of each pose (int32 [B])."""
        dofs = np.ascontiguousarray(np.atleast_2d(dofs), np.float32)
        out = np.zeros(len(dofs), np.int32)
        self._check(self._lib.mmo_clash_poses(
            self._h, len(dofs), dofs.ctypes.data_as(C.POINTER(C.c_float)),
            _L.F_RECENTER if recenter else 0, int(tests), _ip(out)))
        return out

    def dock_exhaustive(self, center, radius, trans_step, n_rotations, topk=1,
                        const_intra=0.0, lig_radius=None) -> dict:
        """Lds.exhaustive_rigid_ligand_docking on the grids and the masks."""
        sp = _L.DockSpec()
        sp.roi_center[:] = [float(v) for v in center]
        sp.roi_radius = float(radius)
        sp.trans_step = float(trans_step)
        sp.n_rotations = int(n_rotations)
        sp.topk = int(topk)
        sp.const_intra = float(const_intra)
        lr = _f64(lig_radius) if lig_radius is not None else None
        sp.lig_radius = lr.ctypes.data if lr is not None else None
        scores = np.zeros(topk, np.float64)
        frames = np.zeros(topk, np.int64)
        res = _L.DockResult()
        self._check(self._lib.mmo_dock_exhaustive(
            self._h, C.byref(sp), _dp(scores), frames.ctypes.data_as(C.POINTER(C.c_longlong)),
            C.byref(res)))
        n = res.n_top
        return {"scores": scores[:n], "frames": frames[:n], "best_score": res.best_score,
                "best_pos": np.array(res.best_pos[:]), "best_rot": res.best_rot,
                "positions": res.positions, "poses": res.poses, "scored": res.scored,
                "clashed": res.clashed, "ms": res.ms}

    def place_in_roi(self, center, radius, n, seed=0):
        """Lds.place_ligand_in_ROI: (dofs float32 [n, 6 + nrb], candidates drawn)."""
        c = _f64(center)
        out = np.zeros((n, 6 + self.ligand.nrb), np.float32)
        tr = C.c_longlong()
        self._check(self._lib.mmo_place_in_roi(self._h, _dp(c), float(radius), int(n),
                                               C.c_ulonglong(seed),
                                               out.ctypes.data_as(C.POINTER(C.c_float)),
                                               C.byref(tr)))
        return out, tr.value

    def set_ligand_radii(self, radius) -> None:
        r = _f64(radius)
        self._check(self._lib.mmo_set_ligand_radii(self._h, _dp(r)))

    def protein_desolv(self, center, radius, download=True):
        """Lds.protein_desolv: float64 [nz, ny, nx] (or None without download)."""
        c = _f64(center)
        out = None
        if download:
            nt, nx, ny, nz = (C.c_int() for _ in range(4))
            self._check(self._lib.mmo_grid_dims(self._h, C.byref(nt), C.byref(nx), C.byref(ny),
                                                C.byref(nz)))
            out = np.zeros((nz.value, ny.value, nx.value), np.float64)
        self._check(self._lib.mmo_protein_desolv(self._h, _dp(c), float(radius),
                                                 _dp(out) if out is not None else None))
        return out

    def desolvation_poses(self, dofs, r_water=1.4, recenter=False):
        """Lds.desolvation_penalty of each pose: (prot, lig, status)."""
        dofs = np.ascontiguousarray(np.atleast_2d(dofs), np.float32)
        B = len(dofs)
        prot, lig = np.zeros(B), np.zeros(B)
        st = np.zeros(B, np.int32)
        self._check(self._lib.mmo_desolvation_poses(
            self._h, B, dofs.ctypes.data_as(C.POINTER(C.c_float)),
            _L.F_RECENTER if recenter else 0, float(r_water), _dp(prot), _dp(lig), _ip(st)))
        return prot, lig, st

    # -- batched poses -----------------------------------------------------
    def score_poses(self, dofs, inter=True, intra=True, grad=False, recenter=False, grid=False,
                    out=None):
        """E (float64 [B]), grad (float32 [B, 6+nrb] or None), status (int32 [B]).

        dofs: float32 [B, 6 + nrb] in the Optim.config layout
        [x, y, z, a, b, g, tau_0 ...] (src/optim.ml:19-22); grid: the inter
        term interpolated from the grids of build_grids / load_grids.  out:
        (E, grad or None, status) arrays to fill instead of new ones (for
        instance views of page-locked memory, which the copies reach by DMA)."""
        dofs = np.ascontiguousarray(dofs, np.float32)
        if dofs.ndim == 1:
            dofs = dofs[None, :]
        B, nd = dofs.shape
        if self.ligand is None or nd != 6 + self.ligand.nrb:
            raise ValueError("dofs must be [B, 6 + nrb] for the ligand of set_ligand")
        flags = ((_L.F_INTER if inter else 0) | (_L.F_INTRA if intra else 0) |
                 (_L.F_GRAD if grad else 0) | (_L.F_RECENTER if recenter else 0) |
                 (_L.F_GRID if grid else 0))
        if out is not None:
            E, G, st = out
            ok = (E.dtype == np.float64 and E.shape == (B,) and st.dtype == np.int32 and
                  st.shape == (B,) and E.flags.c_contiguous and st.flags.c_contiguous and
                  (not grad or (G is not None and G.dtype == np.float32 and G.shape == (B, nd)
                                and G.flags.c_contiguous)))
            if not ok:
                raise ValueError("out must be (float64 [B], float32 [B, 6+nrb] or None, int32 [B])")
            if not grad:
                G = None
        else:
            E = np.zeros(B, np.float64)
            G = np.zeros((B, nd), np.float32) if grad else None
            st = np.zeros(B, np.int32)
        self._check(self._lib.mmo_score_poses(
            self._h, B, dofs.ctypes.data_as(C.POINTER(C.c_float)), flags, _dp(E),
            G.ctypes.data_as(C.POINTER(C.c_float)) if G is not None else None, _ip(st)))
        return E, G, st

    def posed_coords(self, dofs, recenter=False):
        """(xyz float64 [B, L, 3], status int32 [B]): the ligand's atoms after the
        pose map (Optim.apply_config, or the MC map with recenter), as scored."""
        dofs = np.ascontiguousarray(dofs, np.float32)
        if dofs.ndim == 1:
            dofs = dofs[None, :]
        B, nd = dofs.shape
        if self.ligand is None or nd != 6 + self.ligand.nrb:
            raise ValueError("dofs must be [B, 6 + nrb] for the ligand of set_ligand")
        xyz = np.zeros((B, self.ligand.n, 3), np.float64)
        st = np.zeros(B, np.int32)
        self._check(self._lib.mmo_posed_coords(
            self._h, B, dofs.ctypes.data_as(C.POINTER(C.c_float)),
            _L.F_RECENTER if recenter else 0, _dp(xyz), _ip(st)))
        return xyz, st

    def score_config(self, conf, recenter=False) -> float:
        """E_inter + E_intra of one Optim.config, raising TooLong as
        Optim.apply_config does (src/optim.ml:75)."""
        E, _, st = self.score_poses(np.asarray(conf, np.float32)[None, :], recenter=recenter)
        if st[0] & _L.S_TOO_LONG:
            raise TooLong()
        return float(E[0])

    def score_poses_device(self, d_dofs: int, B: int, d_E: int, d_grad: int | None,
                           d_status: int, flags: int, stream: int | None = None) -> None:
        """Raw device-pointer entry point (integers are device addresses)."""
        self._check(self._lib.mmo_score_poses_device(self._h, B, d_dofs, flags, d_E,
                                                     d_grad or None, d_status, stream))

    def sync(self, stream: int | None = None) -> None:
        self._check(self._lib.mmo_sync(self._h, stream))

    # -- measurement ------------------------------------------------------
    def set_profiling(self, on: bool) -> None:
        self._check(self._lib.mmo_set_profiling(self._h, int(on)))

    def stage_times(self):
        """(rebuild, pair sweep, finish, entry sort) device ms of the last
        scoring call."""
        ms = (C.c_float * 4)()
        self._check(self._lib.mmo_stage_times(self._h, ms))
        return tuple(float(v) for v in ms)

    def pair_count(self):
        """(pairs evaluated, all pairs) of the last batched scoring call."""
        ev, al = C.c_double(), C.c_double()
        self._check(self._lib.mmo_pair_count(self._h, C.byref(ev), C.byref(al)))
        return ev.value, al.value

    def pairs_within(self, r: float = 12.0) -> float:
        """(posed ligand atom, protein atom) pairs closer than r in the last
        batched scoring call (mmo_diag_pairs_within)."""
        out = C.c_double()
        self._check(self._lib.mmo_diag_pairs_within(self._h, float(r), C.byref(out)))
        return out.value

    def last_launches(self) -> int:
        """Kernels the last scoring call launched."""
        n = C.c_int()
        self._check(self._lib.mmo_last_launches(self._h, C.byref(n)))
        return n.value

    def fp32_peak_tflops(self) -> float:
        t, ms = C.c_double(), C.c_double()
        self._check(self._lib.mmo_fp32_fma_peak(self._h, C.byref(t), C.byref(ms)))
        return t.value


def so3_rotations(n: int) -> np.ndarray:
    """SO3.rotations (src/SO3.ml:18-46): float64 [n, 3, 3]."""
    out = np.zeros((n, 3, 3), np.float64)
    _L.check(_L.load().mmo_so3_rotations(int(n), _dp(out)))
    return out


def ene_inter_builder(prot: Mol, ff_style: str = "Bst", device: int = 0,
                      physics: Physics = Physics()):
    """``ff0 prot`` of src/lds.ml:1952-1967 on the GPU: Mol -> float."""
    ph = Physics(physics.dielectric, physics.mixing, FF_STYLES[ff_style], physics.intra_form)
    s = UFFScorer(device, ph)
    s.set_protein(prot)

    def ene_inter(lig: Mol) -> float:
        return s.ene_inter(lig)

    ene_inter.scorer = s
    return ene_inter


def ene_inter_interp_builder(prot: Mol, ligands, step=0.5, margin=36.0, roi=None,
                             device: int = 0, physics: Physics = Physics()):
    """``ff1`` of src/lds.ml:1963-1975 on the GPU: the per-type grids of the
    ligands' (element, charge) types built from prot (Grid.from_box over the
    protein's box plus margin; mask sphere of the ROI (centre, outer radius)
    plus 24 A when roi is given), then the closure
    Mol.ene_inter_UFF_interp grid ff_comps : Mol -> float."""
    from . import grids as GR

    s = UFFScorer(device, physics)
    s.set_protein(prot)
    types, _ = GR.type2id(list(ligands))
    p = prot.xyz()
    origin, dims = GR.lattice_from_box(step, p.min(axis=0) - margin, p.max(axis=0) + margin)
    if roi is not None:
        s.build_grids(step, dims, origin, types, mask_center=roi[0],
                      mask_radius=GR.roi_mask_radius(roi[1]))
    else:
        s.build_grids(step, dims, origin, types)

    def ene_inter(lig: Mol) -> float:
        return s.ene_inter_grid(lig)[0]

    ene_inter.scorer = s
    ene_inter.types = types
    return ene_inter


def ene_intra_builder(centered_lig: Mol, tweak_rbonds: bool = True, device: int = 0,
                      physics: Physics = Physics()):
    """``ene_intra_builder UFF_NB`` of src/lds.ml:702-712 on the GPU: for a
    rigid ligand (or no rotatable bond) the constant E_intra of the start
    conformer, else Mol -> E_intra."""
    s = UFFScorer(device, physics)
    s.set_ligand(centered_lig)
    if tweak_rbonds and centered_lig.nrb > 0:
        def ene_intra(lig: Mol) -> float:
            return s.ene_intra(lig)
    else:
        const = s.ene_intra(centered_lig)

        def ene_intra(_lig: Mol) -> float:
            return const
    ene_intra.scorer = s
    return ene_intra
