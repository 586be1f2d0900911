"""ctypes binding of libmmo_gpu.so (include/mmo_gpu.h).

The library is built in-tree (mmo_gb300/build.py).  There is no fallback: if
the shared library is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmmo_gpu.so")

OK, EINVAL, ECUDA, ENOMEM, ESTATE, EELEMENT, ETIMEOUT = 0, -1, -2, -3, -4, -5, -6
DIEL_CONST, DIEL_DIST = 0, 1
MIX_GEOMEAN, MIX_LB = 0, 1
INTER_SHIFTED, INTER_GLOBAL = 0, 1
INTRA_PLAIN, INTRA_SHIFTED = 0, 1
F_INTER, F_INTRA, F_GRAD, F_RECENTER, F_GRID = 1, 2, 4, 8, 16
S_TOO_LONG, S_NONFINITE, S_OFF_GRID = 1, 2, 4

MC_UNIFORM, MC_GAUSSIAN = 0, 1
MC_ACCEPTED, MC_RESET, MC_STOPPED, MC_BLOCKED = 1, 2, 4, 8
CLASH_INTRA, CLASH_HEAVY, CLASH_GRID = 1, 2, 4


class MCParams(C.Structure):
    """mmo_mc_params of include/mmo_mc.h."""
    _fields_ = [("kT", C.c_double), ("rot_step", C.c_double), ("trans_step", C.c_double),
                ("tors_step", C.c_double), ("move_law", C.c_int), ("adapt", C.c_int),
                ("flip_every", C.c_int), ("minimize_every", C.c_int),
                ("minimize_iters", C.c_int), ("gd_step", C.c_double), ("seed", C.c_ulonglong),
                ("use_grid", C.c_int), ("roi_center", C.c_double * 3), ("roi_radius", C.c_double),
                ("reset_on_zero_inter", C.c_int), ("too_long_ends_chain", C.c_int)]


class GridSpec(C.Structure):
    """mmo_grid_spec of include/mmo_grid.h."""
    _fields_ = [("step", C.c_double), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("origin", C.c_double * 3), ("mask_center", C.c_double * 3),
                ("mask_radius", C.c_double), ("max_E", C.c_double), ("ntypes", C.c_int),
                ("type_anum", C.c_void_p), ("type_q", C.c_void_p)]


class DockSpec(C.Structure):
    """mmo_dock_spec of include/mmo_dock.h."""
    _fields_ = [("roi_center", C.c_double * 3), ("roi_radius", C.c_double),
                ("trans_step", C.c_double), ("n_rotations", C.c_int), ("topk", C.c_int),
                ("const_intra", C.c_double), ("lig_radius", C.c_void_p)]


class DockResult(C.Structure):
    """mmo_dock_result of include/mmo_dock.h."""
    _fields_ = [("n_top", C.c_int), ("best_score", C.c_double), ("best_pos", C.c_double * 3),
                ("best_rot", C.c_int), ("positions", C.c_longlong), ("poses", C.c_longlong),
                ("scored", C.c_longlong), ("clashed", C.c_longlong), ("ms", C.c_double)]


class MCState(C.Structure):
    """mmo_mc_state of include/mmo_mc.h (device pointers)."""
    _fields_ = [("dofs", C.c_void_p), ("E", C.c_void_p), ("best_dofs", C.c_void_p),
                ("best_E", C.c_void_p), ("accepted", C.c_void_p), ("status", C.c_void_p),
                ("resets", C.c_void_p), ("trace_dofs", C.c_void_p), ("trace_E", C.c_void_p),
                ("trace_event", C.c_void_p)]


class System(C.Structure):
    """mmo_system of include/mmo_systems.h."""
    _fields_ = [("n_prot", C.c_int), ("prot_x", C.c_void_p), ("prot_y", C.c_void_p),
                ("prot_z", C.c_void_p), ("prot_q", C.c_void_p), ("prot_anum", C.c_void_p),
                ("n_lig", C.c_int), ("lig_x", C.c_void_p), ("lig_y", C.c_void_p),
                ("lig_z", C.c_void_p), ("lig_q", C.c_void_p), ("lig_anum", C.c_void_p),
                ("interacting", C.c_void_p), ("nrb", C.c_int), ("bond_lr", C.c_void_p),
                ("group_offsets", C.c_void_p), ("group_atoms", C.c_void_p), ("poses", C.c_int)]


# every symbol the header declares, with its ctypes signature
_P = C.POINTER
_d, _i, _vp, _cp = C.c_double, C.c_int, C.c_void_p, C.c_char_p
SIGNATURES = {
    "mmo_last_error": (_cp, [_vp]),
    "mmo_ctx_create": (_i, [_i, _P(_vp)]),
    "mmo_ctx_destroy": (_i, [_vp]),
    "mmo_set_physics": (_i, [_vp, _i, _i, _i, _i]),
    "mmo_set_protein": (_i, [_vp, _i, _P(_d), _P(_d), _P(_d), _P(_d), _P(_i)]),
    "mmo_set_ligand": (_i, [_vp, _i, _P(_d), _P(_d), _P(_d), _P(_d), _P(_i), _P(C.c_uint8), _i,
                            _P(_i), _P(_i), _P(_i)]),
    "mmo_ene_inter": (_i, [_vp, _i, _P(_d), _P(_d), _P(_d), _P(_d), _P(_i), _P(_d)]),
    "mmo_ene_intra": (_i, [_vp, _P(_d), _P(_d), _P(_d), _P(_d)]),
    "mmo_ene_inter_parts": (_i, [_vp, _i, _P(_d), _P(_d), _P(_d), _P(_d), _P(_i), _P(_d),
                                 _P(_d)]),
    "mmo_score_poses": (_i, [_vp, _i, _P(C.c_float), _i, _P(_d), _P(C.c_float), _P(_i)]),
    "mmo_score_poses_device": (_i, [_vp, _i, _vp, _i, _vp, _vp, _vp, _vp]),
    "mmo_posed_coords": (_i, [_vp, _i, _P(C.c_float), _i, _P(_d), _P(_i)]),
    "mmo_score_poses_noalloc": (_i, [_vp, _i, _vp, _i, _vp, _vp, _vp, _vp]),
    "mmo_sync": (_i, [_vp, _vp]),
    "mmo_set_tiles": (_i, [_vp, _i, _i, _i]),
    "mmo_set_cull": (_i, [_vp, _i, C.c_double, _i, _i]),
    "mmo_mc_run": (_i, [_vp, _i, _i, _P(MCParams), _P(MCState), _vp, _i]),
    "mmo_set_systems": (_i, [_vp, _i, _P(System)]),
    "mmo_systems_layout": (_i, [_vp, _P(_i), _P(_i), _P(_i), _P(_i)]),
    "mmo_score_systems_device": (_i, [_vp, _vp, _i, _vp, _vp, _vp, _vp]),
    "mmo_score_systems": (_i, [_vp, _P(C.c_float), _i, _P(_d), _P(C.c_float), _P(_i)]),
    "mmo_tune_systems": (_i, [_vp, _vp, _i, _vp, _vp, _vp, _vp, _P(C.c_double)]),
    "mmo_systems_plan": (_i, [_vp, _P(_i), _P(_i), _P(_i)]),
    "mmo_philox4x32": (_i, [_vp, C.c_uint, C.c_uint, C.c_uint, C.c_uint, _i, _vp, _vp]),
    "mmo_tune": (_i, [_vp, _i, _vp, _i, _vp, _vp, _vp, _vp, _P(C.c_double)]),
    "mmo_set_tune_cache": (_i, [_vp, C.c_char_p]),
    "mmo_get_plan": (_i, [_vp, _P(C.c_int), _P(C.c_int), _P(C.c_int), _P(C.c_int),
                          _P(C.c_double)]),
    "mmo_device_sms": (_i, [_vp, _P(_i)]),
    "mmo_set_profiling": (_i, [_vp, _i]),
    "mmo_stage_times": (_i, [_vp, _P(C.c_float)]),
    "mmo_pair_count": (_i, [_vp, _P(C.c_double), _P(C.c_double)]),
    "mmo_last_launches": (_i, [_vp, _P(C.c_int)]),
    "mmo_fp32_fma_peak": (_i, [_vp, _P(_d), _P(_d)]),
    "mmo_diag_set_wait_polls": (_i, [_vp, C.c_longlong]),
    "mmo_diag_sincos": (_i, [_vp, _i, _P(C.c_float), _P(C.c_float)]),
    "mmo_diag_pairs_within": (_i, [_vp, C.c_double, _P(C.c_double)]),
    "mmo_build_grids": (_i, [_vp, _P(GridSpec), _P(_d)]),
    "mmo_load_grids": (_i, [_vp, _P(GridSpec), _P(C.c_float)]),
    "mmo_set_grid_build": (_i, [_vp, _i]),
    "mmo_grid_values": (_i, [_vp, _P(C.c_float)]),
    "mmo_grid_dims": (_i, [_vp, _P(_i), _P(_i), _P(_i), _P(_i)]),
    "mmo_grid_device": (_i, [_vp, _P(_vp)]),
    "mmo_grid_atom_types": (_i, [_vp, _P(_i)]),
    "mmo_grid_build_stats": (_i, [_vp, _P(_d), _P(_d), _P(_d)]),
    "mmo_ene_inter_grid": (_i, [_vp, _i, _P(_d), _P(_d), _P(_d), _P(_d), _P(_i), _P(_d), _P(_i)]),
    "mmo_build_masks": (_i, [_vp, _P(_d), _d]),
    "mmo_load_masks": (_i, [_vp, _P(C.c_uint8), _P(C.c_uint8)]),
    "mmo_mask_values": (_i, [_vp, _P(C.c_uint8), _P(C.c_uint8)]),
    "mmo_clash_poses_device": (_i, [_vp, _i, _vp, _i, _i, _vp, _vp]),
    "mmo_clash_poses": (_i, [_vp, _i, _P(C.c_float), _i, _i, _P(_i)]),
    "mmo_so3_rotations": (_i, [_i, _P(_d)]),
    "mmo_dock_exhaustive": (_i, [_vp, _P(DockSpec), _P(_d), _P(C.c_longlong), _P(DockResult)]),
    "mmo_place_in_roi": (_i, [_vp, _P(_d), _d, _i, C.c_ulonglong, _P(C.c_float),
                              _P(C.c_longlong)]),
    "mmo_set_ligand_radii": (_i, [_vp, _P(_d)]),
    "mmo_protein_desolv": (_i, [_vp, _P(_d), _d, _P(_d)]),
    "mmo_desolvation_poses_device": (_i, [_vp, _i, _vp, _i, _d, _vp, _vp, _vp, _vp]),
    "mmo_desolvation_poses": (_i, [_vp, _i, _P(C.c_float), _i, _d, _P(_d), _P(_d), _P(_i)]),
}


class MMOError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s (code %d)" % (msg, code))
        self.code = code


_lib = None


def load(path: str = LIB_PATH):
    """Load the CUDA library once; raise if it is not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError("libmmo_gpu.so is not built: run mmo_gb300.build.build() "
                               "(nvcc, sm_103a); there is no CPU fallback")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(code: int, ctx=None) -> None:
    if code != OK:
        msg = load().mmo_last_error(ctx)
        raise MMOError(code, msg.decode() if msg else "error")
