"""
ctypes binding of ``libtaichimps_gb300.so`` (the C ABI in include/taichimps_gb300.h).

The library is the only compute path: if it is missing, or no CUDA device is
present, every entry point raises.  There is no CPU fallback.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

from . import build as _build

c_i32 = ctypes.c_int32
c_f64 = ctypes.c_double
c_vp = ctypes.c_void_p


class Box(ctypes.Structure):
    """tmps_box"""

    _fields_ = [
        ("lo", c_f64 * 3), ("hi", c_f64 * 3), ("prd", c_f64 * 3), ("inv_prd", c_f64 * 3),
        ("h_rate", c_f64 * 6),
        ("per", c_i32 * 3), ("vremap", c_i32),
        ("g", c_i32 * 3), ("ncell", c_i32),
        ("csize", c_f64 * 3), ("hcell", c_f64 * 3),
        ("old_lo", c_f64 * 3), ("old_prd", c_f64 * 3),
        ("remap_pending", c_i32), ("pad_", c_i32),
    ]


class Atoms(ctypes.Structure):
    """tmps_atoms"""

    _fields_ = [
        ("n", c_i32), ("pad_", c_i32),
        ("xr", c_vp), ("vm", c_vp), ("om", c_vp), ("f", c_vp), ("torque", c_vp), ("virial", c_vp),
        ("tag", c_vp), ("uid", c_vp), ("x0", c_vp),
        ("pos32", c_vp), ("cell32", c_vp), ("vel32", c_vp), ("om32", c_vp), ("f32", c_vp),
        ("torque32", c_vp), ("o0_32", c_vp), ("rinv", c_vp), ("pos32lo", c_vp), ("lo32", c_vp),
        ("wlz32", c_vp), ("inv32", c_vp),
    ]


class NList(ctypes.Structure):
    """tmps_nlist"""

    _fields_ = [("n", c_i32), ("slots", c_i32), ("nbr", c_vp), ("nnb", c_vp), ("touch", c_vp),
                ("shear", c_vp), ("rolling", c_vp)]


class PairParams(ctypes.Structure):
    """tmps_pair_params"""

    _fields_ = [
        ("style", c_i32), ("normal_id", c_i32), ("damping_id", c_i32), ("tangential_id", c_i32),
        ("limit_damping", c_i32), ("pad_", c_i32),
        ("kn", c_f64), ("kt", c_f64), ("gamman", c_f64), ("gammat", c_f64), ("xmu", c_f64),
        ("damp", c_f64), ("xt", c_f64), ("mu", c_f64),
        ("rolling_id", c_i32), ("pad2_", c_i32),
        ("k_roll", c_f64), ("gamma_roll", c_f64), ("mu_roll", c_f64),
    ]


class Servo(ctypes.Structure):
    """tmps_servo"""

    _fields_ = [
        ("style", c_i32 * 3), ("couple", c_i32), ("normalize", c_i32), ("remap", c_i32),
        ("max_rate", c_f64),
        ("rate", c_f64 * 3), ("vel", c_f64 * 3), ("scale", c_f64 * 3), ("flo", c_f64 * 3),
        ("fhi", c_f64 * 3), ("dlo", c_f64 * 3), ("dhi", c_f64 * 3),
        ("amp", c_f64 * 3), ("tper", c_f64 * 3), ("ptarget", c_f64 * 3), ("pgain", c_f64 * 3),
        ("lo_start", c_f64 * 3), ("hi_start", c_f64 * 3), ("cum", c_f64 * 3),
        ("pressure", c_f64 * 6),
        ("nsteps", ctypes.c_int64), ("nsteps_total", ctypes.c_int64), ("step_count", ctypes.c_int64),
        ("nevery", c_i32), ("post", c_i32),
        ("vsub", c_i32 * 3), ("vfixed", c_i32 * 3), ("vdyn1", c_i32 * 3), ("vdyn2", c_i32 * 3),
        ("vol_balance_p", c_i32), ("box_style", c_i32),
        ("vol_start", c_f64), ("box_ptarget", c_f64), ("box_pgain", c_f64), ("box_vshift", c_f64 * 3),
        ("prior_rate", c_f64 * 3), ("prior_pressure", c_f64 * 3),
        ("saved", c_i32), ("pad2_", c_i32),
    ]


class Engine(ctypes.Structure):
    """tmps_engine"""

    _fields_ = [
        ("step", ctypes.c_int64), ("last_build_step", ctypes.c_int64),
        ("aborted", c_i32), ("disp_stamp", c_i32), ("final_pending", c_i32),
        ("delay", c_i32), ("every", c_i32), ("check", c_i32),
        ("cundall", c_i32), ("servo", c_i32), ("mixed", c_i32), ("single_bin", c_i32 * 3), ("nblocks", c_i32),
        ("dt", c_f64), ("gamma_lin", c_f64), ("gamma_ang", c_f64), ("trigger_sq", c_f64),
        ("lo0", c_f64 * 3), ("h0", c_f64 * 3),
        ("dlo32", ctypes.c_float * 4), ("dh32", ctypes.c_float * 4),
        ("h32", ctypes.c_float * 4), ("prd32", ctypes.c_float * 4), ("iprd32", ctypes.c_float * 4),
        ("hlo32", ctypes.c_float * 4), ("prdlo32", ctypes.c_float * 4),
        ("remap_scale", c_f64 * 3), ("pad2_", c_f64),
        ("dt_hi", ctypes.c_float), ("dt_lo", ctypes.c_float), ("trigger32", ctypes.c_float),
        ("gamma_lin32", ctypes.c_float), ("gamma_ang32", ctypes.c_float), ("pad3_", ctypes.c_float),
        ("eps_hi", ctypes.c_float * 4), ("eps_lo", ctypes.c_float * 4),
        ("prd_ref", c_f64 * 3), ("part_off", ctypes.c_int64),
        ("shift_bound", ctypes.c_float), ("maxd2_bits", ctypes.c_uint32), ("cull", c_i32),
        ("cull_tol", ctypes.c_float),
        ("plog", ctypes.c_void_p), ("plog_len", c_i32), ("order_ready", c_i32),
        ("stop_step", ctypes.c_int64), ("touching", c_i32), ("kick_all", c_i32),
    ]


class Instance(ctypes.Structure):
    """tmps_instance"""

    _fields_ = [
        ("a", Atoms), ("nl", NList), ("p", PairParams),
        ("box", c_vp), ("eng", c_vp), ("servo", c_vp), ("scratch", c_vp),
        ("a_first", c_i32), ("a_blocks", c_i32), ("c_first", c_i32), ("c_blocks", c_i32),
    ]


class WallParams(ctypes.Structure):
    """tmps_wall_params"""

    _fields_ = [("kind", c_i32), ("axis", c_i32), ("side", c_i32), ("history", c_i32), ("hertz", c_i32),
                ("limit_damping", c_i32), ("shear_axis", c_i32), ("has_axis_bounds", c_i32),
                ("coord", c_f64), ("vwall_n", c_f64), ("vwall_s", c_f64), ("c1", c_f64), ("c2", c_f64),
                ("radius", c_f64), ("axis_lo", c_f64), ("axis_hi", c_f64), ("kn", c_f64), ("kt", c_f64),
                ("gamman", c_f64), ("gammat", c_f64), ("xmu", c_f64)]


class AdjParams(ctypes.Structure):
    """tmps_adj_params"""

    _fields_ = [("kn", c_f64), ("kt", c_f64), ("gamman", c_f64), ("gammat", c_f64), ("xmu", c_f64), ("dt", c_f64),
                ("limit_damping", c_i32), ("pad_", c_i32)]


class AdjServo(ctypes.Structure):
    """tmps_adj_servo"""

    _fields_ = [("style", c_i32 * 3), ("couple", c_i32), ("normalize", c_i32), ("pad_", c_i32),
                ("rate", c_f64 * 3), ("ptarget", c_f64 * 3), ("pgain", c_f64 * 3),
                ("lo_start", c_f64 * 3), ("hi_start", c_f64 * 3), ("max_rate", c_f64)]


class AdjRec(ctypes.Structure):
    """tmps_adj_rec"""

    _fields_ = [("lo", c_f64 * 3), ("prd", c_f64 * 3), ("cum", c_f64 * 3), ("w", c_f64 * 6), ("q", c_f64),
                ("elapsed", c_f64), ("clamp", c_i32), ("pad_", c_i32)]


class AdjSys(ctypes.Structure):
    """tmps_adj_sys"""

    _fields_ = [("n", c_i32), ("npairs", c_i32), ("x", c_vp), ("v", c_vp), ("w", c_vp), ("f", c_vp), ("t", c_vp),
                ("radius", c_vp), ("mass", c_vp), ("shear", c_vp), ("pi", c_vp), ("pj", c_vp), ("ibeg", c_vp),
                ("jbeg", c_vp), ("jlist", c_vp)]


class AdjTape(ctypes.Structure):
    """tmps_adj_tape"""

    _fields_ = [("xh", c_vp), ("vh", c_vp), ("wh", c_vp), ("f", c_vp), ("t", c_vp), ("shear", c_vp), ("mask", c_vp)]


class AdjBar(ctypes.Structure):
    """tmps_adj_bar"""

    _fields_ = [("x", c_vp), ("v", c_vp), ("w", c_vp), ("f", c_vp), ("t", c_vp), ("shear", c_vp), ("radius", c_vp),
                ("mass", c_vp), ("params", c_vp), ("box", c_vp)]


TMPS_OK, TMPS_ERR_BAD_ARG, TMPS_ERR_CUDA, TMPS_ERR_TOO_LARGE = 0, 1, 2, 3
NOALLOC_MAX_ATOMS, NOALLOC_MAX_CELLS = 1048576, 200000
STATUS_NLIST_OVERFLOW, STATUS_NONFINITE, STATUS_BOX_NONPOSITIVE, STATUS_CELL_OVERFLOW = 1, 2, 4, 8
# fields of tmps_atoms_read
FIELD = {"x": 0, "v": 1, "omega": 2, "radius": 3, "rmass": 4, "f": 5, "torque": 6, "virial": 7}

# Every entry point the header declares, with its ctypes signature.
_SIGS = {
    "tmps_version": (ctypes.c_char_p, []),
    "tmps_launch_count": (ctypes.c_longlong, []),
    "tmps_last_cuda_error": (ctypes.c_char_p, []),
    "tmps_box_set": (c_i32, [c_vp, ctypes.POINTER(Box), c_vp]),
    "tmps_verlet_initial": (c_i32, [ctypes.POINTER(Atoms), c_f64, c_vp]),
    "tmps_verlet_final": (c_i32, [ctypes.POINTER(Atoms), c_f64, c_vp]),
    "tmps_clear_forces": (c_i32, [ctypes.POINTER(Atoms), c_vp]),
    "tmps_atoms_assemble": (c_i32, [ctypes.POINTER(Atoms), c_vp, c_vp, c_vp, c_vp, c_f64, c_vp, c_f64, c_vp, c_vp,
                                    c_vp]),
    "tmps_atoms_read": (c_i32, [ctypes.POINTER(Atoms), c_i32, c_vp, c_vp, c_vp]),
    "tmps_damping_cundall": (c_i32, [ctypes.POINTER(Atoms), c_f64, c_f64, c_vp]),
    "tmps_skin_check": (c_i32, [ctypes.POINTER(Atoms), c_f64, c_i32, c_vp, c_vp]),
    "tmps_pbc": (c_i32, [ctypes.POINTER(Atoms), c_vp, c_vp]),
    "tmps_nlist_workspace_bytes": (ctypes.c_int64, [c_i32, c_i32]),
    "tmps_nlist_build": (c_i32, [ctypes.POINTER(Atoms), ctypes.POINTER(Atoms), c_vp, c_i32, c_f64,
                                 c_vp, c_vp, c_vp, ctypes.POINTER(NList), c_vp, ctypes.c_int64,
                                 c_vp, c_vp]),
    "tmps_nlist_build_noalloc": (c_i32, [ctypes.POINTER(Atoms), ctypes.POINTER(Atoms), c_vp, c_i32, c_f64,
                                         c_vp, c_vp, c_vp, ctypes.POINTER(NList), c_vp, c_vp]),
    "tmps_history_remap": (c_i32, [ctypes.POINTER(NList), ctypes.POINTER(NList), c_vp, c_vp]),
    "tmps_contact": (c_i32, [ctypes.POINTER(Atoms), ctypes.POINTER(NList), c_vp,
                             ctypes.POINTER(PairParams), c_f64, c_i32, c_i32, c_vp]),
    "tmps_contact_count": (c_i32, [ctypes.POINTER(Atoms), ctypes.POINTER(NList), c_vp, c_vp, c_vp]),
    "tmps_virial_reduce": (c_i32, [ctypes.POINTER(Atoms), c_i32, c_vp, c_vp, ctypes.c_int64, c_vp]),
    "tmps_virial_workspace_bytes": (ctypes.c_int64, [c_i32]),
    "tmps_servo_step": (c_i32, [c_vp, c_vp, c_vp, c_f64, c_f64, c_f64, c_vp, c_vp]),
    "tmps_remap_x": (c_i32, [ctypes.POINTER(Atoms), c_vp, c_vp]),
    "tmps_fused_prepare": (c_i32, [ctypes.POINTER(Atoms), c_vp, c_vp, c_vp, c_vp]),
    "tmps_mixed_unpack": (c_i32, [ctypes.POINTER(Atoms), c_vp, c_vp]),
    "tmps_mixed_history": (c_i32, [ctypes.POINTER(NList), c_i32, c_vp]),
    "tmps_fused_bounds": (c_i32, [ctypes.POINTER(Atoms), ctypes.POINTER(NList), c_vp, c_vp,
                                  ctypes.POINTER(PairParams), c_i32, c_vp, c_vp]),
    "tmps_fused_a": (c_i32, [ctypes.POINTER(Atoms), c_vp, c_vp, c_i32, c_vp, c_vp]),
    "tmps_fused_c": (c_i32, [ctypes.POINTER(Atoms), ctypes.POINTER(NList), c_vp, c_vp,
                             ctypes.POINTER(PairParams), c_i32, c_vp, c_i32, c_vp]),
    "tmps_fused_servo": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "tmps_fused_blocks": (c_i32, [c_i32, c_i32, c_i32]),
    "tmps_probe_fp64": (c_i32, [c_i32, c_i32, c_i32, c_vp, c_vp]),
    "tmps_selftest_arith": (c_i32, [c_i32, c_vp, c_i32, c_vp, c_vp, c_vp]),
    "tmps_fused_shape": (c_i32, [c_i32, c_i32, c_i32, c_i32, c_i32, ctypes.POINTER(c_i32), ctypes.POINTER(c_i32)]),
    "tmps_fused_scratch_bytes": (ctypes.c_int64, [c_i32, c_i32, c_i32]),
    "tmps_fused_settle": (c_i32, [ctypes.POINTER(Atoms), c_vp, c_vp, c_vp]),
    "tmps_fused_pressure_log": (c_i32, [c_vp, c_vp, c_i32, c_vp]),
    "tmps_batch_blocks": (c_i32, [c_i32, c_i32, c_i32, ctypes.POINTER(c_i32), ctypes.POINTER(c_i32)]),
    "tmps_batch_a": (c_i32, [c_vp, c_vp, c_i32, c_i32, c_vp]),
    "tmps_batch_c": (c_i32, [c_vp, c_vp, c_i32, c_i32, c_i32, c_vp]),
    "tmps_batch_servo": (c_i32, [c_vp, c_i32, c_vp, c_vp]),
    "tmps_batch_state": (c_i32, [c_vp, c_i32, c_vp, c_vp]),
    "tmps_wall_gran": (c_i32, [ctypes.POINTER(Atoms), ctypes.POINTER(WallParams), c_f64, c_i32, c_vp, c_vp, c_i32,
                               c_vp]),
    "tmps_adj_workspace_bytes": (ctypes.c_int64, [c_i32, c_i32]),
    "tmps_adj_pairs": (c_i32, [c_i32, c_vp, c_vp, c_vp, c_f64, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "tmps_adj_pair_map": (c_i32, [c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "tmps_adj_carry": (c_i32, [c_i32, c_i32, c_vp, c_vp, c_vp, c_i32, c_vp]),
    "tmps_adj_setup": (c_i32, [ctypes.POINTER(AdjSys), ctypes.POINTER(AdjParams), c_vp, ctypes.POINTER(AdjTape),
                               c_vp, c_vp]),
    "tmps_adj_initial": (c_i32, [ctypes.POINTER(AdjSys), ctypes.POINTER(AdjParams), ctypes.POINTER(AdjTape), c_vp,
                                 c_vp, c_vp]),
    "tmps_adj_finish": (c_i32, [ctypes.POINTER(AdjSys), ctypes.POINTER(AdjParams), ctypes.POINTER(AdjServo),
                                ctypes.POINTER(AdjTape), c_vp, ctypes.c_int64, c_vp, c_vp]),
    "tmps_adj_step_back": (c_i32, [ctypes.POINTER(AdjSys), ctypes.POINTER(AdjParams), ctypes.POINTER(AdjServo),
                                   ctypes.POINTER(AdjTape), c_vp, ctypes.c_int64, c_vp, c_vp, c_f64,
                                   ctypes.POINTER(AdjBar), c_vp, c_vp]),
    "tmps_adj_setup_back": (c_i32, [ctypes.POINTER(AdjSys), ctypes.POINTER(AdjParams), c_vp,
                                    ctypes.POINTER(AdjTape), ctypes.POINTER(AdjBar), c_vp, c_vp]),
}

_lib: ctypes.CDLL | None = None


def lib_path() -> Path:
    return _build.lib_path()


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load the CUDA library (building it first if it is absent and nvcc is present)."""
    global _lib
    if _lib is not None:
        return _lib
    p = lib_path()
    if build_if_missing:
        p = _build.build()
    if not p.exists():
        raise RuntimeError(f"taichimps_gb300 CUDA library not found at {p}; run "
                           "`python -m taichimps_gb300.build` (needs nvcc)")
    L = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class TmpsError(RuntimeError):
    pass


def check(rc: int, what: str) -> None:
    if rc != TMPS_OK:
        kind = {TMPS_ERR_BAD_ARG: "bad argument", TMPS_ERR_CUDA: "CUDA launch failure",
                TMPS_ERR_TOO_LARGE: "size beyond the fixed scratch"}.get(rc, str(rc))
        if rc == TMPS_ERR_CUDA and _lib is not None:
            kind += f" ({_lib.tmps_last_cuda_error().decode()})"
        raise TmpsError(f"{what} failed: {kind}")


def exported_symbols() -> list[str]:
    return list(_SIGS)
