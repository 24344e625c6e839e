"""ctypes binding of libtaufactor_gb300.so (the C ABI declared in include/taufactor_gb300.h).

The library is built in-tree by ``taufactor_gb300.build`` (``__graft_entry__.build()``). If it
is missing, or no CUDA device is present, the solvers raise: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libtaufactor_gb300.so")

TF_OK, TF_ERR_ARG, TF_ERR_CUDA, TF_ERR_TIMEOUT, TF_ERR_UNSUPPORTED, TF_ERR_NOTCONV = range(6)
TF_KIND_BINARY, TF_KIND_ANISOTROPIC, TF_KIND_MULTIPHASE = 0, 1, 2
TF_PERIODIC_Y, TF_PERIODIC_Z = 1, 2
TF_KIND_ELECTRODE = 3
TF_MAX_PHASES = 31
TF_MAX_HALF_SWEEPS = 4

# every symbol the header declares (checked by the CPU tests)
EXPORTS = (
    "tf_version", "tf_status_string", "tf_launch_count", "tf_geometry", "tf_pack", "tf_advance",
    "tf_layer_sums", "tf_unpack", "tf_repack", "tf_check_small_division", "tf_advance_rhs", "tf_widen_f64",
    "tf_narrow_f64", "tf_axpy_f64", "tf_residual_f64", "tf_layer_sums_f64", "tf_batch_desc_bytes", "tf_batch_tile",
    "tf_batch_describe", "tf_batch_advance", "tf_batch_layer_sums", "tf_batch_check", "tf_batch_tick",
    "tf_batch_describe_rhs", "tf_batch_advance_rhs",
    "tf_batch_converge_static", "tf_kappa_pack", "tf_kappa_advance", "tf_kappa_layer_sums",
    "tf_kappa_residual_f64", "tf_kappa_adjoint_rhs", "tf_kappa_gradient", "tf_split_to_natural_f64",
    "tf_kappa_faces", "tf_kappa_advance_faces", "tf_spans_x",
    "tf_impedance_pack", "tf_impedance_fill", "tf_impedance_sweep", "tf_impedance_metrics",
    "tf_batch_advance_tile", "tf_batch_advance_rhs_tile", "tf_label_stats", "tf_anchored_phase",
    "tf_kappa_stats", "tf_mg_coarsen", "tf_mg_restrict", "tf_mg_prolong", "tf_mg_apply", "tf_mg_dot",
    "tf_pcg_update_xr", "tf_pcg_update_p", "tf_kappa_faces_f64", "tf_kappa_residual_faces_f64",
    "tf_kappa_layer_sums_faces_f64", "tf_kappa_gradient_faces_f64", "tf_kappa_advance_fused",
    "tf_refresh_ghosts", "tf_label_map", "tf_label_sums",
)
TF_IMP_TABLE = 56
TF_BATCH_ACTIVE, TF_BATCH_CONVERGED, TF_BATCH_NEEDS_HOST = 0, 1, 2


class TfGeom(C.Structure):
    _fields_ = [("batch", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("halo_y", C.c_int32), ("halo_j", C.c_int32), ("yp", C.c_int32), ("zh", C.c_int32),
                ("zhc", C.c_int32), ("tiled", C.c_int32), ("field_elems", C.c_int64),
                ("code_bytes", C.c_int64)]


class TfOperator(C.Structure):
    _fields_ = [("kind", C.c_int32), ("periodic", C.c_int32), ("omega", C.c_float),
                ("ghost_lo", C.c_float), ("ghost_hi", C.c_float), ("ky", C.c_float), ("kz", C.c_float),
                ("n_phases", C.c_int32), ("tile", C.c_int32), ("k_max", C.c_int32),
                ("divisor", C.c_float * 256), ("face", C.c_float * 1024),
                ("conductive", C.c_uint8 * 32)]


class TfBatchState(C.Structure):
    _fields_ = [("status", C.c_void_p), ("perc", C.c_void_p), ("conv_iter", C.c_void_p),
                ("conv_parity", C.c_void_p), ("old_tau", C.c_void_p), ("tau", C.c_void_p), ("rel", C.c_void_p),
                ("d_rel", C.c_void_p), ("iter_base", C.c_void_p)]


class TfError(RuntimeError):
    """A taufactor_gb300 C-ABI call returned a non-zero status."""

    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what} failed: {status_string(status)} (status {status})")


_lib = None


def lib_path() -> str:
    return _LIB_PATH


def load():
    """Load the shared library (once); raises ImportError with a build hint if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise ImportError(f"{_LIB_PATH} is missing: build it with "
                          "`python -m taufactor_gb300.build` (needs nvcc)")
    L = C.CDLL(_LIB_PATH)
    vp, i32, i64 = C.c_void_p, C.c_int, C.c_int64
    G, O = C.POINTER(TfGeom), C.POINTER(TfOperator)
    sig = {
        "tf_version": (C.c_char_p, []),
        "tf_status_string": (C.c_char_p, [i32]),
        "tf_launch_count": (i64, []),
        "tf_geometry": (i32, [i32, i32, i32, i32, i32, G]),
        "tf_pack": (i32, [G, O, vp, vp, vp, vp, vp]),
        "tf_advance": (i32, [G, O, vp, vp, vp, i32, i32, vp, C.POINTER(C.c_int), vp]),
        "tf_layer_sums": (i32, [G, O, vp, vp, vp, vp, vp]),
        "tf_unpack": (i32, [G, O, vp, vp, vp]),
        "tf_repack": (i32, [G, O, vp, vp, vp]),
        "tf_check_small_division": (i32, [i32, vp, vp]),
        "tf_advance_rhs": (i32, [G, O, vp, vp, vp, vp, i32, i32, vp, C.POINTER(C.c_int), vp]),
        "tf_widen_f64": (i32, [G, vp, vp, vp]),
        "tf_narrow_f64": (i32, [G, O, vp, vp, vp]),
        "tf_axpy_f64": (i32, [G, vp, vp, vp]),
        "tf_residual_f64": (i32, [G, O, vp, vp, vp, vp, vp, vp]),
        "tf_layer_sums_f64": (i32, [G, O, vp, vp, vp, vp, vp]),
        "tf_batch_desc_bytes": (C.c_size_t, [i32]),
        "tf_batch_tile": (None, [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "tf_batch_describe": (i32, [i32, G, O, vp, vp, vp, vp, vp, vp, vp, vp]),
        "tf_batch_advance": (i32, [vp, vp, i32, vp, i32, vp]),
        "tf_batch_describe_rhs": (i32, [i32, G, O, vp, vp, vp, vp, vp, vp]),
        "tf_batch_advance_rhs": (i32, [vp, vp, i32, vp, i32, vp]),
        "tf_batch_advance_tile": (i32, [vp, vp, i32, vp, i32, i32, vp]),
        "tf_label_stats": (i32, [i32, i32, i32, i32, vp, vp, vp, vp]),
        "tf_kappa_stats": (i32, [i32, i32, i32, i32, vp, vp, vp, vp, vp]),
        "tf_label_map": (i32, [vp, i64, vp, vp, vp]),
        "tf_label_sums": (i32, [i32, i32, i32, i32, vp, vp, vp, i32, vp, vp]),
        "tf_anchored_phase": (i32, [i32, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp]),
        "tf_batch_advance_rhs_tile": (i32, [vp, vp, i32, vp, i32, i32, vp]),
        "tf_batch_layer_sums": (i32, [vp, vp, i32, vp, i32, vp, vp, vp]),
        "tf_batch_check": (i32, [vp, i32, vp, TfBatchState, C.c_double, i32, i32, vp]),
        "tf_batch_tick": (i32, [vp, i32, vp]),
        "tf_batch_converge_static": (i32, [vp, vp, i32, i32, i64, i64, TfBatchState, C.c_double, i32, i32, vp]),
        "tf_kappa_pack": (i32, [G, O, vp, vp, vp, vp, vp]),
        "tf_kappa_advance": (i32, [G, O, vp, vp, vp, i32, i32, vp]),
        "tf_kappa_faces": (i32, [G, vp, vp, vp, vp, vp, i32, vp]),
        "tf_spans_x": (i32, [i32, i32, i32, i32, vp, vp, vp, vp, vp, vp]),
        "tf_impedance_pack": (i32, [i32, i32, i32, i32, vp, vp, vp, vp]),
        "tf_impedance_fill": (i32, [i32, i32, i32, i32, vp, vp, C.c_double, vp, vp]),
        "tf_impedance_sweep": (i32, [i32, i32, i32, i32, i32, vp, vp, vp, vp, C.c_double, i32, i32, vp]),
        "tf_impedance_metrics": (i32, [i32, i32, i32, i32, vp, C.c_double, vp, vp, vp, vp]),
        "tf_kappa_advance_faces": (i32, [G, O, vp, vp, vp, vp, vp, vp, i32, i32, vp]),
        "tf_kappa_layer_sums": (i32, [G, vp, i32, i32, vp, vp, vp, vp]),
        "tf_kappa_residual_f64": (i32, [G, O, vp, vp, vp, i32, vp, vp, vp, vp]),
        "tf_kappa_adjoint_rhs": (i32, [G, vp, vp, C.c_double, i32, vp]),
        "tf_kappa_gradient": (i32, [G, O, vp, vp, vp, vp, C.c_double, C.c_double, C.c_double, vp]),
        "tf_split_to_natural_f64": (i32, [G, vp, vp, vp]),
        "tf_mg_coarsen": (i32, [G, vp, vp, vp, G, vp, vp, vp, vp, i32, C.c_float, vp]),
        "tf_mg_restrict": (i32, [G, vp, vp, vp, vp, vp, vp, G, vp, vp]),
        "tf_mg_prolong": (i32, [G, vp, G, vp, i32, vp]),
        "tf_mg_apply": (i32, [G, vp, vp, vp, vp, vp, vp, vp]),
        "tf_mg_dot": (i32, [G, vp, vp, vp, vp, vp, vp, vp]),
        "tf_pcg_update_xr": (i32, [G, vp, vp, vp, vp, vp, vp, vp]),
        "tf_pcg_update_p": (i32, [G, vp, vp, vp, vp, vp]),
        "tf_kappa_faces_f64": (i32, [G, vp, vp, vp, vp, vp, vp]),
        "tf_kappa_advance_fused": (i32, [G, O, vp, vp, vp, vp, vp, vp, vp, i32, i32, vp, C.POINTER(C.c_int), vp]),
        "tf_refresh_ghosts": (i32, [G, i32, vp, vp]),
        "tf_kappa_residual_faces_f64": (i32, [G, O, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
        "tf_kappa_layer_sums_faces_f64": (i32, [G, vp, vp, vp, vp, vp]),
        "tf_kappa_gradient_faces_f64": (i32, [G, O, vp, vp, vp, vp, vp, vp, vp, C.c_double, C.c_double, C.c_double,
                                              vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def status_string(status: int) -> str:
    try:
        return load().tf_status_string(status).decode()
    except ImportError:
        return f"status {status}"


def check(status: int, what: str) -> None:
    if status != TF_OK:
        if status == TF_ERR_ARG:
            raise ValueError(f"{what}: invalid argument (status {status})")
        raise TfError(status, what)
