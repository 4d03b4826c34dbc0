"""ctypes binding of librtg.so (declarations in include/rtg.h).

There is no fallback: if the library cannot be built or loaded, every call
raises.  Device buffers are passed as raw pointers (torch ``data_ptr()``)."""
import ctypes as C
import os
import threading

from . import build as _build

RTG_OK = 0
RTG_ERR_ARG = 1
RTG_ERR_MESH = 2
RTG_ERR_CUDA = 3
RTG_ERR_TIMEOUT = 4
RTG_ERR_NONFINITE = 5
RTG_ERR_SIZE = 6

RTG_MASS = 1
RTG_SCAT = 2
RTG_IC = 4
RTG_BC = 8
RTG_SYSTEM = 16
RTG_MASK_ROWS = 32

RTG_FP64 = 0
RTG_FP32 = 1

RTG_NN_IN = 16
RTG_NN_HIDDEN = 128
RTG_NN_MOM = 8
RTG_NN_OUT = 24
RTG_NN_STATS = 12
RTG_NN_NPARAM = 21784

i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
f64p = C.POINTER(C.c_double)


class MeshDesc(C.Structure):
    _fields_ = [("ncols", C.c_int32), ("nelem", C.c_int32),
                ("col_pos", f64p), ("col_ndofs", i32p), ("col_lv", i32p), ("col_nbr", i32p),
                ("col_elem_start", i32p), ("cell_pos", f64p), ("cell_ndof", i32p),
                ("cell_lv", i32p), ("cell_idx", i32p), ("cell_quadrant", i32p)]


class Coeffs(C.Structure):
    _fields_ = [("kappa", f64p), ("sigma", f64p), ("nsig", C.c_int32), ("sig_off", i64p),
                ("phi", f64p), ("col_sig", i32p)]


class Info(C.Structure):
    _fields_ = [("ndof", C.c_int64), ("ndof_interior", C.c_int64), ("ncols", C.c_int32),
                ("nelem", C.c_int32), ("ncoupling", C.c_int32), ("nsig", C.c_int32),
                ("max_col_ndof", C.c_int32), ("max_nth_col", C.c_int32),
                ("table_bytes", C.c_int64), ("bytes_per_apply_fp64", C.c_int64),
                ("bytes_per_apply_fp32", C.c_int64), ("flops_per_apply", C.c_int64)]


class SolveOpts(C.Structure):
    _fields_ = [("method", C.c_int32), ("restart", C.c_int32), ("max_it", C.c_int32),
                ("rtol", C.c_double), ("atol", C.c_double), ("precond", C.c_int32),
                ("nonzero_guess", C.c_int32), ("inner_rtol", C.c_double),
                ("max_outer", C.c_int32), ("verbose", C.c_int32)]


class SolveInfo(C.Structure):
    _fields_ = [("converged", C.c_int32), ("iterations", C.c_int32), ("outer", C.c_int32),
                ("fp64_applies", C.c_int32), ("fp32_applies", C.c_int32), ("res0", C.c_double),
                ("res_f", C.c_double), ("rhs_norm", C.c_double), ("seconds", C.c_double),
                ("hist_len", C.c_int32), ("sweeps", C.c_int32), ("learned", C.c_int32),
                ("fallbacks", C.c_int32), ("coarse", C.c_int32), ("trial_its", C.c_int32),
                ("learned_kept", C.c_int32)]


# exported symbol -> (restype, argtypes)
SIGNATURES = {
    "rtg_abi_version": (C.c_int, []),
    "rtg_last_error": (C.c_char_p, []),
    "rtg_launch_count": (C.c_int64, []),
    "rtg_quad_nodes": (C.c_int, [C.c_int, C.c_int, f64p, f64p]),
    "rtg_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(Coeffs), C.c_int, C.POINTER(C.c_void_p)]),
    "rtg_destroy": (None, [C.c_void_p]),
    "rtg_get_info": (C.c_int, [C.c_void_p, C.POINTER(Info)]),
    "rtg_apply": (C.c_int, [C.c_void_p, C.c_uint32, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_interior_mask": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_precondition": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_mask_vector": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_split_vector": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_merge_vectors": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_weight_forcing": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(SolveOpts),
                            C.POINTER(SolveInfo), f64p, C.c_int, C.c_void_p]),
    "rtg_solve_hessenberg": (C.c_int, [C.c_void_p, f64p, C.c_int, i32p, C.c_void_p]),
    "rtg_solve_batched": (C.c_int, [C.c_void_p, C.c_int, i64p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.POINTER(SolveOpts), C.POINTER(SolveInfo), C.c_void_p]),
    "rtg_dots_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                   C.c_void_p, C.c_void_p]),
    "rtg_sweep_info": (C.c_int, [C.c_void_p, i32p, i32p, i64p, C.c_void_p]),
    "rtg_apply_tuning": (C.c_int, [C.c_void_p, i32p, C.c_int, i32p, C.c_void_p]),
    "rtg_apply_shape": (C.c_int, [C.c_void_p, C.c_int, i32p]),
    "rtg_error_angular_jump": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_error_spatial_jump": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_hp_steer": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_sweep_maps": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_void_p]),
    "rtg_sweep_trace": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, i32p, C.c_void_p]),
    "rtg_nn_rows": (C.c_int, [C.c_void_p, i64p]),
    "rtg_nn_set_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_nn_features": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_nn_moments": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_nn_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "rtg_nn_correct": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_nn_targets": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                 C.c_void_p, C.c_void_p]),
    "rtg_nn_work_floats": (C.c_int64, []),
    "rtg_nn_loss_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p]),
    "rtg_nn_adam": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_float,
                              C.c_float, C.c_float, C.c_float, C.c_void_p]),
    "rtg_nn_precondition": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
}

_lib = None
_lock = threading.Lock()


class RtgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("librtg error {}: {}".format(code, msg))
        self.code = code


def load():
    """Build (if stale) and load librtg.so; raise if either fails."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.build()
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.rtg_abi_version() != 1:
            raise RuntimeError("librtg ABI version mismatch")
        _lib = lib
        return lib


def check(rc):
    if rc != RTG_OK:
        msg = load().rtg_last_error()
        raise RtgError(rc, msg.decode() if msg else "")


def lib_path():
    return _build.LIB


def ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))
