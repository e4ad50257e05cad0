"""ctypes binding of libflof_gb300.so (declared in include/flof_gb300.h).

The binding is the whole bridge between Python and the CUDA library: plain
pointers, sizes and opaque handles, no torch types.  Loading fails loudly
when the library has not been built; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libflof_gb300.so")

FLOF_REAL = 1
FLOF_VEC4 = 8
FLOF_OPT_CFL_SYNC = 2
FLOF_OPT_AUTOTUNE = 3
FLOF_OPT_STRICT = 4
FLOF_OPT_SLAB_TMA = 5
FLOF_PRECISION_FP32 = 0
FLOF_PRECISION_MIXED = 1
FLOF_SOLVER_PCG = 0
FLOF_SOLVER_MG = 1
MAX_SOLVE_STATS = 64

STATUS = {
    0: "FLOF_OK", 1: "FLOF_E_ARG", 2: "FLOF_E_CUDA", 3: "FLOF_E_OOM", 4: "FLOF_E_NAN",
    5: "FLOF_E_STALL", 6: "FLOF_E_TIMEOUT", 7: "FLOF_E_STATE", 8: "FLOF_E_NOTFOUND",
}


class FlofError(RuntimeError):
    """A non-zero flof_status; mirrors the reference's errMsg exceptions."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class OFParams(ctypes.Structure):
    _fields_ = [
        ("wSmooth", ctypes.c_float), ("wEnergy", ctypes.c_float), ("level", ctypes.c_int),
        ("postVelBlur", ctypes.c_float), ("cgAccuracy", ctypes.c_float), ("blurType", ctypes.c_int),
        ("cfl", ctypes.c_float), ("orderTime", ctypes.c_int), ("orderSpace", ctypes.c_int),
        ("resetBndWidth", ctypes.c_float), ("multiStep", ctypes.c_int),
        ("projSizeThresh", ctypes.c_int), ("minGridSize", ctypes.c_int),
        ("doFinalProject", ctypes.c_int), ("cgMaxIter", ctypes.c_int),
        ("precision", ctypes.c_int), ("warmStart", ctypes.c_int), ("solver", ctypes.c_int),
        ("reserved", ctypes.c_int * 4),
    ]


class SolveStats(ctypes.Structure):
    _fields_ = [
        ("nsolves", ctypes.c_int),
        ("size_x", ctypes.c_int * MAX_SOLVE_STATS),
        ("iterations", ctypes.c_int * MAX_SOLVE_STATS),
        ("residual", ctypes.c_float * MAX_SOLVE_STATS),
        ("status", ctypes.c_int * MAX_SOLVE_STATS),
        ("cg_total_iterations", ctypes.c_int),
        ("syncs", ctypes.c_int),
        ("err_final", ctypes.c_float),
        ("seconds", ctypes.c_double),
        ("true_residual", ctypes.c_float * MAX_SOLVE_STATS),
        ("warm_start", ctypes.c_int),
        ("warm_start_err", ctypes.c_float * 2),
    ]

    def as_dict(self) -> dict:
        n = min(self.nsolves, MAX_SOLVE_STATS)
        return {
            "nsolves": self.nsolves,
            "solves": [(self.size_x[q], self.iterations[q], float(self.residual[q]), self.status[q])
                       for q in range(n)],
            "cg_total_iterations": self.cg_total_iterations,
            "syncs": self.syncs,
            "err_final": float(self.err_final),
            "seconds": float(self.seconds),
            "true_residual": [float(self.true_residual[q]) for q in range(n)],
            "warm_start": self.warm_start,
            "warm_start_err": (float(self.warm_start_err[0]), float(self.warm_start_err[1])),
        }


P = ctypes.c_void_p
I = ctypes.c_int
F = ctypes.c_float
FP = ctypes.POINTER(ctypes.c_float)
IP = ctypes.POINTER(ctypes.c_int)

# name -> (restype, argtypes); the set of entry points of include/flof_gb300.h
SIGNATURES = {
    "flof_version": (ctypes.c_char_p, []),
    "flof_last_error": (ctypes.c_char_p, []),
    "flof_status_string": (ctypes.c_char_p, [I]),
    "flof_of_params_default": (None, [P]),
    "flof_of_params_flof": (None, [P]),
    "flof_ctx_create": (I, [I, P]),
    "flof_ctx_destroy": (I, [P]),
    "flof_ctx_synchronize": (I, [P]),
    "flof_ctx_set_stream": (I, [P, P]),
    "flof_ctx_stream": (P, [P]),
    "flof_ctx_kernel_launches": (ctypes.c_longlong, [P]),
    "flof_ctx_trim": (I, [P]),
    "flof_ctx_set_option": (I, [P, I, I]),
    "flof_ctx_set_mg_params": (I, [P, F, F, F, I, I]),
    "flof_ctx_mg_fallbacks": (ctypes.c_longlong, [P]),
    "flof_ctx_profile": (I, [P, I]),
    "flof_ctx_profile_count": (I, [P, IP]),
    "flof_ctx_profile_record": (I, [P, I, IP, IP, ctypes.POINTER(ctypes.c_double), FP]),
    "flof_kernel_class_name": (ctypes.c_char_p, [I]),
    "flof_grid_create": (I, [P, P, I, P]),
    "flof_grid_wrap": (I, [P, P, I, P, P]),
    "flof_grid_destroy": (I, [P]),
    "flof_grid_dims": (I, [P, P, P]),
    "flof_grid_data": (P, [P]),
    "flof_grid_upload": (I, [P, P]),
    "flof_grid_download": (I, [P, P]),
    "flof_grid_upload_async": (I, [P, P]),
    "flof_grid_download_async": (I, [P, P]),
    "flof_grid_copy_wait": (I, [P]),
    "flof_ctx_copies_sync": (I, [P]),
    "flof_grid_copyFrom": (I, [P, P]),
    "flof_grid_add": (I, [P, P]),
    "flof_grid_sub": (I, [P, P]),
    "flof_grid_setConst": (I, [P, P]),
    "flof_grid_addConst": (I, [P, P]),
    "flof_grid_multConst": (I, [P, P]),
    "flof_grid_addScaled": (I, [P, P, P]),
    "flof_grid_clear": (I, [P]),
    "flof_grid_getMax": (I, [P, FP]),
    "flof_grid_getMin": (I, [P, FP]),
    "flof_grid_getMaxAbs": (I, [P, FP]),
    "flof_grid_setBound": (I, [P, P, I]),
    "flof_grid_setBoundNeumann": (I, [P, I]),
    "flof_opticalFlowMultiscale4d": (I, [P, P, P, P, P, FP, P]),
    "flof_opticalFlow4d": (I, [P, P, P, P, F, F, F, F, I, F, I, IP, FP]),
    "flof_corrVelsOf4d": (I, [P, P, P, P, P, P, F, F, F, F, I]),
    "flof_gaussianBlur4d": (I, [P, P, F, I]),
    "flof_advect4d": (I, [P, P, P, F]),
    "flof_calcLsDiff4d": (I, [P, P, P, P, F, I, FP]),
    "flof_calcLsDiff4d_noalloc": (I, [P, P, P, P, F, I, P, P]),
    "flof_interpolateGrid4d": (I, [P, P, P, P, P, P]),
    "flof_interpolateGrid4dVec": (I, [P, P, P, P, P, P]),
    "flof_deform4d": (I, [P, P, P, P, P, P, F, F, I]),
    "flof_loadAdvectTimeSlice_OptInit": (I, [P, I, P, I, I, F]),
    "flof_loadAdvectTimeSlice_OptRun": (I, [P, I, P, P, F, F, F, P, P, P, P, F, I, F, I, F, F]),
    "flof_loadAdvectTimeSlice_OptRunTwoway": (I, [P, I, I, P, P, P, F, F, F, F, P, P, P, P, F, I, F]),
    "flof_loadAdvectTimeSlice_Finish": (I, [P, I]),
    "flof_repeatFrame4d": (I, [P, F, F, I]),
    "flof_extrap4dLsSimple": (I, [P, I, I]),
    "flof_grid_join": (I, [P, P]),
    "flof_grid3_setBound": (I, [P, P, I]),
    "flof_grid3_setBoundNeumann": (I, [P, I]),
    "flof_simpleBlurSpecial": (I, [P, I, F, I]),
    "flof_shiftForwGrid4d": (I, [P, I]),
    "flof_loadPlaceGrid4d": (I, [P, ctypes.c_char_p, P, I, P, P, I, I, I, F, P, F, I, F, I, F, F]),
    "flof_uni_info": (I, [ctypes.c_char_p, P, IP, IP, IP]),
    "flof_grid_load": (I, [P, ctypes.c_char_p]),
    "flof_grid_save": (I, [P, ctypes.c_char_p, I]),
    "flof_uni_read_slice": (I, [P, ctypes.c_char_p, I]),
    "flof_loadAdvectTimeSlice_OptInitFile": (I, [P, I, ctypes.c_char_p, I, I, F]),
    "flof_loadAdvectTimeSlice": (I, [P, P, ctypes.c_char_p, P, P, F, F, F, P, P, P, P, F, I, F]),
    "flof_opticalFlowMultiscale4d_batch": (I, [P, I, P, P, P, P, FP, I]),
    "flof_model_create": (I, [P, I, P]),
    "flof_model_destroy": (I, [P]),
    "flof_model_num_params": (I, [P, ctypes.POINTER(ctypes.c_longlong)]),
    "flof_model_init": (I, [P, ctypes.c_ulonglong]),
    "flof_model_get_params": (I, [P, P]),
    "flof_model_set_params": (I, [P, P]),
    "flof_model_predict": (I, [P, P, P, P]),
    "flof_model_loss_grad": (I, [P, P, P, P, ctypes.POINTER(ctypes.c_double), P]),
    "flof_model_train_step": (I, [P, I, P, P, P, F, ctypes.POINTER(ctypes.c_double)]),
    "flof_ctx_set_model": (I, [P, P]),
}

_lib = None


def lib():
    """The loaded library; raises if it is missing (no fallback path)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build the CUDA library first "
                "(python -m ofblend_gb300.build); flof-gb300 has no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != 0:
        msg = lib().flof_last_error()
        raise FlofError(status, msg.decode() if msg else "")


def f4(v) -> ctypes.Array:
    """A float[4] from a scalar, a sequence or a vec3/vec4-like object."""
    if v is None:
        return None
    if hasattr(v, "x"):
        vals = [v.x, v.y, v.z, getattr(v, "t", 0.0)]
    elif isinstance(v, (int, float)):
        vals = [v, v, v, v]
    else:
        vals = list(v)
        if len(vals) == 1:
            vals = vals * 4
        while len(vals) < 4:
            vals.append(0.0)
    return (ctypes.c_float * 4)(*[float(a) for a in vals[:4]])
