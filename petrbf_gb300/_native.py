"""ctypes binding of the C ABI in include/petrbf_gb300.h (libpetrbf_gb300.so).

There is no CPU fallback: if the CUDA library is missing or cannot be loaded, every
entry point raises. Build it with ``python -m petrbf_gb300.build``.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libpetrbf_gb300.so")

_D = ctypes.POINTER(ctypes.c_double)
_F = ctypes.POINTER(ctypes.c_float)
_I = ctypes.POINTER(ctypes.c_int)


class Params(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("sigma", ctypes.c_double), ("nsigma_box", ctypes.c_int),
                ("sigma_buffer", ctypes.c_int), ("sigma_trunc", ctypes.c_int),
                ("rtol", ctypes.c_double), ("abstol", ctypes.c_double), ("dtol", ctypes.c_double),
                ("restart", ctypes.c_int), ("max_it", ctypes.c_int), ("precision", ctypes.c_int),
                ("guess", ctypes.c_int), ("device", ctypes.c_int), ("pc_type", ctypes.c_int),
                ("block_fallback", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("its", ctypes.c_int), ("reason", ctypes.c_int), ("outer_its", ctypes.c_int),
                ("ncell", ctypes.c_int), ("max_block", ctypes.c_int),
                ("nblocks_fallback", ctypes.c_int), ("rnorm0", ctypes.c_double),
                ("rnorm", ctypes.c_double), ("true_rel_resid", ctypes.c_double),
                ("t_sort_ms", ctypes.c_double), ("t_setup_ms", ctypes.c_double),
                ("t_solve_ms", ctypes.c_double), ("t_total_ms", ctypes.c_double),
                ("pairs_per_matvec", ctypes.c_longlong), ("guess_used", ctypes.c_int),
                ("guess_rel_resid", ctypes.c_double), ("t_guess_ms", ctypes.c_double),
                ("fp64_fallback", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Problem(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("z", ctypes.c_void_p),
                ("f", ctypes.c_void_p), ("sigma", ctypes.c_double), ("nsigma_box", ctypes.c_int),
                ("sigma_buffer", ctypes.c_int), ("sigma_trunc", ctypes.c_int), ("g_out", ctypes.c_void_p)]


class BatchStats(ctypes.Structure):
    _fields_ = [("nprob", ctypes.c_int), ("nconverged", ctypes.c_int), ("max_its", ctypes.c_int),
                ("total_its", ctypes.c_int), ("points", ctypes.c_longlong),
                ("pairs_per_matvec", ctypes.c_longlong), ("ncell", ctypes.c_int), ("nblocks", ctypes.c_int),
                ("min_block", ctypes.c_int), ("max_block", ctypes.c_int), ("nblocks_fallback", ctypes.c_int),
                ("tile", ctypes.c_int), ("grid", ctypes.c_int), ("max_true_rel_resid", ctypes.c_double),
                ("t_sort_ms", ctypes.c_double), ("t_setup_ms", ctypes.c_double), ("t_tune_ms", ctypes.c_double),
                ("t_solve_ms", ctypes.c_double), ("t_total_ms", ctypes.c_double),
                ("t_matvec_ms", ctypes.c_double), ("t_matvec32_ms", ctypes.c_double),
                ("outer_its", ctypes.c_int), ("nprob_fp64", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# status codes (PRBF_*)
OK, ERR_ARG, ERR_RANGE, ERR_CAPACITY, ERR_CUDA, ERR_NOT_CONVERGED, ERR_BREAKDOWN, ERR_NAN, \
    ERR_STATE, ERR_FACTOR, ERR_DIVERGED, ERR_TIMEOUT = range(12)
PREC_FP64, PREC_MIXED = 0, 1
GUESS_ZERO, GUESS_LEARNED = 0, 1
PC_RASM, PC_ASM = 0, 1
FALLBACK_SHIFT, FALLBACK_LU = 0, 1
ORDER_CALLER, ORDER_CELL, MATVEC_FP32 = 0, 1, 2

# Every function the header declares, with its ctypes signature.
SIGNATURES = {
    "prbf_params_default": (None, [ctypes.POINTER(Params)]),
    "prbf_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "prbf_ctx_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_void_p)]),
    "prbf_ctx_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "prbf_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "prbf_ctx_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "prbf_ctx_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "prbf_interpolate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _D, _D, _D, _D, ctypes.c_int,
                                        _D, ctypes.POINTER(Stats)]),
    "prbf_evaluate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _D, _D, _D, ctypes.c_int, _D, _D,
                                     _D, _D, _D]),
    "prbf_matvec_setup": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _D, _D, _D]),
    "prbf_matvec": (ctypes.c_int, [ctypes.c_void_p, _D, _D]),
    "prbf_matvec_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "prbf_matvec_kernels": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int)]),
    "prbf_matvec_info": (ctypes.c_int, [ctypes.c_void_p, _I, _D, ctypes.POINTER(ctypes.c_longlong)]),
    "prbf_get_permutation": (ctypes.c_int, [ctypes.c_void_p, _I]),
    "prbf_get_cell_start": (ctypes.c_int, [ctypes.c_void_p, _I]),
    "prbf_get_trunc_counts": (ctypes.c_int, [ctypes.c_void_p, _I]),
    "prbf_pc_setup": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "prbf_pc_apply": (ctypes.c_int, [ctypes.c_void_p, _D, _D]),
    "prbf_pc_buffer_lists": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong), _I]),
    "prbf_pc_block": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _I, _I, _D, _D]),
    "prbf_cell_sort_static": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]),
    "prbf_batch_interpolate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Problem), _I, _I,
                                              ctypes.POINTER(BatchStats)]),
    # learned initial guess (include/petrbf_gb300_learned.h)
    "prbf_mlp_param_count": (ctypes.c_longlong, []),
    "prbf_mlp_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_void_p)]),
    "prbf_mlp_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "prbf_mlp_get_weights": (ctypes.c_int, [ctypes.c_void_p, _F]),
    "prbf_mlp_set_weights": (ctypes.c_int, [ctypes.c_void_p, _F]),
    "prbf_mlp_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _F, _F]),
    "prbf_mlp_loss_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _F, _F, _F, _F, _F]),
    "prbf_mlp_train": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _F, _F, _F, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_float, ctypes.c_ulonglong, _F]),
    "prbf_guess_patches": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _D, _D, _D, _D, _F, _F, _F, _F, _I]),
    "prbf_guess_set_weights": (ctypes.c_int, [ctypes.c_void_p, _F]),
    "prbf_guess_eval": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _D, _D, _D, _D]),
    "prbf_RBFInterpolation": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, _F, _F, _F,
                                             _F, ctypes.c_int, _F, _F, _F, _F, ctypes.c_float,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "prbf_selftest_wait_timeout": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint]),
    "prbf_gpumatmult_2d": (ctypes.c_int, [_F, _F, _F, _F, _F, _F, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                          ctypes.c_float, ctypes.c_int, ctypes.c_int]),
    "prbf_gpumatmult_3d": (ctypes.c_int, [_F, _F, _F, _F, _F, _F, _F, _F, ctypes.POINTER(ctypes.c_int),
                                          ctypes.c_int, ctypes.c_float, ctypes.c_int, ctypes.c_int]),
}

_lib = None


def lib():
    """Loads libpetrbf_gb300.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("petrbf_gb300 CUDA library not built (%s); run "
                               "`python -m petrbf_gb300.build`" % LIB_PATH)
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(l, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


class PrbfError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d): %s" % (lib().prbf_status_string(status).decode(), status, msg))
        self.status = status
