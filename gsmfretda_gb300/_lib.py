"""ctypes binding of libgpda.so (the C ABI in include/gpda.h).

The library is built in-tree by gsmfretda_gb300.build. There is no CPU
fallback: if the shared library is missing, importing a compute entry point
raises immediately.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# GPDA_LIB points at another build of the same library (e.g. a variant being timed)
LIB_PATH = os.environ.get("GPDA_LIB") or os.path.join(HERE, "libgpda.so")

GPDA_OK = 0
ERRORS = {-1: "GPDA_ERR_ARG", -2: "GPDA_ERR_SINGULAR", -3: "GPDA_ERR_CUDA",
          -4: "GPDA_ERR_NOMEM", -5: "GPDA_ERR_STATE", -6: "GPDA_ERR_LIMIT"}
MODE_OCCUPANCY = 0
MODE_PHOTON = 1


class GpdaModel(C.Structure):
    _fields_ = [("nbins", C.c_int32), ("left_pad", C.c_int32), ("gamma", C.c_float),
                ("crosstalk", C.c_float), ("bg_d", C.c_float), ("bg_a", C.c_float),
                ("r0", C.c_float), ("rc_gamma", C.c_float), ("rc_de", C.c_float),
                ("rc_ct", C.c_float), ("rc_r0", C.c_float)]


class GpdaError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_VP, _I32, _I64, _U64, _F, _D = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_float, C.c_double
_P_I32 = C.POINTER(C.c_int32)

# name: (restype, argtypes)
SIGNATURES = {
    "gpda_model_defaults": (None, [C.POINTER(GpdaModel)]),
    "gpda_version": (C.c_char_p, []),
    "gpda_create": (_VP, [_I32, C.POINTER(GpdaModel), _P_I32]),
    "gpda_destroy": (None, [_VP]),
    "gpda_last_error": (C.c_char_p, [_VP]),
    "gpda_upload_bursts": (_I32, [_VP, _VP, _VP, _VP, _VP, _I64]),
    "gpda_set_observed": (_I32, [_VP, _VP, _I32]),
    "gpda_bin_values": (_I32, [_VP, _I64, _I32, _VP]),
    "gpda_params_size": (_I32, []),
    "gpda_build_params": (_I32, [C.POINTER(GpdaModel), _I32, _VP, _VP]),
    "gpda_run_plain": (_I32, [_VP, _I32, _I32, _VP, _I64, _I64, _I32, _U64, _VP, _VP]),
    "gpda_run_batched": (_I32, [_VP, _I32, _I32, _I32, _VP, _I32, _U64, _VP, _VP]),
    "gpda_run_units": (_I32, [_VP, _I32, _I32, _I32, _VP, _I64, _I64, _I32, _U64, _VP, _VP]),
    "gpda_launch": (_I32, [_VP, _I32, _I32, _I32, _VP, _I64, _I64, _I32, _U64]),
    "gpda_fetch": (_I32, [_VP, _VP, _VP]),
    "gpda_query": (_I32, [_VP]),
    "gpda_synchronize": (_I32, [_VP]),
    "gpda_stream": (_VP, [_VP]),
    "gpda_launch_count": (_I64, [_VP]),
    "gpda_limit_hits": (_I64, [_VP]),
    "gpda_kernel_ms": (_F, [_VP]),
    "gpda_run_host": (_I32, [_VP, _I32, _I32, _I32, _VP, _VP, _VP, _VP, _VP, _I64, _I32, _U64, _I32,
                             _VP, _VP]),
    "gpda_graph_create": (_I32, [_VP, _I32, _I32, _I32, _I32]),
    "gpda_graph_run": (_I32, [_VP, _VP, _U64, _VP, _VP]),
    "gpda_autotune": (_I32, [_VP, _I32, _I32, _I32, _VP, _I32, _U64, _VP]),
    "gpda_expected_hist": (_I32, [_VP, _I32, _I32, _VP, _VP, _I32, _U64, _VP, _VP]),
    "gpda_expected_hist_adjoint": (_I32, [_VP, _I32, _I32, _VP, _VP, _I32, _U64, _VP, _VP, _VP]),
    "gpda_expected_set_tape_limit": (_I32, [_VP, _I64]),
    "gpda_expected_grad": (_I32, [_VP, _I32, _I32, _VP, _VP, _I32, _U64, _VP, _VP, _VP, _VP]),
    "gpda_run_pda_noalloc": (_I32, [C.POINTER(GpdaModel), _I32, _I32, _I32, _VP, _VP, _VP, _VP, _VP,
                                    _I64, _I32, _U64, _VP, _VP, _VP, _VP]),
    "gpda_mc_create": (_VP, [_I32, _I32, C.c_uint8, _U64, _I32, _P_I32]),
    "gpda_mc_destroy": (None, [_VP]),
    "gpda_mc_last_error": (C.c_char_p, [_VP]),
    "gpda_mc_stream_num": (_I32, [_VP]),
    "gpda_mc_sz_burst": (_I32, [_VP]),
    "gpda_mc_resample_times": (_I32, [_VP]),
    "gpda_mc_set_resample_times": (_I32, [_VP, _I32]),
    "gpda_mc_set_seed": (_I32, [_VP, _U64]),
    "gpda_mc_set_model": (_I32, [_VP, C.POINTER(GpdaModel)]),
    "gpda_mc_init_data_gpu": (_I32, [_VP, _VP, _VP, _VP, _VP, _I64, _I64, _VP, _VP, _VP, _VP, _F, _F, _F]),
    "gpda_mc_set_nstates": (_I32, [_VP, _I32, _I32]),
    "gpda_mc_set_params": (_I32, [_VP, _I32, _I32, _VP, _I32]),
    "gpda_mc_setBurstBd": (_I32, [_VP, _I32, _I32, _I32]),
    "gpda_mc_init_randstate": (_I32, [_VP, _I32, _I32]),
    "gpda_mc_set_params_buff": (_I32, [_VP, _I32, _I32, _I32]),
    "gpda_mc_run_kernel": (_I32, [_VP, _I32, _I32]),
    "gpda_mc_streamQuery": (_I32, [_VP, _I32]),
    "gpda_mc_hmcE": (C.POINTER(C.c_float), [_VP, _I32]),
    "gpda_mc_gpu_uuid": (_I32, [_VP, C.c_char_p]),
    "gpda_mc_set_hist_bins": (_I32, [_VP, _I32]),
    "gpda_mc_hist": (_I32, [_VP, _I32, _VP]),
}

_lib = None


def load():
    """Load libgpda.so; raises if it has not been built (no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m gsmfretda_gb300.build` "
                          "(the GPU path has no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def default_model(**kw) -> GpdaModel:
    m = GpdaModel()
    load().gpda_model_defaults(C.byref(m))
    for k, v in kw.items():
        setattr(m, k, v)
    return m
