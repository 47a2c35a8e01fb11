"""ctypes binding of libglobe_gb300.so (the C ABI in include/globe.h).

The library is built in-tree (``globe_gb300/build.py``).  There is no
fallback: if the shared library is missing or cannot be loaded, ``lib()``
raises.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("GLOBE_LIB", os.path.join(HERE, "libglobe_gb300.so"))

GLOBE_OK = 0
ERRORS = {-1: "GLOBE_ERR_ARG", -2: "GLOBE_ERR_CUDA", -3: "GLOBE_ERR_STATE", -4: "GLOBE_ERR_IO",
          -5: "GLOBE_ERR_FORMAT", -6: "GLOBE_ERR_NOMEM", -7: "GLOBE_ERR_NUMERIC", -8: "GLOBE_ERR_UNSUPPORTED"}
PREC_FP64, PREC_MIXED = 0, 1
RULE_PCGSOLVER, RULE_AIREML = 0, 1
MODEL_FULL, MODEL_NO_TIME = 0, 1
X0_ZERO, X0_PRECOND, X0_GIVEN = 0, 1, 2
PROF_GRM, PROF_GRM_PASS1, PROF_GRM_PASS2, PROF_PCG_ITER = 0, 1, 2, 3
PROF_GRM_BUILD, PROF_GRM_BUILD_GEMM = 4, 5


class PcgOpts(C.Structure):
    _fields_ = [("tol", C.c_double), ("maxit", C.c_int), ("rule", C.c_int), ("x0mode", C.c_int),
                ("mask", C.c_int), ("precision", C.c_int)]


class PcgInfo(C.Structure):
    _fields_ = [("iters", C.c_int), ("inner_iters", C.c_int), ("rhs_iters", C.c_int64),
                ("max_rel_res", C.c_double), ("converged", C.c_int), ("stagnated", C.c_int)]


class BedInfo(C.Structure):
    _fields_ = [("M", C.c_int64), ("kept", C.c_int64)]


class AiremlOpts(C.Structure):
    _fields_ = [("maxiter", C.c_int), ("tol", C.c_double), ("numMC", C.c_int), ("theta0", C.c_double * 5),
                ("pcg_tol", C.c_double), ("pcg_maxit", C.c_int), ("precision", C.c_int), ("mask", C.c_int),
                ("seed", C.c_uint64), ("probes", C.POINTER(C.c_double)), ("probes_len", C.c_int64),
                ("fuse", C.c_int), ("digits", C.c_int)]


class AiremlResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("theta", C.c_double * 5),
                ("se", C.c_double * 5), ("ai", C.c_double * 25), ("grad", C.c_double * 5),
                ("grad_evals", C.c_int64), ("pcg_rhs_iters", C.c_int64)]


_vp = C.c_void_p
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_u8p = C.POINTER(C.c_uint8)

# name -> (restype, argtypes)
SIGNATURES = {
    "globe_create": (C.c_int, [C.POINTER(_vp), C.c_int]),
    "globe_destroy": (None, [_vp]),
    "globe_last_error": (C.c_char_p, [_vp]),
    "globe_get_stream": (C.c_int, [_vp, C.POINTER(_vp)]),
    "globe_synchronize": (C.c_int, [_vp]),
    "globe_device_bytes": (C.c_int64, [_vp]),
    "globe_kernel_launches": (C.c_int64, [_vp]),
    "globe_get_dims": (C.c_int, [_vp, _i64p, _i32p, _i32p, _i64p]),
    "globe_load_records": (C.c_int, [_vp, C.c_int64, C.c_int32, C.c_int32, _i32p, _dp, _dp]),
    "globe_load_bed": (C.c_int, [_vp, _u8p, C.c_int64, C.c_float, C.c_float, _i64p, _i64p, _fp, _fp, _u8p,
                                 C.POINTER(BedInfo)]),
    "globe_load_bed_dev": (C.c_int, [_vp, _vp, C.c_int64, C.c_int64, C.c_float, C.c_float, _vp, _vp, _vp, _vp,
                                     _vp, C.POINTER(BedInfo)]),
    "globe_load_bed_file": (C.c_int, [_vp, C.c_char_p, C.c_float, C.c_float, C.c_int64, _i64p, _i64p, _fp, _fp,
                                      _u8p, C.POINTER(BedInfo)]),
    "globe_load_grm": (C.c_int, [_vp, _fp, C.c_int32]),
    "globe_set_individuals": (C.c_int, [_vp, C.c_int32]),
    "globe_set_digits": (C.c_int, [_vp, C.c_int]),
    "globe_debug_stall_next_gemm": (C.c_int, [_vp]),
    "globe_get_digits": (C.c_int, [_vp]),
    "globe_set_graphs": (C.c_int, [_vp, C.c_int]),
    "globe_get_graphs": (C.c_int, [_vp]),
    "globe_set_device_loop": (C.c_int, [_vp, C.c_int]),
    "globe_get_device_loop": (C.c_int, [_vp]),
    "globe_device_loop_runs": (C.c_int64, [_vp]),
    "globe_set_record_df": (C.c_int, [_vp, C.c_int]),
    "globe_get_record_df": (C.c_int, [_vp]),
    "globe_record_df_solves": (C.c_int64, [_vp]),
    "globe_set_autotune": (C.c_int, [_vp, C.c_int]),
    "globe_get_autotune": (C.c_int, [_vp]),
    "globe_autotune_log": (C.c_int64, [_vp, C.c_char_p, C.c_int64]),
    "globe_debug_force_splits": (C.c_int, [_vp, C.c_int]),
    "globe_debug_bounds": (C.c_int, [C.POINTER(C.c_uint32)]),
    "globe_grm_build": (C.c_int, [_vp, _fp]),
    "globe_grm_build_dev": (C.c_int, [_vp, _vp]),
    "globe_write_grm": (C.c_int, [C.c_char_p, _fp, C.c_int32, C.c_char_p, C.c_int]),
    "globe_set_vc": (C.c_int, [_vp, _dp]),
    "globe_grm_apply": (C.c_int, [_vp, _dp, _dp, C.c_int]),
    "globe_grm_apply_dev": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "globe_vx": (C.c_int, [_vp, _dp, _dp, C.c_int]),
    "globe_vx_dev": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "globe_precond_apply": (C.c_int, [_vp, _dp, _dp, C.c_int]),
    "globe_genetic_diag": (C.c_int, [_vp, _dp]),
    "globe_pcg": (C.c_int, [_vp, _dp, _dp, C.c_int, C.POINTER(PcgOpts), C.POINTER(PcgInfo)]),
    "globe_pcg_dev": (C.c_int, [_vp, _vp, _vp, C.c_int, C.POINTER(PcgOpts), C.POINTER(PcgInfo)]),
    "globe_mme": (C.c_int, [_vp, C.POINTER(PcgOpts), _dp, _dp, _dp, _dp, C.POINTER(PcgInfo)]),
    "globe_aireml_grad": (C.c_int, [_vp, _dp, C.c_int, C.c_uint64, C.POINTER(PcgOpts), _dp, _dp, _dp, _dp,
                                    C.POINTER(PcgInfo)]),
    "globe_aireml_eval": (C.c_int, [_vp, _dp, C.c_int, C.c_uint64, C.POINTER(PcgOpts), _dp, _dp, _dp,
                                    C.POINTER(PcgInfo)]),
    "globe_aireml_ai": (C.c_int, [_vp, C.POINTER(PcgOpts), _dp, C.POINTER(PcgInfo)]),
    "globe_trust_region_step": (C.c_int, [_dp, _dp, _dp, C.c_double, _dp, C.POINTER(C.c_int)]),
    "globe_aireml_run": (C.c_int, [_vp, C.POINTER(AiremlOpts), C.c_char_p, C.POINTER(AiremlResult)]),
    "globe_read_records": (C.c_int, [C.c_char_p, _i64p, _i32p, _i32p, _i32p, _dp, _dp, C.c_char_p, C.c_int]),
    "globe_save_vector_f32": (C.c_int, [C.c_char_p, _dp, C.c_int32]),
    "globe_save_vector_f64": (C.c_int, [C.c_char_p, _dp, C.c_int32]),
    "globe_bed_dims": (C.c_int, [C.c_char_p, C.c_int32, _i64p, C.c_char_p, C.c_int]),
    "globe_read_bed": (C.c_int, [C.c_char_p, C.c_int32, C.c_int64, _u8p, C.c_char_p, C.c_int]),
    "globe_read_grm": (C.c_int, [C.c_char_p, C.c_int32, _fp, C.c_char_p, C.c_int]),
    "globe_set_precision": (C.c_int, [_vp, C.c_int]),
    "globe_set_model": (C.c_int, [_vp, C.c_int]),
    "globe_get_model": (C.c_int, [_vp]),
    "globe_trust_region_step_no_time": (C.c_int, [_dp, _dp, _dp, C.c_double, _dp, C.POINTER(C.c_int)]),
    "globe_read_records_no_time": (C.c_int, [C.c_char_p, _i64p, _i32p, _i32p, _i32p, _dp, _dp, C.c_char_p,
                                             C.c_int]),
    "globe_prof_enable": (C.c_int, [_vp, C.c_int]),
    "globe_prof_query": (C.c_int, [_vp, C.c_int, _i64p, _dp]),
    "globe_precond_apply_dev_noalloc": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp]),
    "globe_synth_bed_dev": (C.c_int, [_vp, _vp, C.c_int64, C.c_int32, C.c_int64, C.c_uint64, C.c_float, C.c_float,
                                      C.c_float]),
}

_lib = None


def lib():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libglobe_gb300.so not found at %s; run `python -c \"import __graft_entry__ as g; "
                           "g.build()\"` (or python globe_gb300/build.py) first" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class GlobeError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "GLOBE_ERR"), code, msg))
        self.code = code
