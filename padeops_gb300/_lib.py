"""ctypes binding of ``libpadeops_gb300.so`` (the C ABI in include/padeops_gb300.h).

The compute path is the native library; there is no Python or CPU fallback.  Loading
fails loudly when the library is missing: run ``padeops_gb300.build.build()`` (or
``__graft_entry__.build()``) first.
"""
import ctypes
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libpadeops_gb300.so")
HEADER_PATH = os.path.join(os.path.dirname(_HERE), "include", "padeops_gb300.h")

PADE_OK = 0
PADE_EREF_NONPERIODIC_N = 2
PADE_EREF_PERIODIC_N = 3
PADE_EREF_FILTER_N = 7
PADE_EREF_STAGG_N = 21
PADE_EREF_BC = 324
PADE_EINVAL = 1001
PADE_ENOMEM = 1002
PADE_ECUDA = 1003
PADE_ENOTSUP = 1004
PADE_ETIMEOUT = 1005
PADE_ERANGE = 1006
PADE_ESCRATCH = 1007
NOALLOC_SCRATCH_BYTES = 32 << 20

PATH_DF = 0
PATH_NATIVE = 1
PATH_FP32 = 2

FAMILY = {"cd06": 0, "cd10": 1, "cf90": 2, "gaussian": 3, "cd06stagg": 4, "fd02": 5}
STAGG_OPS = ("ddz_E2C", "ddz_C2E", "ddz_C2C", "ddz_E2E", "d2dz2_C2C", "d2dz2_E2E", "InterpZ_E2C", "InterpZ_C2E")
# Pade6stagg operations in pade_pade6stagg_apply's numbering
PADE6_OPS = ("ddz_C2E", "ddz_E2C", "interpz_C2E", "interpz_E2C", "d2dz2_C2C", "d2dz2_E2E")

_lib = None

class LesParams(ctypes.Structure):
    """pade_les_params (include/padeops_gb300.h)."""

    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("Lx", ctypes.c_double), ("Ly", ctypes.c_double), ("Lz", ctypes.c_double),
                ("Re", ctypes.c_double), ("isInviscid", ctypes.c_int), ("CFL", ctypes.c_double),
                ("dt", ctypes.c_double), ("useSGS", ctypes.c_int), ("dynamic", ctypes.c_int),
                ("Csgs", ctypes.c_double), ("deltaRatio", ctypes.c_double), ("DynProcFreq", ctypes.c_int),
                ("dealiasFact", ctypes.c_double), ("t_DivergenceCheck", ctypes.c_int),
                ("learnedSGS", ctypes.c_int), ("JudgeFreq", ctypes.c_int), ("learnedPlaneAvg", ctypes.c_int),
                ("SGSModelID", ctypes.c_int), ("JudgeTol", ctypes.c_double)]


MLP_NPARAM = 4929
FFT_DF = 0
FFT_FP64 = 1

LES_FIELDS = {"uhat": 0, "vhat": 1, "what": 2, "u": 3, "v": 4, "wC": 5, "w": 6, "uE": 7, "vE": 8,
              "nu_sgs_C": 30, "nu_sgs_E": 31}

# void (*)(double* kd, int n): modified-wavenumber callback of pade_poisson3d_init
MODK_FN = ctypes.CFUNCTYPE(None, ctypes.POINTER(ctypes.c_double), ctypes.c_int)


class PadeError(RuntimeError):
    """A non-zero status from the library (the reference would GracefulExit here)."""

    def __init__(self, code, where=""):
        self.code = code
        msg = strerror(code) if _lib is not None else str(code)
        super().__init__(f"{where}: status {code} ({msg})" if where else f"status {code} ({msg})")


def exported_symbols():
    """Names of the functions declared in include/padeops_gb300.h."""
    txt = open(HEADER_PATH).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\bint\s+(pade_\w+)\s*\(", txt)) | set(re.findall(r"char\*\s+(pade_\w+)\s*\(", txt)))


def lib():
    """Load the library and declare argument types (once)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} not built; run padeops_gb300.build.build()")
    L = ctypes.CDLL(LIB_PATH)
    vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    pop = ctypes.POINTER(ctypes.c_void_p)
    pi = ctypes.POINTER(ctypes.c_int)
    dp = ctypes.POINTER(ctypes.c_double)
    fp = ctypes.POINTER(ctypes.c_float)
    sig = {
        "pade_cd06_init": [pop, i, d, i, i, i],
        "pade_cd10_init": [pop, i, d, i, i, i],
        "pade_cf90_init": [pop, i, i],
        "pade_gaussian_init": [pop, i, i],
        "pade_cd06stagg_init_periodic": [pop, i, d],
        "pade_cd06stagg_init_nonperiodic": [pop, i, d, i, i, i, i],
        "pade_destroy": [vp],
        "pade_set_path": [vp, i],
        "pade_apply": [vp, i, i, i, vp, vp, i, i, i, i, i, vp],
        "pade_apply_noalloc": [vp, i, i, i, vp, vp, i, i, i, i, vp],
        "pade_get_status": [vp, pi],
        "pade_get_lengths": [vp, i, pi, pi],
        "pade_plan_check": [i, dp, i, i, i, dp, dp, i],
        "pade_plan_dense": [i, dp, i, i, i, dp, pi, pi],
    }
    for nm in ("dd1", "dd2", "dd3", "d2d1", "d2d2", "d2d3"):
        sig[f"pade_cd06_{nm}"] = [vp, vp, vp, i, i, vp]
        sig[f"pade_cd10_{nm}"] = [vp, vp, vp, i, i, i, i, vp]
    for fam in ("cf90", "gaussian"):
        for nm in ("filter1", "filter2", "filter3", "filter3_cmplx"):
            sig[f"pade_{fam}_{nm}"] = [vp, vp, vp, i, i, i, i, vp]
    for nm in STAGG_OPS:
        sig[f"pade_cd06stagg_{nm}"] = [vp, vp, vp, i, i, vp]
        sig[f"pade_cd06stagg_{nm}_cmplx"] = [vp, vp, vp, i, i, vp]
    sig.update({
        "pade_pade6stagg_init": [pop, i, d, i, i],
        "pade_pade6stagg_destroy": [vp],
        "pade_pade6stagg_apply": [vp, i, i, vp, vp, i, i, i, i, vp],
        "pade_pade6stagg_getModifiedWavenumbers": [vp, dp, dp, i],
        "pade_pade6stagg_getApproxPoincareConstant": [vp, dp],
    })
    for nm in PADE6_OPS:
        sig[f"pade_pade6stagg_{nm}"] = [vp, vp, vp, i, i, i, i, vp]
        sig[f"pade_pade6stagg_{nm}_cmplx"] = [vp, vp, vp, i, i, i, i, vp]
    sig.update({
        "pade_wavenumbers": [i, d, dp],
        "pade_modified_wavenumbers_cd06stagg": [dp, i, d, dp],
        "pade_spectral_init": [pop, i, i, i, d, d, i],
        "pade_spectral_destroy": [vp],
        "pade_spectral_get_wavenumbers": [vp, dp, dp],
        "pade_spectral_fft": [vp, vp, vp, vp],
        "pade_spectral_ifft": [vp, vp, vp, i, vp],
        "pade_spectral_ifft_ik": [vp, vp, vp, i, vp],
        "pade_spectral_ifft_and_ddx": [vp, vp, vp, vp, vp],
        "pade_spectral_fft_two": [vp, vp, vp, vp, vp, vp],
        "pade_spectral_ifft_two": [vp, vp, i, vp, i, vp, vp, vp],
        "pade_spectral_ifft_testfilter": [vp, vp, vp, d, vp],
        "pade_poisson_periodic_init": [pop, vp, d, d, d],
        "pade_poisson_wall_init": [pop, vp, d, d, d, d, i],
        "pade_poisson_get_pressure": [vp, vp, vp, vp, vp, vp],
        "pade_poisson_get_pressure_and_update_rhs": [vp, vp, vp, vp, vp, vp],
        "pade_poisson_destroy": [vp],
        "pade_poisson_get_modified_k3": [vp, dp],
        "pade_poisson_projection": [vp, vp, vp, vp, vp],
        "pade_poisson_divergence_check": [vp, vp, vp, vp, vp, i, dp, vp],
        "pade_poisson3d_init": [pop, i, i, i, d, d, d, i, MODK_FN, MODK_FN, MODK_FN],
        "pade_poisson3d_destroy": [vp],
        "pade_poisson3d_solve": [vp, vp, vp, vp],
        "pade_fft_c2c": [i, i, vp, vp, i, i, i, d, vp],
        "pade_fft_r2c_x": [vp, vp, i, i, i, vp],
        "pade_fft_c2r_x": [vp, vp, i, i, i, d, vp],
        "pade_transpose": [i, i, vp, vp, i, i, i, i, vp],
        "pade_fft_set_arith": [i],
        "pade_dense_apply": [vp, i, i, vp, vp, i, i, i, i, vp],
        "pade_dense_status": [pi],
        "pade_fft_get_arith": [],
        "pade_les_init": [pop, ctypes.POINTER(LesParams)],
        "pade_les_destroy": [vp],
        "pade_les_set_fields": [vp, vp, vp, vp, vp],
        "pade_les_step": [vp, i, vp],
        "pade_les_info": [vp, dp, dp, pi, dp],
        "pade_les_set_time": [vp, d, i],
        "pade_les_field": [vp, i, pop],
        "pade_les_scalar_sgs": [vp, vp, vp, vp, vp, vp, vp, vp, d, i, vp, vp],
        "pade_les_judge_info": [vp, dp, dp, ctypes.POINTER(ctypes.c_longlong)],
        "pade_mlp_set_range": [vp, fp, fp],
        "pade_les_set_mlp": [vp, vp],
        "pade_mlp_create": [pop],
        "pade_mlp_destroy": [vp],
        "pade_mlp_set_params": [vp, fp],
        "pade_mlp_get_params": [vp, fp],
        "pade_mlp_loss_grad": [vp, vp, vp, i, fp, fp, vp],
        "pade_mlp_train_step": [vp, vp, vp, i, ctypes.c_float, ctypes.c_float, fp, vp],
        "pade_mlp_features": [pop, ctypes.c_long, d, d, vp, vp],
        "pade_mlp_infer_nu": [vp, pop, ctypes.c_long, d, d, vp, vp, vp],
        "pade_mlp_status": [pi],
    })
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.pade_strerror.argtypes = [i]
    L.pade_strerror.restype = ctypes.c_char_p
    _lib = L
    return L


def strerror(code):
    return lib().pade_strerror(int(code)).decode()


def check(rc, where=""):
    if rc != PADE_OK:
        raise PadeError(rc, where)
    return rc
