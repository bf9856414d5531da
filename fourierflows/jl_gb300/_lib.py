"""ctypes binding of libfourierflows_gb300.so -- the same C ABI a Julia ``ccall`` binds.

The library is loaded from this package directory.  There is no fallback: when the
shared object is missing or a symbol is absent, importing a compute entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

LIBNAME = "libfourierflows_gb300.so"
LIBPATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), LIBNAME)

FF_OK, FF_ERR_ARG, FF_ERR_CUDA, FF_ERR_UNSUPPORTED, FF_ERR_ALLOC, FF_ERR_TIMEOUT = range(6)
FF_VORT_CALC_SLOTS = 16  # include/fourierflows_gb300.h
FF_F64, FF_F32 = 0, 1
FF_COEF_NONE, FF_COEF_REAL, FF_COEF_COMPLEX, FF_COEF_SCALAR = range(4)


class FFError(RuntimeError):
    """A native call failed; ``status`` is the FF_ERR_* code."""

    def __init__(self, status, msg):
        super().__init__(f"[ff status {status}] {msg}")
        self.status = status


class FFArgumentError(FFError, ValueError):
    """Bad argument (the reference raises ArgumentError / DomainError for these)."""


class FFUnsupportedError(FFError, NotImplementedError):
    pass


class ff_coef(C.Structure):
    _fields_ = [("ptr", C.c_void_p), ("kind", C.c_int32), ("pad_", C.c_int32), ("re", C.c_double),
                ("im", C.c_double)]


vp, i32, i64, f64 = C.c_void_p, C.c_int, C.c_int64, C.c_double
i64p = C.POINTER(C.c_int64)

# name -> argtypes; every function returns int
SIGNATURES = {
    "ff_version": [],
    "ff_last_error": [C.c_char_p, C.c_size_t],
    "ff_plan_create": [i32, i64p, i32, i64, C.POINTER(vp)],
    "ff_cplan_create": [i32, i64p, i32, i64, C.POINTER(vp)],
    "ff_plan_destroy": [vp],
    "ff_rfft": [vp, vp, vp, vp],
    "ff_irfft": [vp, vp, vp, vp],
    "ff_fft": [vp, vp, vp, vp],
    "ff_ifft": [vp, vp, vp, vp],
    "ff_dealias": [i32, vp, i64p, i64p, i64p, vp],
    "ff_euler_update": [i32, i64, vp, vp, ff_coef, f64, vp, vp],
    "ff_rk4_substep": [i32, i64, vp, ff_coef, vp, vp, vp, f64, vp],
    "ff_rk4_update": [i32, i64, vp, vp, ff_coef, vp, vp, vp, vp, f64, vp, vp],
    "ff_lsrk54_stage": [i32, i64, vp, vp, vp, ff_coef, f64, f64, f64, i32, vp, vp],
    "ff_etdrk4_substep12": [i32, i64, vp, ff_coef, vp, ff_coef, vp, vp],
    "ff_etdrk4_substep3": [i32, i64, vp, ff_coef, vp, ff_coef, vp, vp, vp],
    "ff_etdrk4_update": [i32, i64, vp, ff_coef, ff_coef, ff_coef, ff_coef, vp, vp, vp, vp, vp, vp],
    "ff_ab3_update": [i32, i64, vp, vp, vp, vp, ff_coef, f64, i32, vp, vp],
    "ff_filter_mul": [i32, i64, vp, vp, vp],
    "ff_linear_step": [i32, i32, i64, vp, ff_coef, f64, vp, i64, vp],
    "ff_mul_ik": [i32, i64, i64, vp, vp, vp, vp],
    "ff_real_mul": [i32, i64, i64, vp, vp, vp],
    "ff_parsevalsum2": [i32, vp, i64, i64, i32, f64, C.POINTER(f64), vp],
    "ff_parsevalsum": [i32, vp, i64, i64, i32, f64, C.POINTER(f64), vp],
    "ff_radialspectrum": [i32, i32, vp, i64, i64, i64, f64, f64, i64, i64, vp, vp],
    "ff_parsevalsum2_weighted": [i32, vp, vp, i64, i64, i32, f64, C.POINTER(f64), vp, vp],
    "ff_vort_velocities": [i32, i64, i64, vp, vp, vp, vp, vp, vp, vp],
    "ff_vort_create": [i32, i32, i32, f64, i64, vp, C.POINTER(vp)],
    "ff_vort_destroy": [vp],
    "ff_vort_step": [vp, i64, vp],
    "ff_vort_calcN": [vp, i64, vp, vp, vp],
    "ff_vort_config": [vp, C.POINTER(C.c_int32)],
    "ff_vort_set_config": [vp, i32, i32, i32, i32],
    "ff_vort_set_split": [vp, i32],
    "ff_vort_calcN_bind": [vp, i32, i64, vp, vp],
    "ff_vort_calcN_slot": [vp, i32, vp],
    "ff_vort_get_split": [vp, C.POINTER(C.c_int32)],
    "ff_vort_autotune": [vp, i32, vp, C.POINTER(f64)],
    "ff_vort_profile": [vp, i32, vp, C.POINTER(f64)],
    "ff_etdrk4_coefficients": [i32, i64, vp, f64, i32, f64, vp, vp, vp, vp, vp],
    "ff_fp64_peak": [C.POINTER(f64), vp],
    "ff_parsevalsum2_noalloc": [i32, vp, i64, i64, i32, f64, vp, vp],
    "ff_vadj_create": [i32, i64, i64, i64, i64, i64, vp, vp, vp, C.POINTER(vp)],
    "ff_vadj_destroy": [vp],
    "ff_vadj_apply": [vp, vp, vp, vp, vp],
    "ff_vort_adj_nu_terms": [vp, vp, f64, vp, vp],
}


class ff_adj_nu(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in
                ("lam", "lam_a", "lam_b", "lam_c", "s", "a", "n1", "n2", "n3", "n4", "dE", "dE2", "dZ", "dA", "dB",
                 "dG")]

FF_STEP_ETDRK4, FF_STEP_RK4, FF_STEP_LSRK54 = 0, 1, 2


class ff_vort_problem(C.Structure):
    _fields_ = [("nx", C.c_int64), ("ny", C.c_int64), ("nkd", C.c_int64), ("la", C.c_int64), ("lb", C.c_int64),
                ("kr", C.c_void_p), ("l", C.c_void_p), ("invKrsq", C.c_void_p), ("sol", C.c_void_p),
                ("buf", C.c_void_p * 5), ("coef", C.c_void_p * 6), ("filter", C.c_void_p),
                ("lsrk_A", C.c_double * 5), ("lsrk_B", C.c_double * 5)]

_LIB = None


def header_symbols():
    """Entry points declared in include/fourierflows_gb300.h (parsed, for the ABI test)."""
    import re
    hdr = os.path.normpath(os.path.join(os.path.dirname(LIBPATH), "..", "..", "include",
                                        "fourierflows_gb300.h"))
    text = open(hdr).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*int\s+(ff_\w+)\s*\(", text, flags=re.M)))


def lib():
    """Load the library (once).  Raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError(f"{LIBNAME} is not built (expected at {LIBPATH}); run "
                               "`python -m fourierflows.jl_gb300.build` or __graft_entry__.build()")
        h = C.CDLL(LIBPATH)
        for name, args in SIGNATURES.items():
            fn = getattr(h, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _LIB = h
    return _LIB


def last_error() -> str:
    buf = C.create_string_buffer(512)
    lib().ff_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(status: int) -> None:
    if status == FF_OK:
        return
    msg = last_error()
    if status == FF_ERR_ARG:
        raise FFArgumentError(status, msg)
    if status == FF_ERR_UNSUPPORTED:
        raise FFUnsupportedError(status, msg)
    raise FFError(status, msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))


def i64_array(values):
    vals = list(values)
    return (C.c_int64 * len(vals))(*vals)
