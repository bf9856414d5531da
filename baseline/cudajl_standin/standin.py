"""Build and ctypes binding of libff_cudajl_standin.so (see ff_unfused.cu).

The stand-in restates the reference's unfused GPU op sequence for the 2D vorticity ETDRK4
step (src/timesteppers.jl:501-547, src/domains.jl:5,457-458): one kernel per broadcast and
cuFFT plans for the transforms.  It is a comparator for bench.py and the tests; the
library in fourierflows/jl_gb300 never links cuFFT.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ff_unfused.cu")
LIB = os.path.join(HERE, "libff_cudajl_standin.so")
FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
         "-shared"]


def build(force=False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc, SRC, "-o", tmp] + FLAGS + ["-lcufft", "-lcudart"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on ff_unfused.cu:\n{r.stdout}{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.ffu_last_error.restype = C.c_char_p
        L.ffu_create.argtypes = [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64,
                                 C.c_int64, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        L.ffu_step.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
        L.ffu_destroy.argtypes = [C.c_void_p]
        L.ffu_launches_per_step.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError(f"cudajl stand-in: {lib().ffu_last_error().decode()}")


class UnfusedETDRK4:
    """The unfused FP64 ETDRK4 vorticity step on a library Problem's grid and coefficients.

    ``prob`` is a ``Vorticity.Problem`` in FP64 with the ETDRK4 stepper: its wavenumbers and
    ETDRK4 coefficient arrays (device, FP64) are read in place, so it must outlive this
    object.  ``step(sol, n)`` advances a device state of shape (nkr, ny)."""

    def __init__(self, prob):
        g, ts = prob.grid, prob.timestepper
        self._keep = (prob,)
        k0 = g.kralias.start if g.kralias is not None else g.nkr
        la, lb = (g.lalias.start, g.lalias.stop) if g.lalias is not None else (0, 0)
        coefs = [ts.expLdt, ts.exp_half_Ldt, ts.zeta, ts.alpha, ts.beta, ts.Gamma]
        for c in coefs + [g.kr, g.l, g.invKrsq]:
            if str(c.dtype) != "torch.float64" or not c.is_cuda:
                raise ValueError("the stand-in needs FP64 device arrays")
        arr = (C.c_void_p * 6)(*[c.data_ptr() for c in coefs])
        self._h = C.c_void_p()
        _check(lib().ffu_create(g.nx, g.ny, g.kr.data_ptr(), g.l.data_ptr(), g.invKrsq.data_ptr(), k0, la, lb,
                                arr, C.byref(self._h)))

    def step(self, sol, nsteps=1, stream=None):
        import torch
        s = stream if stream is not None else torch.cuda.current_stream()
        _check(lib().ffu_step(self._h, C.c_void_p(sol.data_ptr()), int(nsteps), C.c_void_p(s.cuda_stream)))

    @property
    def launches_per_step(self):
        return int(lib().ffu_launches_per_step(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().ffu_destroy(h)
            except Exception:
                pass
            self._h = None
