"""FFT plans: ``plan_flows_rfft`` / ``plan_flows_fft`` and ``mul_`` / ``ldiv_``.

Mirrors src/domains.jl:1-5 (the grids' ``rfftplan`` and ``fftplan``) and the
``LinearAlgebra.mul!(out, plan, in)`` / ``ldiv!(out, plan, in)`` calls every caller in the
reference uses (src/diffusion.jl:137-171).  A plan transforms over all of its planned
dimensions; arrays with extra trailing dimensions are transformed as a batch.
Julia's in-place ``!`` functions are named with a trailing underscore here.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .devices import as_fortran, fortran_empty, on_device, prec_of, ptr, real_dtype_of, stream_handle


class _Plan:
    real = True

    def __init__(self, shape, T=np.float64, batch=1):
        self.shape = tuple(int(s) for s in shape)
        self.ndim = len(self.shape)
        self.T = np.dtype(T).type
        self.prec = _lib.FF_F64 if np.dtype(T) in (np.float64, np.complex128) else _lib.FF_F32
        self.batch = int(batch)
        self._h = C.c_void_p()
        n = _lib.i64_array(list(self.shape) + [1] * (3 - self.ndim))
        fn = "ff_plan_create" if self.real else "ff_cplan_create"
        _lib.call(fn, self.ndim, n, self.prec, self.batch, C.byref(self._h))
        self._batched = {}

    def _handle_for(self, batch):
        if batch == self.batch:
            return self._h
        if batch not in self._batched:
            self._batched[batch] = type(self)(self.shape, self.T, batch)
        return self._batched[batch]._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().ff_plan_destroy(h)
            except Exception:  # interpreter shutdown
                pass
            self._h = None

    @property
    def region(self):
        return tuple(range(1, self.ndim + 1))

    def _batch_of(self, arr, first):
        spatial = (first,) + self.shape[1:]
        got = tuple(arr.shape)
        if got[:self.ndim] != spatial:
            raise ValueError(f"array of size {got} does not match the plan's {spatial}")
        b = 1
        for s in got[self.ndim:]:
            b *= s
        return b


class RFFTPlan(_Plan):
    """Real-to-complex plan over the planned dimensions (``plan_rfft``)."""
    real = True

    @property
    def nkr(self):
        return self.shape[0] // 2 + 1

    def __repr__(self):
        return f"RFFTPlan{{{np.dtype(self.T).name}, dims {self.shape}}}"


class FFTPlan(_Plan):
    """Complex-to-complex plan over the planned dimensions (``plan_fft``)."""
    real = False

    def __repr__(self):
        return f"FFTPlan{{{np.dtype(self.T).name}, dims {self.shape}}}"


def _check_dtypes(plan, arr, want_complex, what):
    torch = __import__("torch")
    rd = real_dtype_of(arr.dtype)
    if prec_of(arr.dtype) != plan.prec:
        raise TypeError(f"{what}: precision {arr.dtype} does not match the plan")
    if want_complex != arr.dtype.is_complex:
        raise TypeError(f"{what}: expected a {'complex' if want_complex else 'real'} array, got {arr.dtype}")
    return rd


def mul_(out, plan, inp, stream=None):
    """mul!(out, plan, in): forward (unnormalised) transform."""
    if plan is None:
        raise NotImplementedError("CPU() grids carry no transforms: this library implements the GPU path")
    if on_device(inp):
        inp = as_fortran(inp)
    if isinstance(plan, RFFTPlan):
        _check_dtypes(plan, inp, False, "mul_ input")
        _check_dtypes(plan, out, True, "mul_ output")
        b = plan._batch_of(inp, plan.shape[0])
        if plan._batch_of(out, plan.nkr) != b:
            raise ValueError("mul_: input and output batch sizes differ")
        _lib.call("ff_rfft", plan._handle_for(b), ptr(inp, "mul_ input"), ptr(out, "mul_ output"),
                  stream_handle(stream))
    else:
        _check_dtypes(plan, inp, True, "mul_ input")
        _check_dtypes(plan, out, True, "mul_ output")
        b = plan._batch_of(inp, plan.shape[0])
        if plan._batch_of(out, plan.shape[0]) != b:
            raise ValueError("mul_: input and output batch sizes differ")
        _lib.call("ff_fft", plan._handle_for(b), ptr(inp, "mul_ input"), ptr(out, "mul_ output"),
                  stream_handle(stream))
    return out


def ldiv_(out, plan, inp, stream=None):
    """ldiv!(out, plan, in): normalised inverse transform; ``inp`` is left unchanged."""
    if plan is None:
        raise NotImplementedError("CPU() grids carry no transforms: this library implements the GPU path")
    if on_device(inp):
        inp = as_fortran(inp)
    if isinstance(plan, RFFTPlan):
        _check_dtypes(plan, inp, True, "ldiv_ input")
        _check_dtypes(plan, out, False, "ldiv_ output")
        b = plan._batch_of(inp, plan.nkr)
        if plan._batch_of(out, plan.shape[0]) != b:
            raise ValueError("ldiv_: input and output batch sizes differ")
        _lib.call("ff_irfft", plan._handle_for(b), ptr(inp, "ldiv_ input"), ptr(out, "ldiv_ output"),
                  stream_handle(stream))
    else:
        _check_dtypes(plan, inp, True, "ldiv_ input")
        _check_dtypes(plan, out, True, "ldiv_ output")
        b = plan._batch_of(inp, plan.shape[0])
        _lib.call("ff_ifft", plan._handle_for(b), ptr(inp, "ldiv_ input"), ptr(out, "ldiv_ output"),
                  stream_handle(stream))
    return out


_PLAN_CACHE = {}


def _cached(kind, shape, T):
    key = (kind, tuple(shape), np.dtype(T).name)
    p = _PLAN_CACHE.get(key)
    if p is None:
        p = (RFFTPlan if kind == "r" else FFTPlan)(shape, T)
        _PLAN_CACHE[key] = p
    return p


def _rt(dtype):
    import torch
    return np.float64 if dtype in (torch.float64, torch.complex128) else np.float32


def plan_flows_rfft(a, dims=None):
    """plan_flows_rfft(a): a real plan for arrays shaped like ``a`` (src/domains.jl:3,5)."""
    shape = tuple(a.shape) if dims is None else tuple(a.shape[d - 1] for d in dims)
    return RFFTPlan(shape, _rt(a.dtype))


def plan_flows_fft(a, dims=None):
    """plan_flows_fft(a): a complex plan for arrays shaped like ``a`` (src/domains.jl:2,4)."""
    shape = tuple(a.shape) if dims is None else tuple(a.shape[d - 1] for d in dims)
    return FFTPlan(shape, _rt(a.dtype))


def rfft(a):
    """Allocating rfft over all dimensions (FFTW.rfft re-exported by the reference)."""
    import torch
    cdt = torch.complex128 if a.dtype == torch.float64 else torch.complex64
    out = fortran_empty((a.shape[0] // 2 + 1,) + tuple(a.shape[1:]), cdt)
    return mul_(out, _cached("r", a.shape, _rt(a.dtype)), a)


def irfft(ah, nx):
    import torch
    rdt = torch.float64 if ah.dtype == torch.complex128 else torch.float32
    shape = (int(nx),) + tuple(ah.shape[1:])
    out = fortran_empty(shape, rdt)
    return ldiv_(out, _cached("r", shape, _rt(ah.dtype)), ah)


def fft(a):
    import torch
    if not a.dtype.is_complex:
        a = a.to(torch.complex128 if a.dtype == torch.float64 else torch.complex64)
    out = fortran_empty(tuple(a.shape), a.dtype)
    return mul_(out, _cached("c", a.shape, _rt(a.dtype)), a)


def ifft(ah):
    out = fortran_empty(tuple(ah.shape), ah.dtype)
    return ldiv_(out, _cached("c", ah.shape, _rt(ah.dtype)), ah)
