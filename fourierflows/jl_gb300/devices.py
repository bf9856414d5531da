"""Devices and device arrays (src/FourierFlows.jl:95-101, src/utils.jl:79-94,329-340).

``GPU()`` arrays are CUDA tensors laid out column-major like Julia's: a tensor of shape
(nkr, ny) has strides (1, nkr), so index [i, j] here is Julia's [i+1, j+1] and the
memory handed to the C ABI is exactly the reference's.  Torch only supplies the device
buffers and the stream; every computation on them goes through libfourierflows_gb300.

``CPU()`` grids hold the host-side set-up arrays (numpy) only: this library implements
the reference's GPU path, and its transforms and steppers refuse CPU arrays.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


class Device:
    pass


class CPU(Device):
    def __eq__(self, other):
        return isinstance(other, CPU)

    def __hash__(self):
        return hash("CPU")

    def __repr__(self):
        return "CPU"


class GPU(Device):
    def __eq__(self, other):
        return isinstance(other, GPU)

    def __hash__(self):
        return hash("GPU")

    def __repr__(self):
        return "GPU"


def _torch():
    import torch
    return torch


_NP2TORCH = None


def torch_dtype(T):
    global _NP2TORCH
    torch = _torch()
    if _NP2TORCH is None:
        _NP2TORCH = {np.dtype(np.float64): torch.float64, np.dtype(np.float32): torch.float32,
                     np.dtype(np.complex128): torch.complex128, np.dtype(np.complex64): torch.complex64}
    return _NP2TORCH[np.dtype(T)]


def np_dtype(tdtype):
    torch = _torch()
    return {torch.float64: np.dtype(np.float64), torch.float32: np.dtype(np.float32),
            torch.complex128: np.dtype(np.complex128), torch.complex64: np.dtype(np.complex64)}[tdtype]


def cxtype(T):
    """cxtype(T): Complex{T} for real T, T for complex (src/utils.jl:18-19)."""
    T = np.dtype(T)
    if T.kind == "c":
        return T.type
    return {np.dtype(np.float64): np.complex128, np.dtype(np.float32): np.complex64,
            np.dtype(np.float16): np.complex64}[T]


def fltype(T):
    """fltype(T): the real type of T (src/utils.jl:26-28); tuples use their first entry."""
    if isinstance(T, tuple):
        return fltype(T[0])
    T = np.dtype(T)
    if T.kind == "f":
        return T.type
    return {np.dtype(np.complex128): np.float64, np.dtype(np.complex64): np.float32}[T]


def fortran_empty(shape, dtype, device="cuda"):
    """Uninitialised column-major CUDA tensor of `shape`."""
    torch = _torch()
    shape = tuple(int(s) for s in shape)
    t = torch.empty(shape[::-1], dtype=dtype, device=device)
    return t.permute(*reversed(range(len(shape))))


def fortran_zeros(shape, dtype, device="cuda"):
    t = fortran_empty(shape, dtype, device)
    t.zero_()
    return t


def is_fortran(t) -> bool:
    """Column-major and dense (the layout the C ABI expects)."""
    expect, s = [], 1
    for n in t.shape:
        expect.append(s)
        s *= n
    return all(st == e for st, e, n in zip(t.stride(), expect, t.shape) if n > 1)


def as_fortran(t):
    """``t`` itself when dense column-major, else a column-major copy."""
    if is_fortran(t):
        return t
    out = fortran_empty(tuple(t.shape), t.dtype, t.device)
    out.copy_(t)
    return out


def zeros(dev, T, dims):
    """zeros(dev, T, dims) (src/utils.jl:79-80)."""
    dims = (dims,) if np.isscalar(dims) else tuple(dims)
    if isinstance(dev, GPU):
        return fortran_zeros(dims, torch_dtype(T))
    return np.zeros(dims, dtype=T, order="F")


def device_array(dev, T=None, dim=None):
    """device_array(dev): a converter to the device's array type (src/utils.jl:329-332)."""
    if isinstance(dev, GPU):
        def to_gpu(x, dtype=None):
            torch = _torch()
            if isinstance(x, torch.Tensor):
                a = x.detach().cpu().numpy()
            else:
                a = np.asarray(x)
            if dtype is not None:
                a = a.astype(dtype)
            elif T is not None:
                a = a.astype(T)
            t = fortran_empty(a.shape, torch_dtype(a.dtype))
            if a.ndim > 1 and a.flags.f_contiguous:
                # same memory order on both sides: a plain copy, no host transpose
                src = torch.from_numpy(a.T).permute(*reversed(range(a.ndim)))
            else:
                src = torch.from_numpy(np.ascontiguousarray(a))
            t.copy_(src)
            return t
        return to_gpu

    def to_cpu(x, dtype=None):
        a = to_numpy(x)
        if dtype is not None:
            a = a.astype(dtype)
        elif T is not None:
            a = a.astype(T)
        return np.asfortranarray(a)
    return to_cpu


def to_numpy(x):
    """Host copy of a device array (``Array(x)`` in Julia)."""
    try:
        import torch
        if isinstance(x, torch.Tensor):
            return x.detach().cpu().numpy()
    except ImportError:  # pragma: no cover
        pass
    return np.asarray(x)


def on_device(x) -> bool:
    try:
        import torch
        return isinstance(x, torch.Tensor) and x.is_cuda
    except ImportError:  # pragma: no cover
        return False


def ptr(t, what="array"):
    """Raw device pointer of a column-major CUDA tensor, checked for the C ABI."""
    if not on_device(t):
        raise TypeError(f"{what}: expected a CUDA (GPU()) array, got {type(t).__name__}; "
                        "this library implements the GPU path only")
    if not is_fortran(t):
        raise ValueError(f"{what}: array must be dense column-major (shape {tuple(t.shape)}, "
                         f"strides {tuple(t.stride())})")
    return C.c_void_p(t.data_ptr())


def stream_handle(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def prec_of(dtype) -> int:
    torch = _torch()
    if dtype in (torch.float64, torch.complex128):
        return _lib.FF_F64
    if dtype in (torch.float32, torch.complex64):
        return _lib.FF_F32
    raise TypeError(f"unsupported dtype {dtype}")


def real_dtype_of(dtype):
    torch = _torch()
    return {torch.complex128: torch.float64, torch.complex64: torch.float32, torch.float64: torch.float64,
            torch.float32: torch.float32}[dtype]
