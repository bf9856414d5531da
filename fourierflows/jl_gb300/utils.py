"""Utilities (src/utils.jl): Parseval sums, Jacobians, array helpers."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .devices import (CPU, GPU, cxtype, device_array, fltype, np_dtype, on_device, prec_of, ptr, stream_handle,
                      to_numpy, zeros)
from .plans import fft, ifft, irfft, rfft


def innereltype(x):
    """The innermost element type of a (nested) collection (src/utils.jl:7-11)."""
    if isinstance(x, (list, tuple)):
        return innereltype(x[0])
    return getattr(x, "dtype", type(x))


def superzeros(T, dims=None):
    """superzeros(T, dims) / superzeros(dims) (src/utils.jl:36-40)."""
    if dims is None:
        T, dims = np.float64, T
    if isinstance(dims, tuple) and dims and isinstance(dims[0], tuple):
        if isinstance(T, tuple):
            return [np.zeros(d, dtype=t) for t, d in zip(T, dims)]
        return [np.zeros(d, dtype=T) for d in dims]
    return np.zeros(dims, dtype=T)


def _grid_norm(grid):
    if grid.ndim == 2:
        return float(grid.Lx) * float(grid.Ly) / (grid.nx ** 2 * grid.ny ** 2)
    if grid.ndim == 1:
        return float(grid.Lx) / grid.nx ** 2
    raise NotImplementedError("parsevalsum2 is defined for OneDGrid and TwoDGrid (src/utils.jl:113-139)")


def _parseval(name, uh, grid, stream=None):
    if not on_device(uh):
        raise TypeError(f"{name}: expected a GPU() array")
    n0 = uh.shape[0]
    rest = uh.numel() // n0
    rfft_form = 1 if n0 == grid.nkr else 0
    out = C.c_double()
    if uh.dtype.is_complex:
        arr = uh
    else:
        import torch
        arr = uh.to(torch.complex128 if uh.dtype == torch.float64 else torch.complex64)
    _lib.call(name, prec_of(arr.dtype), ptr(arr, name), n0, rest, rfft_form, _grid_norm(grid), C.byref(out),
              stream_handle(stream))
    return out.value


def parsevalsum2(uh, grid, stream=None):
    """sum |uh|^2 over the modes, normalised to the domain integral of u^2, counting the
    0 < k < nx/2 modes of a real transform twice (src/utils.jl:113-139)."""
    return _parseval("ff_parsevalsum2", uh, grid, stream)


def parsevalsum(uh, grid, stream=None):
    """Real part of the normalised sum of uh (src/utils.jl:157-183)."""
    return _parseval("ff_parsevalsum", uh, grid, stream)


def _mul_ik(out, inp, k, stream=None):
    """out = i k inp with k broadcast along dimension 0 (ff_mul_ik)."""
    n0 = inp.shape[0]
    _lib.call("ff_mul_ik", prec_of(inp.dtype), n0, inp.numel() // n0, ptr(out, "out"), ptr(inp, "in"),
              ptr(k, "k"), stream_handle(stream))
    return out


def jacobianh(a, b, grid):
    """Fourier transform of J(a, b) = a_x b_y - a_y b_x (src/utils.jl:190-205)."""
    if not a.dtype.is_complex:
        bh = rfft(b)
        bx = irfft(1j * grid.kr * bh, grid.nx)
        by = irfft(1j * grid.l * bh, grid.nx)
        return 1j * grid.kr * rfft(a * by) - 1j * grid.l * rfft(a * bx)
    bh = fft(b)
    bx = ifft(1j * grid.k * bh)
    by = ifft(1j * grid.l * bh)
    return 1j * grid.k * fft(a * by) - 1j * grid.l * fft(a * bx)


def jacobian(a, b, grid):
    """J(a, b) on the grid (src/utils.jl:212-218)."""
    if not a.dtype.is_complex:
        return irfft(jacobianh(a, b, grid), grid.nx)
    return ifft(jacobianh(a, b, grid))


def radialspectrum(fh, grid, n=None, m=None, refinement=2, stream=None):
    """(rho, fhr): fh on a TwoDGrid interpolated onto a polar grid and integrated over
    angle, fhr = [2] rho int fh(rho, theta) dtheta (src/utils.jl:239-283), one native
    binned reduction (``ff_radialspectrum``).  fh is the conjugate-symmetric (nkr, nl) or
    full (nk, nl) form, real or complex, on the GPU; rho is returned on the host (the
    reference's range), fhr on the device with fh's element type."""
    from .domains import TwoDGrid
    if not isinstance(grid, TwoDGrid):
        raise TypeError("radialspectrum is defined for a TwoDGrid (src/utils.jl:239)")
    if not on_device(fh):
        raise ValueError("radialspectrum: fh must be a GPU array")
    n = refinement * max(grid.nk, grid.nl) if n is None else int(n)
    m = refinement * max(grid.nk, grid.nl) if m is None else int(m)
    if fh.shape[0] == grid.nkr:
        if m % 2:
            raise ValueError("radialspectrum: m must be even for the conjugate-symmetric form")
        m //= 2
    elif fh.shape[0] != grid.nk:
        raise ValueError(f"radialspectrum: fh of size {tuple(fh.shape)} on a {grid.nx} x {grid.ny} grid")
    if tuple(fh.shape[1:]) != (grid.nl,):
        raise ValueError(f"radialspectrum: fh of size {tuple(fh.shape)} on a {grid.nx} x {grid.ny} grid")
    out = zeros(grid.device, np_dtype(fh.dtype), (n,))
    _lib.call("ff_radialspectrum", prec_of(fh.dtype), 1 if fh.dtype.is_complex else 0, ptr(fh, "fh"), fh.shape[0],
              grid.nk, grid.nl, float(grid.Lx), float(grid.Ly), n, m, ptr(out, "out"), stream_handle(stream))
    rhomax = min((grid.nk / 2 - 1) * 2 * np.pi / float(grid.Lx), (grid.nl / 2 - 1) * 2 * np.pi / float(grid.Ly))
    return np.linspace(0.0, rhomax, n), out


def on_grid(func, grid):
    """func evaluated at the grid points, as a device array (src/utils.jl:291-320)."""
    if grid.ndim == 1:
        f = func(grid.x.astype(np.float64))
    elif grid.ndim == 2:
        f = func(grid.x.reshape(-1, 1).astype(np.float64), grid.y.reshape(1, -1).astype(np.float64))
    else:
        f = func(grid.x.reshape(-1, 1, 1).astype(np.float64), grid.y.reshape(1, -1, 1).astype(np.float64),
                 grid.z.reshape(1, 1, -1).astype(np.float64))
    f = np.broadcast_to(np.asarray(f, dtype=grid.T), grid.physical_shape)
    return device_array(grid.device)(np.array(f))
