"""Grids, alias ranges, ``dealias_`` and ``makefilter`` (src/domains.jl).

Wavenumbers, alias ranges and filters are one-time set-up computed on the host in FP64
and converted to the grid's float type, as the reference does (its grid constructors
build them with ``fftfreq`` on the CPU and copy them to the device, src/domains.jl:77-78,
193-195; ``makefilter`` on a CuArray goes through the host, :543-546).  Dealiasing,
transforms and everything per time step run in libfourierflows_gb300.

Alias ranges are Python ``range`` objects, 0-based: Julia's ``kalias = 342:683`` is
``range(341, 683)`` here.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

from . import _lib
from .devices import CPU, GPU, device_array, prec_of, ptr, stream_handle, to_numpy
from .plans import FFTPlan, RFFTPlan


class DomainError(ValueError):
    """Julia's DomainError (odd grid sizes)."""


def _fftfreq(n, fs):
    """AbstractFFTs.fftfreq(n, fs) values: (0..ceil(n/2)-1, -floor(n/2)..-1) * fs/n, in FP64."""
    mult = fs / n
    nn = (n + 1) // 2
    return np.array([(i if i < nn else i - n) * mult for i in range(n)], dtype=np.float64)


def _rfftfreq(n, fs):
    mult = fs / n
    return np.array([i * mult for i in range(n // 2 + 1)], dtype=np.float64)


def _range_points(x0, dx, n, T):
    """``range(T(x0), step=T(dx), length=n)``: each point the rounded exact sum."""
    T = np.dtype(T).type
    f0, fd = Fraction(float(T(x0))), Fraction(float(T(dx)))
    return np.array([T(float(f0 + i * fd)) for i in range(n)], dtype=T)


def getaliasedwavenumbers(nk, nkr, aliased_fraction):
    """src/domains.jl:408-421; 0-based ranges, ``(None, None)`` when nothing is aliased."""
    L = (1 - aliased_fraction) / 2
    R = (1 + aliased_fraction) / 2
    iL = math.floor(L * nk) + 1
    iR = math.ceil(R * nk)
    if not aliased_fraction < 1:
        raise ValueError("`aliased_fraction` must be less than 1")
    if aliased_fraction > 0:
        return range(iL - 1, iR), range(iL - 1, nkr)
    return None, None


class AbstractGrid:
    ndim = 0

    @property
    def T(self):
        return self._T

    def eltype(self):
        return self._T

    def _upload(self, a):
        return device_array(self.device)(np.asarray(a, dtype=self._T))

    def _make_plans(self, shape):
        if isinstance(self.device, GPU):
            self.fftplan = FFTPlan(shape, self._T)
            self.rfftplan = RFFTPlan(shape, self._T)
        else:
            self.fftplan = None
            self.rfftplan = None

    @property
    def spectral_shape(self):
        return (self.nkr,) + tuple(self._n[1:])

    @property
    def physical_shape(self):
        return tuple(self._n)

    def _alias_bounds(self, first_dim):
        """(lo, hi) per dimension for ff_dealias, 0-based; empty where nothing is aliased."""
        lo, hi = [0, 0, 0], [0, 0, 0]
        if self.kalias is None:
            return lo, hi
        kal = self.kralias if first_dim == self.nkr else self.kalias
        lo[0], hi[0] = kal.start, kal.stop
        if self.ndim >= 2:
            lo[1], hi[1] = self.lalias.start, self.lalias.stop
        if self.ndim == 3:
            lo[2], hi[2] = self.malias.start, self.malias.stop
        return lo, hi


def _show_float(v):
    r = repr(float(v))
    return r


class OneDGrid(AbstractGrid):
    """OneDGrid(dev; nx, Lx, x0=-Lx/2, T=Float64, aliased_fraction=1/3), src/domains.jl:61-101."""
    ndim = 1

    def __init__(self, dev=None, *, nx, Lx, x0=None, nthreads=None, effort=None, T=np.float64,
                 aliased_fraction=1 / 3):
        dev = dev if dev is not None else CPU()
        if nx % 2 != 0:
            raise DomainError("nx must be even")
        T = np.dtype(T).type
        self._T, self.device = T, dev
        self.nx, self.nk, self.nkr = int(nx), int(nx), int(nx) // 2 + 1
        self._n = (self.nx,)
        self.Lx = T(Lx)
        self.dx = T(Lx / nx)
        x0 = -Lx / 2 if x0 is None else x0
        self.x = _range_points(x0, Lx / nx, nx, T)
        k = _fftfreq(nx, 2 * math.pi / Lx * nx).astype(T)
        kr = _rfftfreq(nx, 2 * math.pi / Lx * nx).astype(T)
        with np.errstate(divide="ignore"):
            invksq = (1 / k ** 2).astype(T)
            invkrsq = (1 / kr ** 2).astype(T)
        invksq[0] = 0
        invkrsq[0] = 0
        self.k_host, self.kr_host = k, kr
        self.k, self.kr = self._upload(k), self._upload(kr)
        self.invksq, self.invkrsq = self._upload(invksq), self._upload(invkrsq)
        self._make_plans((self.nx,))
        self.aliased_fraction = T(aliased_fraction)
        self.kalias, self.kralias = getaliasedwavenumbers(self.nk, self.nkr, aliased_fraction)

    def __repr__(self):
        return ("OneDimensionalGrid\n"
                f"  ├─────────── Device: {self.device!r}\n"
                f"  ├──────── FloatType: {_jl_type(self._T)}\n"
                f"  ├────────── size Lx: {_show_float(self.Lx)}\n"
                f"  ├──── resolution nx: {self.nx}\n"
                f"  ├── grid spacing dx: {_show_float(self.dx)}\n"
                f"  ├─────────── domain: x ∈ [{_show_float(self.x[0])}, {_show_float(self.x[-1])}]\n"
                f"  └─ aliased fraction: {_show_float(self.aliased_fraction)}")


class TwoDGrid(AbstractGrid):
    """TwoDGrid(dev; nx, Lx, ny=nx, Ly=Lx, ...), src/domains.jl:175-223."""
    ndim = 2

    def __init__(self, dev=None, *, nx, Lx, ny=None, Ly=None, x0=None, y0=None, nthreads=None, effort=None,
                 T=np.float64, aliased_fraction=1 / 3):
        dev = dev if dev is not None else CPU()
        ny = nx if ny is None else ny
        Ly = Lx if Ly is None else Ly
        if nx % 2 != 0 or ny % 2 != 0:
            raise DomainError("nx and ny must be even")
        T = np.dtype(T).type
        self._T, self.device = T, dev
        self.nx, self.ny = int(nx), int(ny)
        self.nk, self.nl, self.nkr = self.nx, self.ny, self.nx // 2 + 1
        self._n = (self.nx, self.ny)
        self.Lx, self.Ly = T(Lx), T(Ly)
        self.dx, self.dy = T(Lx / nx), T(Ly / ny)
        x0 = -Lx / 2 if x0 is None else x0
        y0 = -Ly / 2 if y0 is None else y0
        self.x = _range_points(x0, Lx / nx, nx, T)
        self.y = _range_points(y0, Ly / ny, ny, T)
        k = _fftfreq(nx, 2 * math.pi / Lx * nx).astype(T).reshape(nx, 1)
        l = _fftfreq(ny, 2 * math.pi / Ly * ny).astype(T).reshape(1, ny)
        kr = _rfftfreq(nx, 2 * math.pi / Lx * nx).astype(T).reshape(self.nkr, 1)
        Ksq = (k ** 2 + l ** 2).astype(T)
        Krsq = (kr ** 2 + l ** 2).astype(T)
        with np.errstate(divide="ignore"):
            invKsq = (1 / Ksq).astype(T)
            invKrsq = (1 / Krsq).astype(T)
        invKsq[0, 0] = 0
        invKrsq[0, 0] = 0
        self.k_host, self.l_host, self.kr_host = k, l, kr
        self.Krsq_host, self.invKrsq_host = Krsq, invKrsq
        self.k, self.l, self.kr = self._upload(k), self._upload(l), self._upload(kr)
        self.Ksq, self.invKsq = self._upload(Ksq), self._upload(invKsq)
        self.Krsq, self.invKrsq = self._upload(Krsq), self._upload(invKrsq)
        self._make_plans((self.nx, self.ny))
        self.aliased_fraction = T(aliased_fraction)
        self.kalias, self.kralias = getaliasedwavenumbers(self.nk, self.nkr, aliased_fraction)
        self.lalias, _ = getaliasedwavenumbers(self.nl, self.nl, aliased_fraction)

    def __repr__(self):
        return ("TwoDimensionalGrid\n"
                f"  ├───────────────── Device: {self.device!r}\n"
                f"  ├────────────── FloatType: {_jl_type(self._T)}\n"
                f"  ├────────── size (Lx, Ly): ({_show_float(self.Lx)}, {_show_float(self.Ly)})\n"
                f"  ├──── resolution (nx, ny): ({self.nx}, {self.ny})\n"
                f"  ├── grid spacing (dx, dy): ({_show_float(self.dx)}, {_show_float(self.dy)})\n"
                f"  ├───────────────── domain: x ∈ [{_show_float(self.x[0])}, {_show_float(self.x[-1])}]\n"
                f"  |                          y ∈ [{_show_float(self.y[0])}, {_show_float(self.y[-1])}]\n"
                f"  └─ aliased fraction: {_show_float(self.aliased_fraction)}")


class ThreeDGrid(AbstractGrid):
    """ThreeDGrid(dev; nx, Lx, ny=nx, Ly=Lx, nz=nx, Lz=Lx, ...), src/domains.jl:311-366."""
    ndim = 3

    def __init__(self, dev=None, *, nx, Lx, ny=None, Ly=None, nz=None, Lz=None, x0=None, y0=None, z0=None,
                 nthreads=None, effort=None, T=np.float64, aliased_fraction=1 / 3):
        dev = dev if dev is not None else CPU()
        ny = nx if ny is None else ny
        Ly = Lx if Ly is None else Ly
        nz = nx if nz is None else nz
        Lz = Lx if Lz is None else Lz
        if nx % 2 != 0 or ny % 2 != 0 or nz % 2 != 0:
            raise DomainError("nx, ny, and nz must be even")
        T = np.dtype(T).type
        self._T, self.device = T, dev
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        self.nk, self.nl, self.nm, self.nkr = self.nx, self.ny, self.nz, self.nx // 2 + 1
        self._n = (self.nx, self.ny, self.nz)
        self.Lx, self.Ly, self.Lz = T(Lx), T(Ly), T(Lz)
        self.dx, self.dy, self.dz = T(Lx / nx), T(Ly / ny), T(Lz / nz)
        x0 = -Lx / 2 if x0 is None else x0
        y0 = -Ly / 2 if y0 is None else y0
        z0 = -Lz / 2 if z0 is None else z0
        self.x = _range_points(x0, Lx / nx, nx, T)
        self.y = _range_points(y0, Ly / ny, ny, T)
        self.z = _range_points(z0, Lz / nz, nz, T)
        k = _fftfreq(nx, 2 * math.pi / Lx * nx).astype(T).reshape(nx, 1, 1)
        l = _fftfreq(ny, 2 * math.pi / Ly * ny).astype(T).reshape(1, ny, 1)
        m = _fftfreq(nz, 2 * math.pi / Lz * nz).astype(T).reshape(1, 1, nz)
        kr = _rfftfreq(nx, 2 * math.pi / Lx * nx).astype(T).reshape(self.nkr, 1, 1)
        Ksq = (k ** 2 + l ** 2 + m ** 2).astype(T)
        Krsq = (kr ** 2 + l ** 2 + m ** 2).astype(T)
        with np.errstate(divide="ignore"):
            invKsq = (1 / Ksq).astype(T)
            invKrsq = (1 / Krsq).astype(T)
        invKsq[0, 0, 0] = 0
        invKrsq[0, 0, 0] = 0
        self.k_host, self.l_host, self.m_host, self.kr_host = k, l, m, kr
        self.Krsq_host = Krsq
        self.k, self.l, self.m, self.kr = self._upload(k), self._upload(l), self._upload(m), self._upload(kr)
        self.Ksq, self.invKsq = self._upload(Ksq), self._upload(invKsq)
        self.Krsq, self.invKrsq = self._upload(Krsq), self._upload(invKrsq)
        self._make_plans((self.nx, self.ny, self.nz))
        self.aliased_fraction = T(aliased_fraction)
        self.kalias, self.kralias = getaliasedwavenumbers(self.nk, self.nkr, aliased_fraction)
        self.lalias, _ = getaliasedwavenumbers(self.nl, self.nl // 2 + 1, aliased_fraction)
        self.malias, _ = getaliasedwavenumbers(self.nm, self.nm // 2 + 1, aliased_fraction)

    def __repr__(self):
        return ("ThreeDimensionalGrid\n"
                f"  ├───────────────────── Device: {self.device!r}\n"
                f"  ├────────────────── FloatType: {_jl_type(self._T)}\n"
                f"  ├────────── size (Lx, Ly, Lz): ({_show_float(self.Lx)}, {_show_float(self.Ly)}, "
                f"{_show_float(self.Lz)})\n"
                f"  ├──── resolution (nx, ny, nz): ({self.nx}, {self.ny}, {self.nz})\n"
                f"  ├── grid spacing (dx, dy, dz): ({_show_float(self.dx)}, {_show_float(self.dy)}, "
                f"{_show_float(self.dz)})\n"
                f"  ├────────────────────  domain: x ∈ [{_show_float(self.x[0])}, {_show_float(self.x[-1])}]\n"
                f"  |                              y ∈ [{_show_float(self.y[0])}, {_show_float(self.y[-1])}]\n"
                f"  |                              z ∈ [{_show_float(self.z[0])}, {_show_float(self.z[-1])}]\n"
                f"  └─ aliased fraction: {_show_float(self.aliased_fraction)}")


def _jl_type(T):
    return {np.float64: "Float64", np.float32: "Float32"}.get(np.dtype(T).type, str(T))


def gridpoints(grid):
    """gridpoints(grid): the collocation points as device arrays (src/domains.jl:379-398)."""
    conv = device_array(grid.device)
    if grid.ndim == 1:
        return conv(grid.x.copy())
    if grid.ndim == 2:
        X = np.broadcast_to(grid.x.reshape(-1, 1), (grid.nx, grid.ny))
        Y = np.broadcast_to(grid.y.reshape(1, -1), (grid.nx, grid.ny))
        return conv(np.array(X)), conv(np.array(Y))
    shp = (grid.nx, grid.ny, grid.nz)
    X = np.broadcast_to(grid.x.reshape(-1, 1, 1), shp)
    Y = np.broadcast_to(grid.y.reshape(1, -1, 1), shp)
    Z = np.broadcast_to(grid.z.reshape(1, 1, -1), shp)
    return conv(np.array(X)), conv(np.array(Y)), conv(np.array(Z))


def dealias_(fh, grid, stream=None):
    """dealias!(fh, grid): zero the aliased index ranges in place (src/domains.jl:428-476).

    The first dimension uses ``kralias`` when ``size(fh, 1) == nkr`` and ``kalias``
    otherwise; trailing dimensions beyond the grid's are treated as a batch.  A no-op
    for grids built with ``aliased_fraction = 0`` (src/domains.jl:434)."""
    if grid.kalias is None:
        return None
    lo, hi = grid._alias_bounds(fh.shape[0])
    shape = tuple(fh.shape)
    nd = grid.ndim
    dims = list(shape[:nd]) + [1] * (3 - nd)
    b = 1
    for s in shape[nd:]:
        b *= s
    dims.append(b)
    _lib.call("ff_dealias", prec_of(fh.dtype), ptr(fh, "dealias_"), _lib.i64_array(dims), _lib.i64_array(lo),
              _lib.i64_array(hi), stream_handle(stream))
    return None


def makefilter_K(K, order=4, innerK=2 / 3, outerK=1, tol=1e-15):
    """makefilter(K; order, innerK, outerK, tol) on a host array (src/domains.jl:506-516)."""
    K = np.asarray(K)
    decay = -math.log(tol) / (outerK - innerK) ** order
    with np.errstate(invalid="ignore", over="ignore"):
        f = np.exp(-decay * (K.astype(np.float64) - innerK) ** order)
    f[K < innerK] = 1
    return f


def _filter_K(g, realvars):
    T = g._T
    pi = T(math.pi)
    if g.ndim == 1:
        return g.kr_host.reshape(-1) * g.dx / pi if realvars else np.abs(g.k_host.reshape(-1) * g.dx / pi)
    kk = g.kr_host if realvars else g.k_host
    if g.ndim == 2:
        return np.sqrt((kk * g.dx / pi) ** 2 + (g.l_host * g.dy / pi) ** 2)
    return np.sqrt((kk * g.dx / pi) ** 2 + (g.l_host * g.dy / pi) ** 2 + (g.m_host * g.dz / pi) ** 2)


def makefilter(g, T=None, sz=None, realvars=True, **kw):
    """makefilter(grid; realvars, kwargs...) and makefilter(grid, T, sz; kwargs...)
    (src/domains.jl:520-546).  Returned as a device array on the grid's device; the
    values are computed in FP64 as in the reference and stored in ``T`` (default FP64)."""
    if sz is None:
        f = makefilter_K(_filter_K(g, realvars), **kw)
        return device_array(g.device)(f)
    sz = tuple(sz)
    f = makefilter_K(_filter_K(g, sz[0] == g.nkr), **kw)
    full = np.ones(sz) * f.reshape(f.shape + (1,) * (len(sz) - f.ndim))
    return device_array(g.device)(full.astype(T if T is not None else np.float64))


def makefilter_host(g, sz, **kw):
    """The FP64 filter for an array of size ``sz`` on grid ``g`` (host numpy)."""
    sz = tuple(sz)
    f = makefilter_K(_filter_K(g, sz[0] == g.nkr), **kw)
    return np.ones(sz) * f.reshape(f.shape + (1,) * (len(sz) - f.ndim))
