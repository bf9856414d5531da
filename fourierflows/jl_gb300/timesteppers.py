"""Time steppers (src/timesteppers.jl) on libfourierflows_gb300.

Each ``*TimeStepper`` keeps the reference's buffers and coefficients as device arrays.
Its ``step`` calls the equation's ``calcN`` exactly where the reference does and runs
every group of broadcasts between two ``calcN`` calls as ONE fused native pass
(``ff_euler_update``, ``ff_rk4_substep``, ``ff_lsrk54_stage``, ``ff_etdrk4_*``,
``ff_ab3_update``), filter included.  When ``calcN`` is a native functor that can fuse
the whole step (the 2D vorticity term), ``step`` hands the step to it instead.

Coefficient set-up follows the reference: ``getexpLs`` in L's float type, the ETDRK4
contour means in FP64 (src/timesteppers.jl:689-718) -- stored in the state's float
type, which for FP32 states rounds the coefficients the reference keeps in FP64.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

from . import _lib
from .devices import (CPU, GPU, device_array, fltype, on_device, prec_of, ptr, real_dtype_of, stream_handle,
                      to_numpy, zeros)
from .domains import makefilter_host

FULLY_EXPLICIT = ["ForwardEuler", "RK4", "AB3", "LSRK54", "FilteredForwardEuler", "FilteredRK4", "FilteredAB3",
                  "FilteredLSRK54"]


def isexplicit(stepper) -> bool:
    """src/timesteppers.jl:37-48."""
    return str(stepper) in FULLY_EXPLICIT


def TimeStepper(stepper, equation, dt=None, dev=None, **kw):
    """TimeStepper(stepper, equation, dt, dev; kw...): the stepper named ``stepper``
    (src/timesteppers.jl:57-69)."""
    dev = dev if dev is not None else equation.grid.device
    name = f"{stepper}TimeStepper"
    cls = globals().get(name)
    if cls is None or not isinstance(cls, type):
        raise ValueError(f"UndefVarError: {name} not defined")
    if isexplicit(stepper):
        return cls(equation, dev, **kw)
    return cls(equation, dt, dev, **kw)


# ----------------------------------------------------------------------------------------
# helpers
# ----------------------------------------------------------------------------------------
def _require_gpu(dev):
    if not isinstance(dev, GPU):
        raise NotImplementedError("time-stepping runs on the GPU() device only: this library implements the "
                                  "reference's GPU path")


def _coef(x, n=None):
    """ff_coef for L or an ETDRK4 coefficient: scalar, real array or complex array."""
    c = _lib.ff_coef()
    if x is None:
        c.kind = _lib.FF_COEF_NONE
        return c
    if on_device(x):
        if x.numel() == 1 and (n is None or n > 1):
            v = complex(x.reshape(-1)[0].item())
            c.kind, c.re, c.im = _lib.FF_COEF_SCALAR, v.real, v.imag
            return c
        if n is not None and x.numel() != n:
            raise ValueError(f"coefficient has {x.numel()} entries, the state has {n}")
        c.ptr = ptr(x, "coefficient").value
        c.kind = _lib.FF_COEF_COMPLEX if x.dtype.is_complex else _lib.FF_COEF_REAL
        return c
    a = np.asarray(x)
    if a.size != 1:
        raise TypeError("array coefficients must be device arrays (GPU())")
    v = complex(a.reshape(-1)[0])
    c.kind, c.re, c.im = _lib.FF_COEF_SCALAR, v.real, v.imag
    return c


def _opt(t):
    return None if t is None else ptr(t, "array")


def _numel(eq):
    n = 1
    for d in eq.dims:
        n *= d
    return n


def _host_L(L):
    if on_device(L):
        return to_numpy(L)
    return np.asarray(L)


def _to_device_like(a, eq, dev):
    """Coefficient array (host numpy) to a device array in the state's real precision,
    or a Python scalar for 0-dimensional coefficients."""
    a = np.asarray(a)
    rt = fltype(eq.T)
    if a.ndim == 0 or a.size == 1 and len(eq.dims) and _numel(eq) > 1:
        v = a.reshape(-1)[0]
        return complex(v) if np.iscomplexobj(v) else float(v)
    if np.iscomplexobj(a):
        return device_array(dev)(a.astype(np.complex64 if rt == np.float32 else np.complex128))
    return device_array(dev)(a.astype(rt))


class AbstractTimeStepper:
    """Abstract supertype for timesteppers (src/FourierFlows.jl:83)."""
    _fused = None
    _fused_checked = False

    def _native(self, eqn):
        if not self._fused_checked:
            self._fused_checked = True
            maker = getattr(eqn.calcN, "fused_stepper", None)
            if maker is not None:
                self._fused = maker(self, eqn)
        return self._fused

    def step(self, sol, clock, eqn, vars, params, grid):
        fused = self._native(eqn)
        if fused is not None:
            fused.step(sol, clock, vars, params, grid)
        else:
            self._step(sol, clock, eqn, vars, params, grid)
        clock.t = clock.t + clock.dt
        clock.step += 1

    def _filter_for(self, eq):
        return None


def _setup_filter(eq, dev, kw):
    f = makefilter_host(eq.grid, eq.dims, **kw)
    return device_array(dev)(f.astype(fltype(eq.T)))


# ----------------------------------------------------------------------------------------
# Forward Euler
# ----------------------------------------------------------------------------------------
class ForwardEulerTimeStepper(AbstractTimeStepper):
    """u^{n+1} = u^n + dt RHS(u^n, t^n)  (src/timesteppers.jl:98-119)."""

    def __init__(self, equation, dev=None, **kw):
        dev = dev if dev is not None else GPU()
        _require_gpu(dev)
        self.N = zeros(dev, equation.T, equation.dims)
        self.filter = _setup_filter(equation, dev, kw) if self._filtered else None

    _filtered = False

    def _step(self, sol, clock, eq, vars, params, grid):
        eq.calcN(self.N, sol, clock.t, clock, vars, params, grid)
        _lib.call("ff_euler_update", prec_of(sol.dtype), sol.numel(), ptr(sol, "sol"), ptr(self.N, "N"),
                  _coef(eq.L, sol.numel()), float(clock.dt), _opt(self.filter), stream_handle())


class FilteredForwardEulerTimeStepper(ForwardEulerTimeStepper):
    """Forward Euler with spectral filtering (src/timesteppers.jl:126-150)."""
    _filtered = True


# ----------------------------------------------------------------------------------------
# RK4
# ----------------------------------------------------------------------------------------
class RK4TimeStepper(AbstractTimeStepper):
    """Classic 4th-order Runge-Kutta (src/timesteppers.jl:180-274)."""
    _filtered = False

    def __init__(self, equation, dev=None, **kw):
        dev = dev if dev is not None else GPU()
        _require_gpu(dev)
        T, d = equation.T, equation.dims
        self.sol1, self.RHS1, self.RHS2, self.RHS3, self.RHS4 = (zeros(dev, T, d) for _ in range(5))
        self.filter = _setup_filter(equation, dev, kw) if self._filtered else None

    def _step(self, sol, clock, eq, vars, params, grid):
        n, p, s = sol.numel(), prec_of(sol.dtype), stream_handle()
        L = _coef(eq.L, n)
        Tf = type(clock.dt)
        dt, t = clock.dt, clock.t
        half = Tf(dt / Tf(2))
        ps, p1 = ptr(sol, "sol"), ptr(self.sol1, "sol1")
        eq.calcN(self.RHS1, sol, t, clock, vars, params, grid)
        _lib.call("ff_rk4_substep", p, n, ptr(self.RHS1), L, ps, ps, p1, float(half), s)
        eq.calcN(self.RHS2, self.sol1, Tf(t + half), clock, vars, params, grid)
        _lib.call("ff_rk4_substep", p, n, ptr(self.RHS2), L, p1, ps, p1, float(half), s)
        eq.calcN(self.RHS3, self.sol1, Tf(t + half), clock, vars, params, grid)
        _lib.call("ff_rk4_substep", p, n, ptr(self.RHS3), L, p1, ps, p1, float(dt), s)
        eq.calcN(self.RHS4, self.sol1, Tf(t + dt), clock, vars, params, grid)
        _lib.call("ff_rk4_update", p, n, ps, ptr(self.RHS4), L, p1, ptr(self.RHS1), ptr(self.RHS2),
                  ptr(self.RHS3), float(Tf(dt / Tf(6))), _opt(self.filter), s)


class FilteredRK4TimeStepper(RK4TimeStepper):
    """RK4 with spectral filtering (src/timesteppers.jl:204-223,276-285)."""
    _filtered = True


# ----------------------------------------------------------------------------------------
# LSRK54
# ----------------------------------------------------------------------------------------
_LSRK_A = [Fraction(0), Fraction(-567301805773, 1357537059087), Fraction(-2404267990393, 2016746695238),
           Fraction(-3550918686646, 2091501179385), Fraction(-1275806237668, 842570457699)]
_LSRK_B = [Fraction(1432997174477, 9575080441755), Fraction(5161836677717, 13612068292357),
           Fraction(1720146321549, 2090206949498), Fraction(3134564353537, 4481467310338),
           Fraction(2277821191437, 14882151754819)]
_LSRK_C = [Fraction(0), Fraction(1432997174477, 9575080441755), Fraction(2526269341429, 6820363962896),
           Fraction(2006345519317, 3224310063776), Fraction(2802321613138, 2924317926251)]


class LSRK54TimeStepper(AbstractTimeStepper):
    """4th-order 5-stage 2-register Runge-Kutta, Carpenter-Kennedy coefficients
    (src/timesteppers.jl:318-404)."""
    _filtered = False

    def __init__(self, equation, dev=None, **kw):
        dev = dev if dev is not None else GPU()
        _require_gpu(dev)
        T, d = equation.T, equation.dims
        self.S2, self.RHS = zeros(dev, T, d), zeros(dev, T, d)
        Tf = fltype(T)
        self.A = tuple(Tf(float(a)) for a in _LSRK_A)
        self.B = tuple(Tf(float(b)) for b in _LSRK_B)
        self.C = tuple(Tf(float(c)) for c in _LSRK_C)
        self.filter = _setup_filter(equation, dev, kw) if self._filtered else None

    def _step(self, sol, clock, eq, vars, params, grid):
        n, p, s = sol.numel(), prec_of(sol.dtype), stream_handle()
        L = _coef(eq.L, n)
        Tf = type(clock.dt)
        dt, t = clock.dt, clock.t
        ps = ptr(sol, "sol")
        for i in range(5):
            eq.calcN(self.RHS, sol, Tf(t + self.C[i] * dt), clock, vars, params, grid)
            last = i == 4
            _lib.call("ff_lsrk54_stage", p, n, ps, ptr(self.RHS), ptr(self.S2), L, float(self.A[i]),
                      float(self.B[i]), float(dt), 1 if i == 0 else 0, _opt(self.filter) if last else None, s)


class FilteredLSRK54TimeStepper(LSRK54TimeStepper):
    """LSRK54 with spectral filtering (src/timesteppers.jl:361-414)."""
    _filtered = True


# ----------------------------------------------------------------------------------------
# ETDRK4
# ----------------------------------------------------------------------------------------
def getexpLs(dt, equation):
    """exp(dt L), exp(dt L / 2) in L's float type (src/timesteppers.jl:673-678); host arrays."""
    L = _host_L(equation.L)
    if L.dtype.kind in "fc":
        dtL = (L.dtype.type(dt) * L).astype(L.dtype)
        half = (dtL / L.dtype.type(2)).astype(L.dtype)
    else:
        Tf = type(dt)
        dtL = np.asarray(dt * L, dtype=Tf)
        half = np.asarray(dtL / Tf(2), dtype=Tf)
    with np.errstate(over="ignore"):
        return np.exp(dtL), np.exp(half)


def getetdcoeffs(dt, L, ncirc=32, rcirc=1):
    """zeta, alpha, beta, Gamma by the Kassam-Trefethen contour means in FP64
    (src/timesteppers.jl:689-718); host arrays of L's shape."""
    L = _host_L(L)
    circ = rcirc * np.exp(2j * math.pi / ncirc * (np.arange(ncirc) + 0.5))
    if L.dtype.kind in "fc":
        dtL = (L.dtype.type(dt) * L).astype(L.dtype)
    else:
        dtL = np.asarray(type(dt)(dt) * L)
    return _etd_contour(np.asarray(dtL), dt, circ, L.dtype.kind != "c")


def _etd_contour(dtL, dt, circ, real):
    zc = dtL[..., None].astype(np.complex128) + circ
    ez, ez2 = np.exp(zc), np.exp(zc / 2)
    zeta = (ez2 - 1) / zc
    alpha = (-4 - zc + ez * (4 - 3 * zc + zc ** 2)) / zc ** 3
    beta = (2 + zc + ez * (-2 + zc)) / zc ** 3
    gamma = (-4 - 3 * zc - zc ** 2 + ez * (4 - zc)) / zc ** 3
    dt64 = np.float64(dt)
    out = [dt64 * c.mean(axis=-1) for c in (zeta, alpha, beta, gamma)]
    if real:
        out = [np.real(c) for c in out]
    return tuple(out)


class ETDRK4TimeStepper(AbstractTimeStepper):
    """Exponential time differencing RK4 (Kassam & Trefethen 2005), src/timesteppers.jl:434-547."""
    _filtered = False

    def __init__(self, equation, dt, dev=None, coefficients="host", **kw):
        """``coefficients="device"`` evaluates the contour means in FP64 on the GPU
        (``ff_etdrk4_coefficients``) instead of on the host; meant for very large real L."""
        dev = dev if dev is not None else GPU()
        _require_gpu(dev)
        Tf = fltype(equation.T)
        dt = Tf(dt)
        eL, ehL = getexpLs(dt, equation)
        self.expLdt, self.exp_half_Ldt = _to_device_like(eL, equation, dev), _to_device_like(ehL, equation, dev)
        if coefficients == "device" and on_device(equation.L) and not equation.L.dtype.is_complex:
            L = equation.L
            self.zeta, self.alpha, self.beta, self.Gamma = (zeros(dev, Tf, tuple(L.shape)) for _ in range(4))
            _lib.call("ff_etdrk4_coefficients", prec_of(L.dtype), L.numel(), ptr(L, "L"), float(dt), 32, 1.0,
                      ptr(self.zeta), ptr(self.alpha), ptr(self.beta), ptr(self.Gamma), stream_handle())
        else:
            z, a, b, g = getetdcoeffs(dt, equation.L)
            self.zeta, self.alpha, self.beta, self.Gamma = (_to_device_like(c, equation, dev) for c in (z, a, b, g))
        T, d = equation.T, equation.dims
        self.sol1, self.sol2, self.N1, self.N2, self.N3, self.N4 = (zeros(dev, T, d) for _ in range(6))
        self.filter = _setup_filter(equation, dev, kw) if self._filtered else None
        self.dt = dt

    def _step(self, sol, clock, eq, vars, params, grid):
        n, p, s = sol.numel(), prec_of(sol.dtype), stream_handle()
        Tf = type(clock.dt)
        t, dt = clock.t, clock.dt
        eh, z = _coef(self.exp_half_Ldt, n), _coef(self.zeta, n)
        ps, p1, p2 = ptr(sol, "sol"), ptr(self.sol1), ptr(self.sol2)
        eq.calcN(self.N1, sol, t, clock, vars, params, grid)
        _lib.call("ff_etdrk4_substep12", p, n, p1, eh, ps, z, ptr(self.N1), s)
        t2 = Tf(t + dt / Tf(2))
        eq.calcN(self.N2, self.sol1, t2, clock, vars, params, grid)
        _lib.call("ff_etdrk4_substep12", p, n, p2, eh, ps, z, ptr(self.N2), s)
        eq.calcN(self.N3, self.sol2, t2, clock, vars, params, grid)
        _lib.call("ff_etdrk4_substep3", p, n, p2, eh, p1, z, ptr(self.N1), ptr(self.N3), s)
        eq.calcN(self.N4, self.sol2, Tf(t + dt), clock, vars, params, grid)
        _lib.call("ff_etdrk4_update", p, n, ps, _coef(self.expLdt, n), _coef(self.alpha, n), _coef(self.beta, n),
                  _coef(self.Gamma, n), ptr(self.N1), ptr(self.N2), ptr(self.N3), ptr(self.N4), _opt(self.filter),
                  s)


class FilteredETDRK4TimeStepper(ETDRK4TimeStepper):
    """ETDRK4 with spectral filtering (src/timesteppers.jl:471-499,549-558)."""
    _filtered = True


# ----------------------------------------------------------------------------------------
# AB3
# ----------------------------------------------------------------------------------------
class AB3TimeStepper(AbstractTimeStepper):
    """3rd-order Adams-Bashforth, forward Euler for the first two steps
    (src/timesteppers.jl:586-651)."""
    _filtered = False

    def __init__(self, equation, dev=None, **kw):
        dev = dev if dev is not None else GPU()
        _require_gpu(dev)
        T, d = equation.T, equation.dims
        self.RHS, self.RHSm1, self.RHSm2 = zeros(dev, T, d), zeros(dev, T, d), zeros(dev, T, d)
        self.filter = _setup_filter(equation, dev, kw) if self._filtered else None

    def _step(self, sol, clock, eq, vars, params, grid):
        n, p, s = sol.numel(), prec_of(sol.dtype), stream_handle()
        eq.calcN(self.RHS, sol, clock.t, clock, vars, params, grid)
        _lib.call("ff_ab3_update", p, n, ptr(sol, "sol"), ptr(self.RHS), ptr(self.RHSm1), ptr(self.RHSm2),
                  _coef(eq.L, n), float(clock.dt), 1 if clock.step < 3 else 0, _opt(self.filter), s)


class FilteredAB3TimeStepper(AB3TimeStepper):
    """AB3 with spectral filtering (src/timesteppers.jl:609-667)."""
    _filtered = True


# ----------------------------------------------------------------------------------------
# drivers
# ----------------------------------------------------------------------------------------
def _one(prob):
    prob.timestepper.step(prob.sol, prob.clock, prob.eqn, prob.vars, prob.params, prob.grid)


def _many(prob, nsteps):
    """nsteps steps; a fused native stepper advances them in one call (graph replays)."""
    fused = prob.timestepper._native(prob.eqn)
    if fused is not None and hasattr(fused, "advance") and nsteps > 0:
        fused.advance(prob.sol, prob.clock, nsteps)
        clock = prob.clock
        for _ in range(nsteps):  # the reference's clock arithmetic, step by step
            clock.t = clock.t + clock.dt
            clock.step += 1
        return
    for _ in range(nsteps):
        _one(prob)


def stepforward_(*args):
    """stepforward!(prob), stepforward!(prob, nsteps), stepforward!(prob, diags, nsteps)
    (src/timesteppers.jl:6-35), and the per-stepper form
    stepforward!(sol, clock, ts, equation, vars, params, grid)."""
    from .problem import Problem
    from .diagnostics import increment_
    if args and isinstance(args[0], Problem):
        prob = args[0]
        if len(args) == 1:
            _one(prob)
        elif len(args) == 2:
            _many(prob, int(args[1]))
        elif len(args) == 3:
            diags, nsteps = args[1], int(args[2])
            for _ in range(nsteps):
                _one(prob)
                increment_(diags)
        else:
            raise TypeError("stepforward_(prob[, diags], nsteps)")
        return None
    if len(args) == 7:
        sol, clock, ts, eqn, vars, params, grid = args
        ts.step(sol, clock, eqn, vars, params, grid)
        return None
    raise TypeError("stepforward_: unsupported arguments")


def step_until_(prob, stop_time):
    """step_until!(prob, stop_time) for fully explicit steppers (src/timesteppers.jl:734-760),
    including the reference's ``t_remaining = time_interval - clock.t`` (:752)."""
    if isinstance(prob.timestepper, ETDRK4TimeStepper):
        raise RuntimeError("step_until! requires fully explicit time stepper; does not work with ETDRK4")
    if not stop_time > prob.clock.t:
        raise RuntimeError("stop_time must be greater than prob.clock.t")
    dt = prob.clock.dt
    time_interval = stop_time - prob.clock.t
    nsteps = math.floor(time_interval / dt)
    stepforward_(prob, nsteps)
    t_remaining = time_interval - prob.clock.t
    prob.clock.dt = t_remaining
    stepforward_(prob)
    prob.clock.dt = dt
    return None
