"""The Diffusion module (src/diffusion.jl:1-178) on libfourierflows_gb300.

``Problem(dev; nx, Lx, kappa, dt, stepper, aliased_fraction, T)`` builds the 1D diffusion
problem of the reference: constant kappa gives L = -kappa kr^2 and N = 0; an array kappa
gives L = 0 and N = d/dx(kappa dc/dx) computed with two transforms.  ``Problem3D`` is
the ThreeDGrid constant-kappa variant (L = -kappa Krsq) used by the ensemble form.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib
from .devices import GPU, cxtype, device_array, on_device, prec_of, ptr, stream_handle, zeros
from .domains import OneDGrid, ThreeDGrid
from .plans import ldiv_, mul_
from .problem import AbstractParams, AbstractVars, Equation as _Equation, Problem as _Problem
from .utils import _mul_ik


class Params(AbstractParams):
    """Params(kappa): diffusivity, a number or an array on the grid (src/diffusion.jl:68-74)."""

    def __init__(self, kappa):
        self.κ = kappa

    @property
    def kappa(self):
        return self.κ


def make_params(grid, kappa):
    if np.ndim(kappa) == 0 and not on_device(kappa):
        return Params(kappa)
    return Params(device_array(grid.device)(np.asarray(kappa.cpu() if on_device(kappa) else kappa, dtype=grid.T)))


class Vars(AbstractVars):
    """c, cx (physical) and ch, cxh (spectral) (src/diffusion.jl:99-122)."""

    def __init__(self, grid):
        T = grid.T
        dev = grid.device
        self.c = zeros(dev, T, (grid.nx,))
        self.cx = zeros(dev, T, (grid.nx,))
        self.ch = zeros(dev, cxtype(T), (grid.nkr,))
        self.cxh = zeros(dev, cxtype(T), (grid.nkr,))


class _LinearStep:
    """Whole steps of a constant-kappa problem, where calcN! gives N = 0: one native pass
    per step (``ff_linear_step``) instead of the stepper's four N fills and four substep
    passes.  ETDRK4 then computes sol = exp(L dt) sol exactly (every N term adds an exact
    zero); RK4 runs its four linear stages in registers in the generic kernels' order.
    The stepper's intermediate buffers are not touched.  Falls back to the generic
    substeps if params.kappa is an array at step time."""

    def __init__(self, ts, eq):
        from . import timesteppers as tsm
        self.ts, self.eq = ts, eq
        self.kind = _lib.FF_STEP_ETDRK4 if isinstance(ts, tsm.ETDRK4TimeStepper) else _lib.FF_STEP_RK4

    def step(self, sol, clock, vars, params, grid):
        from .timesteppers import _coef, _opt
        if on_device(params.κ):
            self.ts._step(sol, clock, self.eq, vars, params, grid)
            return
        n = sol.numel()
        c = self.ts.expLdt if self.kind == _lib.FF_STEP_ETDRK4 else self.eq.L
        _lib.call("ff_linear_step", prec_of(sol.dtype), self.kind, n, ptr(sol, "sol"), _coef(c, n), float(clock.dt),
                  _opt(self.ts.filter), 1, stream_handle())


class _DiffusionCalcN:
    """calcN!(N, sol, t, clock, vars, params, grid), src/diffusion.jl:129-143.

    Constant kappa: N = 0.  Array kappa: cxh = i kr sol; cx = irfft(cxh); cx *= kappa;
    cxh = rfft(cx); N = i kr cxh -- four native launches."""
    __name__ = "calcN!"

    def fused_stepper(self, ts, eq):
        """A one-pass step for an equation built with constant kappa (N = 0) under the
        ETDRK4 and RK4 steppers (plain or Filtered), or None for the generic substeps."""
        from . import timesteppers as tsm
        if not getattr(eq, "zero_N", False) or not isinstance(eq.grid.device, GPU):
            return None
        if isinstance(ts, (tsm.ETDRK4TimeStepper, tsm.RK4TimeStepper)):
            return _LinearStep(ts, eq)
        return None

    def __call__(self, N, sol, t, clock, vars, params, grid):
        k = params.κ
        if not on_device(k):
            N.zero_()  # @. N = 0 on a device buffer
            return None
        _mul_ik(vars.cxh, sol, grid.kr)
        ldiv_(vars.cx, grid.rfftplan, vars.cxh)
        _lib.call("ff_real_mul", prec_of(vars.cx.dtype), vars.cx.numel(), k.numel(), ptr(vars.cx, "cx"),
                  ptr(k, "kappa"), stream_handle())
        mul_(vars.cxh, grid.rfftplan, vars.cx)
        _mul_ik(N, vars.cxh, grid.kr)
        return None


calcN_ = _DiffusionCalcN()


def Equation(grid, params):
    """L = -kappa kr^2 for constant kappa, else L = 0 with dims (nkr,) (src/diffusion.jl:82-90)."""
    if on_device(params.κ):
        return _Equation(0, calcN_, grid, dims=(grid.nkr,), T=cxtype(grid.T))
    kr = grid.kr_host.reshape(-1).astype(np.float64)
    L = (-params.κ * kr ** 2).astype(grid.T)
    return _linear(_Equation(device_array(grid.device)(L), calcN_, grid))


def _linear(eq):
    """Mark an equation whose calcN! is this module's with constant kappa (N = 0)."""
    eq.zero_N = True
    return eq


def Problem(dev=None, *, nx=128, Lx=2 * math.pi, κ=0, kappa=None, dt=0.01, stepper="RK4", aliased_fraction=0,
            T=np.float64):
    """Diffusion.Problem(dev; nx=128, Lx=2pi, kappa=0, dt=0.01, stepper="RK4",
    aliased_fraction=0, T=Float64), src/diffusion.jl:44-59."""
    dev = dev if dev is not None else GPU()
    kappa = κ if kappa is None else kappa
    grid = OneDGrid(dev, nx=nx, Lx=Lx, aliased_fraction=aliased_fraction, T=T)
    params = make_params(grid, kappa)
    vars = Vars(grid)
    eq = Equation(grid, params)
    return _Problem(eq, stepper, dt, grid, vars, params)


def updatevars_(prob_or_vars, grid=None, sol=None):
    """updatevars!(vars, grid, sol) / updatevars!(prob) (src/diffusion.jl:150-162)."""
    if grid is None:
        prob = prob_or_vars
        vars, grid, sol = prob.vars, prob.grid, prob.sol
    else:
        vars = prob_or_vars
    vars.ch.copy_(sol)
    _mul_ik(vars.cxh, sol, grid.kr)
    ldiv_(vars.c, grid.rfftplan, vars.ch)  # the native inverse never clobbers its input
    ldiv_(vars.cx, grid.rfftplan, vars.cxh)
    return None


def set_c_(prob, c):
    """set_c!(prob, c): sol = rfft(c), then updatevars! (src/diffusion.jl:167-176)."""
    src = c if on_device(c) else device_array(prob.grid.device)(np.asarray(c, dtype=prob.grid.T))
    prob.vars.c.copy_(src.reshape(prob.vars.c.shape))
    mul_(prob.sol, prob.grid.rfftplan, prob.vars.c)
    updatevars_(prob)
    return None


def Problem3D(dev=None, *, n, L=2 * math.pi, kappa, dt, stepper="ETDRK4", T=np.float64):
    """Constant-kappa diffusion on a ThreeDGrid n^3: L = -kappa Krsq, N = 0."""
    dev = dev if dev is not None else GPU()
    grid = ThreeDGrid(dev, nx=n, Lx=L, aliased_fraction=0, T=T)
    params = Params(kappa)
    Lop = (-kappa * grid.Krsq_host.astype(np.float64)).astype(T)
    eq = _linear(_Equation(device_array(dev)(Lop), calcN_, grid))
    return _Problem(eq, stepper, dt, grid, None, params)


class Ensemble3D:
    """B independent constant-kappa diffusion problems on one ThreeDGrid n^3, stacked along
    a trailing batch dimension and advanced as one problem: L = -kappa_b Krsq has shape
    (nkr, n, n, B), and with N = 0 each ETDRK4 or RK4 step is one native pass over all
    members (``ff_linear_step``).
    Initial conditions are Gaussian blobs (width sigma) at counter-based random centres."""

    def __init__(self, kappas, n=128, L=2 * math.pi, dt=2e-3, stepper="ETDRK4", T=np.float32, sigma=0.3, seed=7,
                 dev=None):
        from .vorticity import uniform01
        dev = dev if dev is not None else GPU()
        self.kappas = np.asarray(kappas, dtype=np.float64)
        B = len(self.kappas)
        self.grid = ThreeDGrid(dev, nx=n, Lx=L, aliased_fraction=0, T=T)
        g = self.grid
        Krsq = g.Krsq_host.astype(np.float64)
        Lop = np.empty(g.spectral_shape + (B,), dtype=T, order="F")
        for b in range(B):
            Lop[..., b] = -self.kappas[b] * Krsq
        eq = _linear(_Equation(device_array(dev)(Lop), calcN_, g, dims=Lop.shape))
        kw = {"coefficients": "device"} if stepper.replace("Filtered", "") == "ETDRK4" else {}
        self.prob = _Problem(eq, stepper, dt, g, None, Params(0.0), **kw)
        # Gaussian blobs at random centres (minimum-image distance on the periodic box)
        u = uniform01(seed, 3 * B).reshape(B, 3)
        x = [g.x.astype(np.float64), g.y.astype(np.float64), g.z.astype(np.float64)]
        c = np.empty((n, n, n, B), dtype=T, order="F")
        for b in range(B):
            d2 = 0.0
            for ax in range(3):
                xc = x[ax][0] + u[b, ax] * L
                d = (x[ax] - xc + L / 2) % L - L / 2
                shape = [1, 1, 1]
                shape[ax] = n
                d2 = d2 + (d ** 2).reshape(shape)
            c[..., b] = np.exp(-d2 / (2 * sigma ** 2))
        mul_(self.prob.sol, g.rfftplan, device_array(dev)(c))
        self.B = B

    def stepforward_(self, nsteps=1):
        from .timesteppers import stepforward_
        stepforward_(self.prob, nsteps)

    @property
    def grid_points(self):
        return self.B * self.grid.nx * self.grid.ny * self.grid.nz
