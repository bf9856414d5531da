"""Equation, Clock, Problem (src/problem.jl:11-136)."""
from __future__ import annotations

import numpy as np

from .devices import cxtype, zeros


class AbstractParams:
    def __repr__(self):
        return _show_fields("Parameters", "parameter", self)


class AbstractVars:
    def __repr__(self):
        return _show_fields("Variables", "variable", self)


def _summary(v):
    if callable(v) and not hasattr(v, "shape"):
        return "Function"
    if hasattr(v, "shape") and hasattr(v, "dtype"):
        shape = tuple(v.shape)
        if len(shape) == 1:
            return f"{shape[0]}-element array of {v.dtype}"
        return f"{'×'.join(str(s) for s in shape)} array of {v.dtype}"
    return type(v).__name__


def _show_fields(title, word, obj):
    names = [n for n in vars(obj) if not n.startswith("_")]
    if not names:
        return title + "\n"
    s = ""
    for n in names[:-1]:
        s += f"  ├───── {word}: {n} -> {_summary(getattr(obj, n))}\n"
    n = names[-1]
    s += f"  └───── {word}: {n} -> {_summary(getattr(obj, n))}\n"
    return title + "\n" + s


class EmptyParams(AbstractParams):
    """A placeholder for parameters (src/problem.jl:81)."""


class EmptyVars(AbstractVars):
    """A placeholder for variables (src/problem.jl:88)."""


def supersize(a):
    """supersize(a): size of an array, or a tuple of sizes (src/utils.jl:55-57)."""
    if isinstance(a, (list, tuple)):
        return tuple(tuple(x.shape) for x in a)
    return tuple(a.shape)


class Equation:
    """Equation(L, calcN!, grid; dims=supersize(L), T=cxtype(eltype(grid))), src/problem.jl:11-34.

    ``L`` holds the coefficients of the linear term L*u (a device array, or a scalar
    with explicit ``dims``); ``calcN`` is called as ``calcN(N, sol, t, clock, vars,
    params, grid)`` and must write the nonlinear term into ``N``."""

    def __init__(self, L, calcN, grid, dims=None, T=None):
        self.L = L
        self.calcN = calcN
        self.grid = grid
        self.dims = tuple(dims) if dims is not None else supersize(L)
        self.T = np.dtype(T).type if T is not None else cxtype(grid.T)

    def __repr__(self):
        Lt = getattr(self.L, "dtype", type(self.L).__name__)
        Ls = tuple(getattr(self.L, "shape", ()))
        return ("Equation\n"
                "  ├──────── linear coefficients: L\n"
                f"  │                              ├───type: {Lt}\n"
                f"  │                              └───size: {Ls}\n"
                "  ├───────────── nonlinear term: calcN!()\n"
                f"  └─── type of state vector sol: {np.dtype(self.T).name}")


class Clock:
    """Clock{T}(dt, t, step), src/problem.jl:43-50; dt and t are in the grid's float type."""

    def __init__(self, dt, t=0, step=0, T=np.float64):
        self._T = np.dtype(T).type
        self.dt = self._T(dt)
        self.t = self._T(t)
        self.step = int(step)

    def __setattr__(self, name, value):
        if name in ("dt", "t") and "_T" in self.__dict__:
            value = self._T(value)
        object.__setattr__(self, name, value)

    def __repr__(self):
        return ("Clock\n"
                f"  ├─── timestep dt: {float(self.dt)!r}\n"
                f"  ├────────── step: {self.step}\n"
                f"  └──────── time t: {float(self.t)!r}")


class Problem:
    """Problem(eqn, stepper, dt, grid, vars=EmptyVars(), params=EmptyParams(); stepperkwargs...),
    src/problem.jl:99-111.  The device is the grid's; ``sol`` starts at zero."""

    def __init__(self, eqn, stepper, dt, grid, vars=None, params=None, **stepperkwargs):
        from .timesteppers import TimeStepper
        dev = grid.device
        self.eqn = eqn
        self.grid = grid
        self.vars = vars if vars is not None else EmptyVars()
        self.params = params if params is not None else EmptyParams()
        self.clock = Clock(dt, 0, 0, grid.T)
        self.timestepper = TimeStepper(stepper, eqn, dt, dev, **stepperkwargs)
        self.sol = zeros(dev, eqn.T, eqn.dims)

    def __repr__(self):
        return ("Problem\n"
                f"  ├─────────── grid: grid (on {self.grid.device!r})\n"
                "  ├───── parameters: params\n"
                "  ├────── variables: vars\n"
                "  ├─── state vector: sol\n"
                "  ├─────── equation: eqn\n"
                "  ├────────── clock: clock\n"
                f"  │                  └──── dt: {float(self.clock.dt)!r}\n"
                f"  └──── timestepper: {type(self.timestepper).__name__}")
