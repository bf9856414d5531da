"""Diagnostics (src/diagnostics.jl:8-126): host-side time series of ``calc(prob)``.

The bookkeeping stays on the host exactly as in the reference; the reductions a
``calc`` usually performs (``parsevalsum2``, the vorticity energy and enstrophy) are
native and return host scalars.
"""
from __future__ import annotations

import math


class AbstractDiagnostic:
    pass


class Diagnostic(AbstractDiagnostic):
    """Diagnostic(calc, prob; freq=1, nsteps=100, ndata=ceil((nsteps+1)/freq)).

    ``data``, ``t`` and ``steps`` are preallocated to ``ndata`` entries and doubled
    (``extend_``) when full; ``i`` counts the stored samples (1-based, as in Julia)."""

    def __init__(self, calc, prob, freq=1, nsteps=100, ndata=None):
        ndata = int(ndata) if ndata is not None else math.ceil((nsteps + 1) / freq)
        first = calc(prob)
        self.calc, self.prob, self.freq = calc, prob, int(freq)
        self.data = [None] * ndata
        self.t = [0.0] * ndata
        self.steps = [0] * ndata
        self.data[0] = first
        self.t[0] = float(prob.clock.t)
        self.steps[0] = prob.clock.step
        self.i = 1
        self.N = ndata

    def __call__(self):
        return self.calc(self.prob)

    def __getitem__(self, key):
        """d["t"] / d[:t]-style field access returns the stored part; d[idx] indexes data."""
        if isinstance(key, str):
            return getattr(self, key)[:self.i]
        if isinstance(key, range):
            return [self.data[j - 1] for j in key]  # Julia 1-based ranges
        return self.data[key]

    def __repr__(self):
        name = getattr(self.calc, "__name__", "calc")
        return ("Diagnostic\n"
                f"  ├─── calc: {name}\n"
                f"  ├─── prob: {type(self.prob).__name__}\n"
                f"  ├─── data: {len(self.data)}-element list\n"
                f"  ├────── t: {len(self.t)}-element list\n"
                f"  ├── steps: {len(self.steps)}-element list\n"
                f"  ├─── freq: {self.freq}\n"
                f"  └────── i: {self.i}")


def extend_(diag, n=None):
    """extend!(diag, n) / extend!(diag): grow the storage by n (default: the initial size)."""
    n = diag.N if n is None else int(n)
    diag.data += [None] * n
    diag.t += [0.0] * n
    diag.steps += [0] * n


def update_(diag, i=None):
    """update!(diag, i): store the current value at 1-based position i (src/diagnostics.jl:76-85)."""
    i = diag.i + 1 if i is None else int(i)
    if i > len(diag.steps):
        extend_(diag)
    diag.data[i - 1] = diag()
    diag.t[i - 1] = float(diag.prob.clock.t)
    diag.steps[i - 1] = diag.prob.clock.step
    diag.i = i


def increment_(diags):
    """increment!(diag) / increment!(diags): sample when step % freq == 0 (src/diagnostics.jl:92-104)."""
    if isinstance(diags, (list, tuple)):
        for d in diags:
            increment_(d)
        return None
    if diags.prob.clock.step % diags.freq == 0:
        update_(diags, diags.i + 1)
    return None
