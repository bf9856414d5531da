"""CPU oracle for the FourierFlows.jl pseudospectral time-stepping path (TEST INFRASTRUCTURE).

This module checks the product and is never part of it: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import it.
The GPU library in ``fourierflows/jl_gb300`` never calls it.

It is a plain numpy / scipy.fft FP64 restatement of the reference's algorithm, written
line-for-line against the Julia sources (paths relative to the FourierFlows.jl tree):

* grids, wavenumbers, alias ranges, dealias!, makefilter  -- src/domains.jl:61-101,175-223,311-366,408-476,506-546
* getexpLs, getetdcoeffs                                   -- src/timesteppers.jl:673-721
* the ten time-steppers and step_until!                    -- src/timesteppers.jl:98-760
* Equation / Clock / Problem                               -- src/problem.jl:11-111
* Diffusion module                                         -- src/diffusion.jl:44-176
* parsevalsum2 / parsevalsum / jacobianh / jacobian        -- src/utils.jl:113-218
* radialspectrum                                           -- src/utils.jl:239-283
* Diagnostic / increment! / update! / extend!              -- src/diagnostics.jl:8-116

The reference's FFT is FFTW.jl (compat "1", Project.toml:25; no Manifest, so the exact
version is unpinned) on the CPU and CUFFT through CUDA.jl on the GPU.  Both compute the
unnormalised forward DFT with sign -1 and a 1/N-normalised inverse; here that DFT is
restated with scipy.fft (pocketfft).  Parity of this restatement is pinned by the
reference's own known-answer tests (test/createffttestfunctions.jl, test/test_grid.jl,
test/test_timesteppers.jl, test/test_utils.jl, test/test_diagnostics.jl), restated in
tests/test_oracle_pins.py.

The 2D vorticity nonlinear term is not part of FourierFlows.jl (it lives in the child
package GeophysicalFlows.jl, absent here).  ``vorticity_calcN`` defines it from the
reference's Jacobian convention (src/utils.jl:190-205): N = -J(psi, zeta), written in flux
form -(d/dx (u zeta) + d/dy (v zeta)) with psi_hat = -zeta_hat / |k|^2, the input and the
output both 2/3-dealiased.

Arrays follow Julia's shapes: a 2D real field is (nx, ny) and its rfft is (nkr, ny); index
[i, j] here is Julia's [i+1, j+1].  Alias ranges are stored 0-based half-open.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np
import scipy.fft as sfft

WORKERS = 1  # scipy.fft worker threads; the CPU baseline raises this to all host cores


def set_workers(n: int) -> None:
    global WORKERS
    WORKERS = max(1, int(n))


# ----------------------------------------------------------------------------------------
# FFT restatement (FFTW semantics: forward unnormalised e^{-ikx}, inverse normalised)
# ----------------------------------------------------------------------------------------

def rfft(a):
    """rfft over every dimension, real transform along dim 1 (Julia's x) first."""
    axes = tuple(reversed(range(a.ndim)))
    return sfft.rfftn(a, axes=axes, workers=WORKERS)


def irfft(ah, nx):
    """Normalised inverse of ``rfft``; ``nx`` is the length of the real first dimension."""
    shape = (nx,) + ah.shape[1:]
    axes = tuple(reversed(range(ah.ndim)))
    s = tuple(shape[ax] for ax in axes)
    return sfft.irfftn(ah, s=s, axes=axes, workers=WORKERS)


def fft(a):
    return sfft.fftn(a, workers=WORKERS)


def ifft(ah):
    return sfft.ifftn(ah, workers=WORKERS)


def rfft_dims(a, ndim):
    """rfft over the first ``ndim`` dims only (trailing dims are fields/batch)."""
    axes = tuple(reversed(range(ndim)))
    return sfft.rfftn(a, axes=axes, workers=WORKERS)


def irfft_dims(ah, nx, ndim):
    axes = tuple(reversed(range(ndim)))
    shape = (nx,) + ah.shape[1:]
    s = tuple(shape[ax] for ax in axes)
    return sfft.irfftn(ah, s=s, axes=axes, workers=WORKERS)


# ----------------------------------------------------------------------------------------
# Grids -- src/domains.jl
# ----------------------------------------------------------------------------------------

def fftfreq(n, fs):
    """AbstractFFTs.fftfreq(n, fs): (0..n/2-1, -n/2..-1) * fs/n."""
    mult = fs / n
    i = np.arange(n)
    idx = np.where(i < (n + 1) // 2, i, i - n)
    return idx * mult


def rfftfreq(n, fs):
    mult = fs / n
    return np.arange(n // 2 + 1) * mult


def julia_range(x0, dx, n, T):
    """range(T(x0), step=T(dx), length=n): each point rounded from the exact sum."""
    x0t = T(x0)
    dxt = T(dx)
    f0, fd = Fraction(float(x0t)), Fraction(float(dxt))
    return np.array([T(float(f0 + i * fd)) for i in range(n)], dtype=T)


def getaliasedwavenumbers(nk, nkr, aliased_fraction):
    """src/domains.jl:408-421, returned 0-based half-open: (lo, hi) pairs or None."""
    L = (1 - aliased_fraction) / 2
    R = (1 + aliased_fraction) / 2
    iL = math.floor(L * nk) + 1
    iR = math.ceil(R * nk)
    if not aliased_fraction < 1:
        raise ValueError("`aliased_fraction` must be less than 1")
    if aliased_fraction > 0:
        return (iL - 1, iR), (iL - 1, nkr)
    return None, None


class Grid:
    """OneDGrid / TwoDGrid / ThreeDGrid restated (src/domains.jl:61-101,175-223,311-366)."""

    def __init__(self, ndim, n, L, x0=None, T=np.float64, aliased_fraction=1 / 3):
        n = tuple(int(v) for v in n)
        L = tuple(float(v) for v in L)
        if any(v % 2 != 0 for v in n):
            raise ValueError("DomainError: grid sizes must be even")
        self.ndim, self.T = ndim, T
        self.n, self.L = n, L
        self.nx = n[0]
        self.Lx = T(L[0])
        self.nk = n[0]
        self.nkr = n[0] // 2 + 1
        self.dx = T(L[0] / n[0])
        x0 = x0 if x0 is not None else tuple(-v / 2 for v in L)
        self.x = julia_range(x0[0], L[0] / n[0], n[0], T)
        shape_k = [1] * ndim
        shape_k[0] = n[0]
        shape_kr = [1] * ndim
        shape_kr[0] = self.nkr
        self.k = fftfreq(n[0], 2 * math.pi / L[0] * n[0]).astype(T).reshape(shape_k)
        self.kr = rfftfreq(n[0], 2 * math.pi / L[0] * n[0]).astype(T).reshape(shape_kr)
        self.aliased_fraction = T(aliased_fraction)
        self.kalias, self.kralias = getaliasedwavenumbers(self.nk, self.nkr, aliased_fraction)
        self.lalias = self.malias = None
        if ndim >= 2:
            self.ny, self.Ly, self.nl = n[1], T(L[1]), n[1]
            self.dy = T(L[1] / n[1])
            self.y = julia_range(x0[1], L[1] / n[1], n[1], T)
            sl = [1] * ndim
            sl[1] = n[1]
            self.l = fftfreq(n[1], 2 * math.pi / L[1] * n[1]).astype(T).reshape(sl)
            self.lalias, _ = getaliasedwavenumbers(self.nl, self.nl // 2 + 1 if ndim == 3 else self.nl,
                                                   aliased_fraction)
        if ndim == 3:
            self.nz, self.Lz, self.nm = n[2], T(L[2]), n[2]
            self.dz = T(L[2] / n[2])
            self.z = julia_range(x0[2], L[2] / n[2], n[2], T)
            sm = [1, 1, n[2]]
            self.m = fftfreq(n[2], 2 * math.pi / L[2] * n[2]).astype(T).reshape(sm)
            self.malias, _ = getaliasedwavenumbers(self.nm, self.nm // 2 + 1, aliased_fraction)
        with np.errstate(divide="ignore"):
            if ndim == 1:
                self.ksq = self.k ** 2
                self.krsq = self.kr ** 2
                self.invksq = (1 / self.ksq).astype(T)
                self.invkrsq = (1 / self.krsq).astype(T)
                self.invksq[0] = 0
                self.invkrsq[0] = 0
            else:
                if ndim == 2:
                    self.Ksq = (self.k ** 2 + self.l ** 2).astype(T)
                    self.Krsq = (self.kr ** 2 + self.l ** 2).astype(T)
                else:
                    self.Ksq = (self.k ** 2 + self.l ** 2 + self.m ** 2).astype(T)
                    self.Krsq = (self.kr ** 2 + self.l ** 2 + self.m ** 2).astype(T)
                self.invKsq = (1 / self.Ksq).astype(T)
                self.invKrsq = (1 / self.Krsq).astype(T)
                self.invKsq.flat[0] = 0
                self.invKrsq.flat[0] = 0

    @property
    def spectral_shape(self):
        return (self.nkr,) + self.n[1:]


def OneDGrid(nx, Lx, x0=None, T=np.float64, aliased_fraction=1 / 3):
    return Grid(1, (nx,), (Lx,), None if x0 is None else (x0,), T, aliased_fraction)


def TwoDGrid(nx, Lx, ny=None, Ly=None, T=np.float64, aliased_fraction=1 / 3):
    ny = nx if ny is None else ny
    Ly = Lx if Ly is None else Ly
    return Grid(2, (nx, ny), (Lx, Ly), None, T, aliased_fraction)


def ThreeDGrid(nx, Lx, ny=None, Ly=None, nz=None, Lz=None, T=np.float64, aliased_fraction=1 / 3):
    ny = nx if ny is None else ny
    Ly = Lx if Ly is None else Ly
    nz = nx if nz is None else nz
    Lz = Lx if Lz is None else Lz
    return Grid(3, (nx, ny, nz), (Lx, Ly, Lz), None, T, aliased_fraction)


def dealias(fh, g):
    """dealias!(fh, grid), src/domains.jl:428-476 (in place; returns fh)."""
    if g.kalias is None:
        return fh
    kal = g.kralias if fh.shape[0] == g.nkr else g.kalias
    fh[kal[0]:kal[1], ...] = 0
    if g.ndim >= 2:
        fh[:, g.lalias[0]:g.lalias[1], ...] = 0
    if g.ndim == 3:
        fh[:, :, g.malias[0]:g.malias[1], ...] = 0
    return fh


def makefilter_K(K, order=4, innerK=2 / 3, outerK=1, tol=1e-15):
    """makefilter(K::Array; ...), src/domains.jl:506-516 (FP64 result)."""
    K = np.asarray(K)
    decay = -math.log(tol) / (outerK - innerK) ** order
    with np.errstate(invalid="ignore", over="ignore"):
        f = np.exp(-decay * (K.astype(np.float64) - innerK) ** order)
    f[K < innerK] = 1
    return f


def makefilter(g, realvars=True, **kw):
    """src/domains.jl:520-538: K is formed in the grid's float type, the filter in FP64."""
    T = g.T
    pi = T(math.pi)
    if g.ndim == 1:
        K = g.kr * g.dx / pi if realvars else np.abs(g.k * g.dx / pi)
    elif g.ndim == 2:
        kk = g.kr if realvars else g.k
        K = np.sqrt((kk * g.dx / pi) ** 2 + (g.l * g.dy / pi) ** 2)
    else:
        kk = g.kr if realvars else g.k
        K = np.sqrt((kk * g.dx / pi) ** 2 + (g.l * g.dy / pi) ** 2 + (g.m * g.dz / pi) ** 2)
    return makefilter_K(K, **kw)


def makefilter_eq(eq, **kw):
    """makefilter(eq) = ones(T, dims) .* makefilter(grid; realvars=dims[1]==nkr), :540-541."""
    f = makefilter(eq.grid, realvars=eq.dims[0] == eq.grid.nkr, **kw)
    return np.ones(eq.dims) * f.reshape(f.shape + (1,) * (len(eq.dims) - f.ndim))


# ----------------------------------------------------------------------------------------
# Problem model -- src/problem.jl
# ----------------------------------------------------------------------------------------

class Equation:
    def __init__(self, L, calcN, grid, dims=None, T=None):
        self.L = L
        self.calcN = calcN
        self.grid = grid
        self.dims = tuple(dims) if dims is not None else tuple(np.shape(L))
        self.T = T if T is not None else (np.complex64 if grid.T == np.float32 else np.complex128)


class Clock:
    def __init__(self, dt, t, step, T=np.float64):
        self.T = T
        self.dt = T(dt)
        self.t = T(t)
        self.step = int(step)


class Problem:
    def __init__(self, eqn, stepper, dt, grid, vars=None, params=None, **stepperkw):
        self.eqn, self.grid, self.vars, self.params = eqn, grid, vars, params
        self.clock = Clock(dt, 0, 0, grid.T)
        self.timestepper = TimeStepper(stepper, eqn, dt, **stepperkw)
        self.sol = np.zeros(eqn.dims, dtype=eqn.T)


# ----------------------------------------------------------------------------------------
# Time steppers -- src/timesteppers.jl
# ----------------------------------------------------------------------------------------

FULLY_EXPLICIT = ["ForwardEuler", "RK4", "AB3", "LSRK54", "FilteredForwardEuler", "FilteredRK4",
                  "FilteredAB3", "FilteredLSRK54"]


def isexplicit(stepper):
    return stepper in FULLY_EXPLICIT


def _fl(eqT):
    return np.float32 if np.dtype(eqT) == np.complex64 else np.float64


def getexpLs(dt, eq):
    """src/timesteppers.jl:673-678, in L's type (dt already converted to fltype(T))."""
    L = np.asarray(eq.L)
    Tl = L.dtype if L.dtype.kind in "fc" else np.dtype(type(dt))
    dtL = (dt * L).astype(Tl) if L.ndim else Tl.type(dt * L)
    with np.errstate(over="ignore"):
        return np.exp(dtL), np.exp(dtL / Tl.type(2))


def getetdcoeffs(dt, L, ncirc=32, rcirc=1):
    """Kassam-Trefethen contour means, src/timesteppers.jl:689-718 (always FP64)."""
    L = np.asarray(L)
    circ = rcirc * np.exp(2j * math.pi / ncirc * (np.arange(ncirc) + 0.5))
    dtL = dt * L
    if L.dtype.kind in "fc":
        dtL = dtL.astype(L.dtype)
    zc = np.asarray(dtL)[..., None].astype(np.complex128) + circ
    ez = np.exp(zc)
    ez2 = np.exp(zc / 2)
    zeta_c = (ez2 - 1) / zc
    alpha_c = (-4 - zc + ez * (4 - 3 * zc + zc ** 2)) / zc ** 3
    beta_c = (2 + zc + ez * (-2 + zc)) / zc ** 3
    gamma_c = (-4 - 3 * zc - zc ** 2 + ez * (4 - zc)) / zc ** 3
    dt64 = np.float64(dt)
    out = [dt64 * c.mean(axis=-1) for c in (zeta_c, alpha_c, beta_c, gamma_c)]
    if L.dtype.kind != "c":
        out = [np.real(c) for c in out]
    return tuple(out)


class _TS:
    pass


def TimeStepper(stepper, eq, dt=None, **kw):
    """String-dispatched constructor, src/timesteppers.jl:57-69."""
    ts = _TS()
    ts.name = stepper + "TimeStepper"
    ts.kind = stepper.replace("Filtered", "")
    ts.filtered = stepper.startswith("Filtered")
    z = lambda: np.zeros(eq.dims, dtype=eq.T)
    if ts.kind == "ForwardEuler":
        ts.N = z()
    elif ts.kind == "RK4":
        ts.sol1, ts.RHS1, ts.RHS2, ts.RHS3, ts.RHS4 = z(), z(), z(), z(), z()
    elif ts.kind == "LSRK54":
        ts.S2, ts.RHS = z(), z()
        T = _fl(eq.T)
        A = [Fraction(0), Fraction(-567301805773, 1357537059087), Fraction(-2404267990393, 2016746695238),
             Fraction(-3550918686646, 2091501179385), Fraction(-1275806237668, 842570457699)]
        B = [Fraction(1432997174477, 9575080441755), Fraction(5161836677717, 13612068292357),
             Fraction(1720146321549, 2090206949498), Fraction(3134564353537, 4481467310338),
             Fraction(2277821191437, 14882151754819)]
        C = [Fraction(0), Fraction(1432997174477, 9575080441755), Fraction(2526269341429, 6820363962896),
             Fraction(2006345519317, 3224310063776), Fraction(2802321613138, 2924317926251)]
        ts.A = [T(float(a)) for a in A]
        ts.B = [T(float(b)) for b in B]
        ts.C = [T(float(c)) for c in C]
    elif ts.kind == "ETDRK4":
        dtT = _fl(eq.T)(dt)
        ts.expLdt, ts.exp_half_Ldt = getexpLs(dtT, eq)
        ts.zeta, ts.alpha, ts.beta, ts.Gamma = getetdcoeffs(dtT, eq.L)
        ts.sol1, ts.sol2, ts.N1, ts.N2, ts.N3, ts.N4 = z(), z(), z(), z(), z(), z()
    elif ts.kind == "AB3":
        ts.RHS, ts.RHSm1, ts.RHSm2 = z(), z(), z()
    else:
        raise ValueError(f"unknown stepper {stepper}")
    if ts.filtered:
        ts.filter = makefilter_eq(eq, **kw)
    return ts


def _cast(a, T):
    return np.asarray(a).astype(T, copy=False)


def stepforward(prob, nsteps=1, diags=None):
    for _ in range(nsteps):
        _step(prob.sol, prob.clock, prob.timestepper, prob.eqn, prob.vars, prob.params, prob.grid)
        if diags is not None:
            increment(diags)


def _step(sol, clock, ts, eq, vars, params, grid):
    T = eq.T
    L = eq.L
    dt, t = clock.dt, clock.t
    if ts.kind == "ForwardEuler":
        eq.calcN(ts.N, sol, t, clock, vars, params, grid)
        if ts.filtered:
            sol[...] = _cast(ts.filter * (sol + dt * (ts.N + L * sol)), T)
        else:
            sol += _cast(dt * (L * sol + ts.N), T)
    elif ts.kind == "RK4":
        half = dt / clock.T(2)
        eq.calcN(ts.RHS1, sol, t, clock, vars, params, grid)
        ts.RHS1 += _cast(L * sol, T)
        ts.sol1[...] = sol + half * ts.RHS1
        eq.calcN(ts.RHS2, ts.sol1, t + half, clock, vars, params, grid)
        ts.RHS2 += _cast(L * ts.sol1, T)
        ts.sol1[...] = sol + half * ts.RHS2
        eq.calcN(ts.RHS3, ts.sol1, t + half, clock, vars, params, grid)
        ts.RHS3 += _cast(L * ts.sol1, T)
        ts.sol1[...] = sol + dt * ts.RHS3
        eq.calcN(ts.RHS4, ts.sol1, t + dt, clock, vars, params, grid)
        ts.RHS4 += _cast(L * ts.sol1, T)
        sol += dt / clock.T(6) * (ts.RHS1 + 2 * ts.RHS2 + 2 * ts.RHS3 + ts.RHS4)
        if ts.filtered:
            sol[...] = _cast(sol * ts.filter, T)
    elif ts.kind == "LSRK54":
        ts.S2[...] = 0
        for i in range(5):
            eq.calcN(ts.RHS, sol, t + ts.C[i] * dt, clock, vars, params, grid)
            ts.RHS += _cast(L * sol, T)
            ts.S2[...] = ts.A[i] * ts.S2 + dt * ts.RHS
            sol += ts.B[i] * ts.S2
        if ts.filtered:
            sol[...] = _cast(sol * ts.filter, T)
    elif ts.kind == "ETDRK4":
        eq.calcN(ts.N1, sol, t, clock, vars, params, grid)
        ts.sol1[...] = _cast(ts.exp_half_Ldt * sol + ts.zeta * ts.N1, T)
        t2 = t + dt / clock.T(2)
        eq.calcN(ts.N2, ts.sol1, t2, clock, vars, params, grid)
        ts.sol2[...] = _cast(ts.exp_half_Ldt * sol + ts.zeta * ts.N2, T)
        eq.calcN(ts.N3, ts.sol2, t2, clock, vars, params, grid)
        ts.sol2[...] = _cast(ts.exp_half_Ldt * ts.sol1 + ts.zeta * (2 * ts.N3 - ts.N1), T)
        eq.calcN(ts.N4, ts.sol2, t + dt, clock, vars, params, grid)
        sol[...] = _cast(ts.expLdt * sol + ts.alpha * ts.N1 + 2 * ts.beta * (ts.N2 + ts.N3)
                         + ts.Gamma * ts.N4, T)
        if ts.filtered:
            sol[...] = _cast(sol * ts.filter, T)
    elif ts.kind == "AB3":
        eq.calcN(ts.RHS, sol, t, clock, vars, params, grid)
        ts.RHS += _cast(L * sol, T)
        if clock.step < 3:
            sol += dt * ts.RHS
        else:
            sol += _cast(dt * (23 / 12 * ts.RHS - 16 / 12 * ts.RHSm1 + 5 / 12 * ts.RHSm2), T)
        if ts.filtered:
            sol[...] = _cast(sol * ts.filter, T)
        ts.RHSm2[...] = ts.RHSm1
        ts.RHSm1[...] = ts.RHS
    clock.t = clock.T(clock.t + clock.dt)
    clock.step += 1


def step_until(prob, stop_time):
    """src/timesteppers.jl:734-760, including the t_remaining quirk of :752."""
    if prob.timestepper.kind == "ETDRK4":
        raise RuntimeError("step_until! requires fully explicit time stepper; does not work with ETDRK4")
    if not stop_time > prob.clock.t:
        raise RuntimeError("stop_time must be greater than prob.clock.t")
    dt = prob.clock.dt
    time_interval = stop_time - prob.clock.t
    nsteps = math.floor(time_interval / dt)
    stepforward(prob, nsteps)
    t_remaining = time_interval - prob.clock.t
    prob.clock.dt = prob.clock.T(t_remaining)
    stepforward(prob)
    prob.clock.dt = dt


# ----------------------------------------------------------------------------------------
# Diffusion module -- src/diffusion.jl
# ----------------------------------------------------------------------------------------

class DiffusionVars:
    def __init__(self, g):
        T = g.T
        C = np.complex64 if T == np.float32 else np.complex128
        self.c = np.zeros(g.nx, T)
        self.cx = np.zeros(g.nx, T)
        self.ch = np.zeros(g.nkr, C)
        self.cxh = np.zeros(g.nkr, C)


class DiffusionParams:
    def __init__(self, kappa):
        self.kappa = kappa


def diffusion_calcN(N, sol, t, clock, vars, params, grid):
    """src/diffusion.jl:129-143."""
    if np.ndim(params.kappa) == 0:
        N[...] = 0
        return
    kr = grid.kr.reshape(-1)
    vars.cxh[...] = 1j * kr * sol
    vars.cx[...] = irfft(vars.cxh, grid.nx)
    vars.cx *= params.kappa
    vars.cxh[...] = rfft(vars.cx)
    N[...] = 1j * kr * vars.cxh


def DiffusionProblem(nx=128, Lx=2 * math.pi, kappa=0, dt=0.01, stepper="RK4", aliased_fraction=0,
                     T=np.float64):
    """src/diffusion.jl:44-59 (OneDGrid)."""
    g = OneDGrid(nx, Lx, T=T, aliased_fraction=aliased_fraction)
    params = DiffusionParams(np.asarray(kappa, dtype=np.float64) if np.ndim(kappa) else kappa)
    vars = DiffusionVars(g)
    if np.ndim(kappa) == 0:
        L = (-kappa * g.kr.reshape(-1) ** 2).astype(T)
        eq = Equation(L, diffusion_calcN, g)
    else:
        eq = Equation(0, diffusion_calcN, g, dims=(g.nkr,),
                      T=np.complex64 if T == np.float32 else np.complex128)
    return Problem(eq, stepper, dt, g, vars, params)


def diffusion_updatevars(prob):
    """src/diffusion.jl:150-160."""
    v, g, sol = prob.vars, prob.grid, prob.sol
    v.ch[...] = sol
    v.cxh[...] = 1j * g.kr.reshape(-1) * sol
    v.c[...] = irfft(v.ch.copy(), g.nx)
    v.cx[...] = irfft(v.cxh.copy(), g.nx)


def diffusion_set_c(prob, c):
    """src/diffusion.jl:167-176."""
    prob.vars.c[...] = c
    prob.sol[...] = rfft(prob.vars.c)
    diffusion_updatevars(prob)


def Diffusion3DProblem(n, L, kappa, dt, stepper="ETDRK4", T=np.float64):
    """Constant-kappa diffusion on a ThreeDGrid: L = -kappa * Krsq, N = 0."""
    g = ThreeDGrid(n, L, T=T, aliased_fraction=0)
    Lop = (-kappa * g.Krsq).astype(T)
    eq = Equation(Lop, lambda N, *a: N.__setitem__(Ellipsis, 0), g)
    return Problem(eq, stepper, dt, g)


# ----------------------------------------------------------------------------------------
# Utilities -- src/utils.jl
# ----------------------------------------------------------------------------------------

def parsevalsum2(uh, g):
    """src/utils.jl:113-139."""
    if g.ndim == 2:
        norm = g.Lx * g.Ly / (g.nx ** 2 * g.ny ** 2)
    elif g.ndim == 1:
        norm = g.Lx / g.nx ** 2
    else:
        raise NotImplementedError("parsevalsum2 is defined for OneDGrid and TwoDGrid")
    a2 = np.abs(uh) ** 2
    if uh.shape[0] == g.nkr:
        s = a2[0].sum() + a2[g.nkr - 1].sum() + 2 * a2[1:g.nkr - 1].sum()
    else:
        s = a2.sum()
    return float(s * norm)


def parsevalsum(uh, g):
    """src/utils.jl:157-183."""
    if g.ndim == 2:
        norm = g.Lx * g.Ly / (g.nx ** 2 * g.ny ** 2)
    else:
        norm = g.Lx / g.nx ** 2
    if uh.shape[0] == g.nkr:
        s = uh[0].sum() + uh[g.nkr - 1].sum() + 2 * uh[1:g.nkr - 1].sum()
    else:
        s = uh.sum()
    return float(np.real(s * norm))


def jacobianh(a, b, g):
    """src/utils.jl:190-205."""
    if np.isrealobj(a):
        bh = rfft(b)
        bx = irfft(1j * g.kr * bh, g.nx)
        by = irfft(1j * g.l * bh, g.nx)
        return 1j * g.kr * rfft(a * by) - 1j * g.l * rfft(a * bx)
    bh = fft(b)
    bx = ifft(1j * g.k * bh)
    by = ifft(1j * g.l * bh)
    return 1j * g.k * fft(a * by) - 1j * g.l * fft(a * bx)


def jacobian(a, b, g):
    """src/utils.jl:212-218."""
    if np.isrealobj(a):
        return irfft(jacobianh(a, b, g), g.nx)
    return ifft(jacobianh(a, b, g))


def _lin_interp_index(x, x0, dx, n):
    """0-based lower index and weight of linear interpolation on the uniform grid
    x0 + i dx, i = 0..n-1 (Interpolations.jl's scaled BSpline(Linear()) inside its range)."""
    u = (x - x0) / dx
    i = np.clip(np.floor(u).astype(np.int64), 0, n - 2)
    return i, u - i


def radialspectrum(fh, g, n=None, m=None, refinement=2):
    """src/utils.jl:239-283: fh (rfft form (nkr, nl) or full form (nk, nl)) bilinearly
    interpolated from its fftshifted layout onto a polar (rho, theta) grid and integrated
    over theta: fhr = [2] rho sum_theta fh(rho, theta) dtheta, fhr[0] = fh[0, 0].
    Returns (rho, fhr)."""
    n = refinement * max(g.nk, g.nl) if n is None else n
    m = refinement * max(g.nk, g.nl) if m is None else m
    lshift = np.linspace(-g.nl / 2, g.nl / 2 - 1, g.nl) * 2 * np.pi / g.Ly
    if fh.shape[0] == g.nkr:
        m = m // 2
        theta = np.linspace(-np.pi / 2, np.pi / 2, m)
        fhs = np.fft.fftshift(fh, axes=1)
        kshift = np.linspace(0, g.nkr - 1, g.nkr) * 2 * np.pi / g.Lx
        fac = 2.0
    else:
        theta = np.linspace(0, 2 * np.pi, m)
        fhs = np.fft.fftshift(fh, axes=(0, 1))
        kshift = np.linspace(-g.nk / 2, g.nk / 2 - 1, g.nk) * 2 * np.pi / g.Lx
        fac = 1.0
    rhomax = min((g.nk / 2 - 1) * 2 * np.pi / g.Lx, (g.nl / 2 - 1) * 2 * np.pi / g.Ly)
    rho = np.linspace(0, rhomax, n)
    R, TH = np.meshgrid(rho[1:], theta, indexing="ij")
    i, wi = _lin_interp_index(R * np.cos(TH), kshift[0], kshift[1] - kshift[0], len(kshift))
    j, wj = _lin_interp_index(R * np.sin(TH), lshift[0], lshift[1] - lshift[0], len(lshift))
    vals = ((1 - wi) * (1 - wj) * fhs[i, j] + wi * (1 - wj) * fhs[i + 1, j] + (1 - wi) * wj * fhs[i, j + 1]
            + wi * wj * fhs[i + 1, j + 1])
    dtheta = theta[1] - theta[0]
    fhr = np.zeros(n, dtype=np.result_type(fh.dtype, np.float64))
    fhr[1:] = fac * rho[1:] * vals.sum(axis=1) * dtheta
    fhr[0] = fh[0, 0]
    return rho, fhr


# ----------------------------------------------------------------------------------------
# 2D vorticity (the nonlinear term defined for this path; not in FourierFlows.jl)
# ----------------------------------------------------------------------------------------

class VorticityParams:
    def __init__(self, nu, mu):
        self.nu, self.mu = nu, mu


def vorticity_calcN(N, sol, t, clock, vars, params, g):
    """N = -J(psi, zeta) = -(d/dx(u zeta) + d/dy(v zeta)), input and output 2/3-dealiased."""
    zh = dealias(np.array(sol, copy=True), g)
    psih = -zh * g.invKrsq
    uh = -1j * g.l * psih
    vh = 1j * g.kr * psih
    u = irfft(uh, g.nx)
    v = irfft(vh, g.nx)
    z = irfft(zh, g.nx)
    out = -(1j * g.kr * rfft(u * z) + 1j * g.l * rfft(v * z))
    N[...] = dealias(out, g).astype(N.dtype)


def vorticity_bilinear(ah, bh, g):
    """B(a, b) = -dealias(d/dx(u_a zeta_b) + d/dy(v_a zeta_b)), velocity from a, vorticity
    from b, both inputs dealiased; vorticity_calcN is B(s, s)."""
    ad = dealias(np.array(ah, copy=True), g)
    bd = dealias(np.array(bh, copy=True), g)
    psih = -ad * g.invKrsq
    u = irfft(-1j * g.l * psih, g.nx)
    v = irfft(1j * g.kr * psih, g.nx)
    z = irfft(bd, g.nx)
    return dealias(-(1j * g.kr * rfft(u * z) + 1j * g.l * rfft(v * z)), g)


def vorticity_calcN_tangent(sh, dsh, g):
    """Forward-mode tangent of the vorticity term at s along ds: B(ds, s) + B(s, ds)."""
    return vorticity_bilinear(dsh, sh, g) + vorticity_bilinear(sh, dsh, g)


def etdrk4_vorticity_tangent_step(s, ds, ts, g):
    """One ETDRK4 step (src/timesteppers.jl:501-547) of the vorticity problem and its
    tangent along ds: returns (s', ds')."""
    def N(x):
        out = np.zeros_like(x)
        vorticity_calcN(out, x, 0.0, None, None, None, g)
        return out

    E, E2, Z, al, be, ga = ts.expLdt, ts.exp_half_Ldt, ts.zeta, ts.alpha, ts.beta, ts.Gamma
    N1 = N(s)
    dN1 = vorticity_calcN_tangent(s, ds, g)
    a, da = E2 * s + Z * N1, E2 * ds + Z * dN1
    N2, dN2 = N(a), vorticity_calcN_tangent(a, da, g)
    b, db = E2 * s + Z * N2, E2 * ds + Z * dN2
    N3, dN3 = N(b), vorticity_calcN_tangent(b, db, g)
    c, dc = E2 * a + Z * (2 * N3 - N1), E2 * da + Z * (2 * dN3 - dN1)
    N4, dN4 = N(c), vorticity_calcN_tangent(c, dc, g)
    s2 = E * s + al * N1 + 2 * be * (N2 + N3) + ga * N4
    ds2 = E * ds + al * dN1 + 2 * be * (dN2 + dN3) + ga * dN4
    return s2, ds2


def VorticityProblem(n, L, nu, mu, dt, stepper="ETDRK4", T=np.float64, aliased_fraction=1 / 3, **kw):
    g = TwoDGrid(n, L, T=T, aliased_fraction=aliased_fraction)
    Lop = (-nu * g.Krsq - mu).astype(T)
    eq = Equation(Lop, vorticity_calcN, g)
    return Problem(eq, stepper, dt, g, None, VorticityParams(nu, mu), **kw)


def vorticity_energy(zh, g):
    """E = 1/2 <|grad psi|^2> (domain average)."""
    return 0.5 * parsevalsum2(zh * np.sqrt(g.invKrsq), g) / (g.Lx * g.Ly)


def vorticity_enstrophy(zh, g):
    """Z = 1/2 <zeta^2> (domain average)."""
    return 0.5 * parsevalsum2(zh, g) / (g.Lx * g.Ly)


# ----------------------------------------------------------------------------------------
# Diagnostics -- src/diagnostics.jl
# ----------------------------------------------------------------------------------------

class Diagnostic:
    def __init__(self, calc, prob, freq=1, nsteps=100, ndata=None):
        ndata = ndata if ndata is not None else math.ceil((nsteps + 1) / freq)
        self.calc, self.prob, self.freq = calc, prob, freq
        self.data = [None] * ndata
        self.t = [0.0] * ndata
        self.steps = [0] * ndata
        self.data[0] = calc(prob)
        self.t[0] = float(prob.clock.t)
        self.steps[0] = prob.clock.step
        self.i = 1  # number of stored samples
        self.N = ndata

    def update(self):
        if self.i >= len(self.steps):
            self.data += [None] * self.N
            self.t += [0.0] * self.N
            self.steps += [0] * self.N
        self.data[self.i] = self.calc(self.prob)
        self.t[self.i] = float(self.prob.clock.t)
        self.steps[self.i] = self.prob.clock.step
        self.i += 1


def increment(diags):
    if isinstance(diags, (list, tuple)):
        for d in diags:
            increment(d)
        return
    if diags.prob.clock.step % diags.freq == 0:
        diags.update()
