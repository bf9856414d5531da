"""2D incompressible vorticity equation on a TwoDGrid, with a native fused nonlinear term.

    d zeta / dt = -J(psi, zeta) - nu |k|^2 zeta - mu zeta,    psi_hat = -zeta_hat / |k|^2

The nonlinear term is not part of FourierFlows.jl (its physics modules live in the child
package GeophysicalFlows.jl).  It is defined here from the reference's Jacobian
convention J(a, b) = a_x b_y - a_y b_x (``jacobianh``, src/utils.jl:190-205), written
in flux form N = -(d/dx (u zeta) + d/dy (v zeta)), u = -psi_y, v = psi_x, with the input
and the output 2/3-dealiased (``dealias!``, src/domains.jl:428-476).

``calcN_`` is a native functor: called as ``calcN!(N, sol, t, clock, vars, params,
grid)`` it evaluates N with three fused passes (``ff_vort_calcN``); handed to the
ETDRK4 / RK4 / LSRK54 steppers (plain or Filtered) it takes over the whole step
(``ff_vort_create`` / ``ff_vort_step``), with each substep's combination fused into
the pass that produces N and the step replayed from a CUDA graph.

Energy and enstrophy are domain averages, E = 1/2 <|grad psi|^2>, Z = 1/2 <zeta^2>,
computed with ``parsevalsum2``'s half-spectrum weighting.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .devices import GPU, cxtype, device_array, fltype, on_device, prec_of, ptr, stream_handle, zeros
from .domains import TwoDGrid
from .plans import ldiv_, mul_
from .problem import AbstractParams, AbstractVars, Equation as _Equation, Problem as _Problem


class Params(AbstractParams):
    """nu (viscosity) and mu (linear drag)."""

    def __init__(self, nu, mu=0.0):
        self.ν = nu
        self.μ = mu

    @property
    def nu(self):
        return self.ν

    @property
    def mu(self):
        return self.μ


class Vars(AbstractVars):
    """zeta, u, v (physical) and zetah, uh, vh (spectral)."""

    def __init__(self, grid):
        T, dev = grid.T, grid.device
        self.zeta = zeros(dev, T, (grid.nx, grid.ny))
        self.u = zeros(dev, T, (grid.nx, grid.ny))
        self.v = zeros(dev, T, (grid.nx, grid.ny))
        self.zetah = zeros(dev, cxtype(T), (grid.nkr, grid.ny))
        self.uh = zeros(dev, cxtype(T), (grid.nkr, grid.ny))
        self.vh = zeros(dev, cxtype(T), (grid.nkr, grid.ny))


def _vort_problem_struct(grid, sol):
    q = _lib.ff_vort_problem()
    q.nx, q.ny = grid.nx, grid.ny
    q.nkd = grid.kralias.start if grid.kralias is not None else grid.nkr
    if grid.lalias is not None:
        q.la, q.lb = grid.lalias.start, grid.lalias.stop
    else:
        q.la = q.lb = 0
    q.kr, q.l, q.invKrsq = ptr(grid.kr).value, ptr(grid.l).value, ptr(grid.invKrsq).value
    q.sol = ptr(sol, "sol").value
    return q


_STEPPERS = {"ETDRK4": _lib.FF_STEP_ETDRK4, "RK4": _lib.FF_STEP_RK4, "LSRK54": _lib.FF_STEP_LSRK54}


class FusedStepper:
    """A whole-step native handle for one or more vorticity problems (ff_vort_*)."""

    def __init__(self, kind, filtered, dt, prec, structs, keepalive):
        self.kind, self.filtered = kind, filtered
        self._structs = (_lib.ff_vort_problem * len(structs))(*structs)
        self._keep = keepalive
        self._h = C.c_void_p()
        _lib.call("ff_vort_create", prec, _STEPPERS[kind], 1 if filtered else 0, float(dt), len(structs),
                  C.cast(self._structs, C.c_void_p), C.byref(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().ff_vort_destroy(h)
            except Exception:
                pass
            self._h = None

    def advance(self, nsteps=1, stream=None):
        _lib.call("ff_vort_step", self._h, int(nsteps), stream_handle(stream))

    def config(self):
        cfg = (C.c_int32 * 8)()
        _lib.call("ff_vort_config", self._h, cfg)
        keys = ("tile_a", "tile_c", "rows_b", "radix_order", "threads_a", "threads_b", "threads_c", "graph")
        out = dict(zip(keys, list(cfg)))
        split = C.c_int32()
        _lib.call("ff_vort_get_split", self._h, C.byref(split))
        out["split_c"] = split.value
        return out

    def set_config(self, tile_a, tile_c, rows_b, radix_order=0):
        _lib.call("ff_vort_set_config", self._h, tile_a, tile_c, rows_b, radix_order)

    def set_split(self, mode):
        """Pass C split by field: -1 automatic, 0 off, 1 on (see ff_vort_set_split)."""
        _lib.call("ff_vort_set_split", self._h, int(mode))

    def autotune(self, steps_per_trial=3, stream=None):
        best = C.c_double()
        _lib.call("ff_vort_autotune", self._h, int(steps_per_trial), stream_handle(stream), C.byref(best))
        return best.value

    def calcN(self, N, sol, prob=0, stream=None):
        _lib.call("ff_vort_calcN", self._h, int(prob), ptr(sol, "sol"), ptr(N, "N"), stream_handle(stream))

    def calcN_bind(self, slot, N, sol, prob=0):
        """Stage calcN!(sol) -> N of problem `prob` in a slot once (see ff_vort_calcN_bind);
        the caller keeps N and sol alive while the slot is used."""
        _lib.call("ff_vort_calcN_bind", self._h, int(slot), int(prob), ptr(sol, "sol"), ptr(N, "N"))

    def calcN_slot(self, slot, stream=None):
        """The bound calcN! of a slot: kernel launches only, safe inside a CUDA graph capture."""
        _lib.call("ff_vort_calcN_slot", self._h, int(slot), stream_handle(stream))

    def profile(self, reps=10, stream=None):
        """Average device ms of passes A, B, C (CUDA events inside the library)."""
        ms = (C.c_double * 3)()
        _lib.call("ff_vort_profile", self._h, int(reps), stream_handle(stream), ms)
        return tuple(ms)


def _stepper_struct(ts, eq, sol):
    """Fill an ff_vort_problem from a TimeStepper's buffers and coefficients (or None)."""
    from . import timesteppers as tsm
    grid = eq.grid
    q = _vort_problem_struct(grid, sol)
    n = grid.nkr * grid.ny
    keep = []

    def arr(x):
        if not on_device(x) or x.numel() != n or x.dtype.is_complex:
            return None
        keep.append(x)
        return ptr(x).value

    if isinstance(ts, tsm.ETDRK4TimeStepper):
        kind = "ETDRK4"
        bufs = [ts.sol1, ts.sol2, ts.N1, ts.N2, ts.N3]
        coefs = [arr(c) for c in (ts.expLdt, ts.exp_half_Ldt, ts.zeta, ts.alpha, ts.beta, ts.Gamma)]
    elif isinstance(ts, tsm.RK4TimeStepper):
        kind = "RK4"
        bufs = [ts.sol1, ts.RHS1, ts.RHS2, ts.RHS3]
        coefs = [arr(eq.L)]
    elif isinstance(ts, tsm.LSRK54TimeStepper):
        kind = "LSRK54"
        bufs = [ts.S2]
        coefs = [arr(eq.L)]
        for i in range(5):
            q.lsrk_A[i] = float(ts.A[i])
            q.lsrk_B[i] = float(ts.B[i])
    else:
        return None
    if any(c is None for c in coefs):
        return None
    for i, b in enumerate(bufs):
        q.buf[i] = ptr(b).value
    for i, c in enumerate(coefs):
        q.coef[i] = c
    filt = getattr(ts, "filter", None)
    if filt is not None:
        if arr(filt) is None:
            return None
        q.filter = ptr(filt).value
    keep += bufs + [sol, grid.kr, grid.l, grid.invKrsq]
    return kind, filt is not None, q, keep


class _BoundStep:
    """Adapter between a TimeStepper and its FusedStepper.

    The handle bakes in the state pointer and, for the explicit steppers, clock.dt;
    it is rebuilt when either changes (step_until! shortens the last step)."""

    def __init__(self, ts, eq):
        self.ts, self.eq = ts, eq
        self.fs = None
        self._key = None

    def ensure(self, sol, clock):
        key = (sol.data_ptr(), float(clock.dt))
        if self.fs is None or self._key != key:
            made = _stepper_struct(self.ts, self.eq, sol)
            if made is None:
                raise RuntimeError("fused vorticity step unavailable for this stepper configuration")
            kind, filtered, q, keep = made
            self.fs = FusedStepper(kind, filtered, float(clock.dt), prec_of(sol.dtype), [q], keep)
            self._key = key
        return self.fs

    def step(self, sol, clock, vars, params, grid):
        self.ensure(sol, clock).advance(1)

    def advance(self, sol, clock, nsteps):
        self.ensure(sol, clock).advance(nsteps)


class VorticityCalcN:
    """Native N = -J(psi, zeta) with 2/3 dealiasing; see the module docstring."""
    __name__ = "calcN!"

    def _handle(self, grid, sol):
        # the handle lives on the grid (same lifetime as the arrays it points to), one per
        # precision; never keyed by id(), which a later grid can reuse
        if tuple(sol.shape) != (grid.nkr, grid.ny):
            raise ValueError(f"calcN!: state of size {tuple(sol.shape)} on a {grid.nx} x {grid.ny} grid")
        handles = grid.__dict__.setdefault("_vort_calcN_handles", {})
        key = str(sol.dtype)
        fs = handles.get(key)
        if fs is None:
            q = _vort_problem_struct(grid, sol)
            scratch = zeros(grid.device, cxtype(grid.T), (grid.nkr, grid.ny))
            n = grid.nkr * grid.ny
            coefs = [grid.invKrsq] * 6  # placeholders: the bare calcN! never reads them
            for i in range(5):
                q.buf[i] = ptr(scratch).value
            for i in range(6):
                q.coef[i] = ptr(coefs[i]).value
            q.sol = ptr(scratch).value
            fs = FusedStepper("ETDRK4", False, 0.0, prec_of(sol.dtype), [q],
                              [scratch, grid.kr, grid.l, grid.invKrsq])
            handles[key] = fs
        return fs

    def __call__(self, N, sol, t, clock, vars, params, grid):
        self._handle(grid, sol).calcN(N, sol)
        return None

    def fused_stepper(self, ts, eq):
        """A whole-step native path for ``ts``, or None (then ``ts`` runs its generic
        substeps around this functor)."""
        from . import timesteppers as tsm
        g = eq.grid
        if not isinstance(g, TwoDGrid) or not isinstance(g.device, GPU):
            return None
        if not isinstance(ts, (tsm.ETDRK4TimeStepper, tsm.RK4TimeStepper, tsm.LSRK54TimeStepper)):
            return None
        n = g.nkr * g.ny
        if tuple(eq.dims) != (g.nkr, g.ny):
            return None

        def real_arr(x):
            return on_device(x) and x.numel() == n and not x.dtype.is_complex

        if isinstance(ts, tsm.ETDRK4TimeStepper):
            coefs = (ts.expLdt, ts.exp_half_Ldt, ts.zeta, ts.alpha, ts.beta, ts.Gamma)
        else:
            coefs = (eq.L,)
        if not all(real_arr(c) for c in coefs):
            return None
        if getattr(ts, "filter", None) is not None and not real_arr(ts.filter):
            return None
        return _BoundStep(ts, eq)


calcN_ = VorticityCalcN()


def Equation(params, grid):
    """L = -nu |k|^2 - mu on the rfft half spectrum, N = calcN_."""
    Krsq = grid.Krsq_host.astype(np.float64)
    L = (-params.ν * Krsq - params.μ).astype(grid.T)
    return _Equation(device_array(grid.device)(L), calcN_, grid)


def Problem(dev=None, *, nx=256, Lx=2 * math.pi, ny=None, Ly=None, ν=0.0, μ=0.0, nu=None, mu=None, dt=0.01,
            stepper="ETDRK4", T=np.float64, aliased_fraction=1 / 3, **stepperkw):
    """A 2D vorticity problem; ``stepperkw`` (filter keywords) go to the time stepper."""
    dev = dev if dev is not None else GPU()
    nu = ν if nu is None else nu
    mu = μ if mu is None else mu
    grid = TwoDGrid(dev, nx=nx, Lx=Lx, ny=ny, Ly=Ly, T=T, aliased_fraction=aliased_fraction)
    params = Params(nu, mu)
    vars = Vars(grid)
    eq = Equation(params, grid)
    return _Problem(eq, stepper, dt, grid, vars, params, **stepperkw)


def set_zeta_(prob, zeta):
    """sol = rfft(zeta) for a physical vorticity field (host or device), then updatevars!."""
    g = prob.grid
    src = zeta if on_device(zeta) else device_array(g.device)(np.asarray(zeta, dtype=g.T))
    prob.vars.zeta.copy_(src.reshape(prob.vars.zeta.shape))
    mul_(prob.sol, g.rfftplan, prob.vars.zeta)
    updatevars_(prob)
    return None


def updatevars_(prob):
    """zetah = sol; uh, vh from psi; zeta, u, v by inverse transforms."""
    g, v, sol = prob.grid, prob.vars, prob.sol
    v.zetah.copy_(sol)
    _lib.call("ff_vort_velocities", prec_of(sol.dtype), g.nkr, g.ny, ptr(sol), ptr(g.kr), ptr(g.l),
              ptr(g.invKrsq), ptr(v.uh), ptr(v.vh), stream_handle())
    ldiv_(v.zeta, g.rfftplan, v.zetah)
    ldiv_(v.u, g.rfftplan, v.uh)
    ldiv_(v.v, g.rfftplan, v.vh)
    return None


def _weighted(zh, grid, wt):
    out = C.c_double()
    norm = float(grid.Lx) * float(grid.Ly) / (grid.nx ** 2 * grid.ny ** 2)
    _lib.call("ff_parsevalsum2_weighted", prec_of(zh.dtype), ptr(zh), None if wt is None else ptr(wt), zh.shape[0],
              zh.numel() // zh.shape[0], 1 if zh.shape[0] == grid.nkr else 0, norm, C.byref(out), None,
              stream_handle())
    return out.value


def energy(prob):
    """E = 1/2 parsevalsum2(zeta_hat sqrt(invKrsq)) / (Lx Ly)."""
    g = prob.grid
    return 0.5 * _weighted(prob.sol, g, g.invKrsq) / (float(g.Lx) * float(g.Ly))


def enstrophy(prob):
    """Z = 1/2 parsevalsum2(zeta_hat) / (Lx Ly)."""
    g = prob.grid
    return 0.5 * _weighted(prob.sol, g, None) / (float(g.Lx) * float(g.Ly))


# ----------------------------------------------------------------------------------------
# initial conditions
# ----------------------------------------------------------------------------------------
def _splitmix64(x):
    """SplitMix64 finaliser on uint64 numpy arrays (Steele, Lea & Flood 2014)."""
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    return z ^ (z >> np.uint64(31))


def uniform01(seed, n):
    """n counter-based uniforms in [0, 1) from (seed, counter): identical on every host."""
    with np.errstate(over="ignore"):
        ctr = np.arange(n, dtype=np.uint64) + (np.uint64(seed) << np.uint64(32))
        bits = _splitmix64(ctr) >> np.uint64(11)
    return bits.astype(np.float64) * (1.0 / 9007199254740992.0)


def random_phase_vorticity(nx, ny=None, Lx=2 * math.pi, Ly=None, seed=1234, k0=6.0, E0=0.5, aliased_fraction=1 / 3):
    """A physical FP64 vorticity field (nx, ny) with random phases (uniform on [0, 2pi),
    counter-based from ``seed``) and isotropic energy spectrum E(k) ~ k^4 exp(-2 (k/k0)^2),
    2/3-dealiased and scaled to total energy E0 (domain-averaged 1/2 |u|^2)."""
    ny = nx if ny is None else ny
    Ly = Lx if Ly is None else Ly
    nkr = nx // 2 + 1
    kr = np.arange(nkr) * (2 * math.pi / Lx)
    lidx = np.where(np.arange(ny) < (ny + 1) // 2, np.arange(ny), np.arange(ny) - ny)
    l = lidx * (2 * math.pi / Ly)
    K = np.sqrt(kr[:, None] ** 2 + l[None, :] ** 2)
    # |zeta_hat|^2 ~ E(K) K / (2 pi): energy per mode |psi_hat|^2 K^2 = |zeta_hat|^2 / K^2
    amp = np.sqrt(K ** 5 * np.exp(-2.0 * (K / k0) ** 2))
    amp[0, 0] = 0.0
    phase = 2 * math.pi * uniform01(seed, nkr * ny).reshape(ny, nkr).T
    zh = amp * np.exp(1j * phase)
    # 2/3 mask (same ranges as the grids)
    from .domains import getaliasedwavenumbers
    if aliased_fraction > 0:
        _, kral = getaliasedwavenumbers(nx, nkr, aliased_fraction)
        lal, _ = getaliasedwavenumbers(ny, ny, aliased_fraction)
        zh[kral.start:kral.stop, :] = 0
        zh[:, lal.start:lal.stop] = 0
    zeta = np.fft.irfft2(zh.T, s=(ny, nx)).T  # real field (nx, ny); Hermitian part enforced
    # energy of the field: E = 1/2 <|u|^2> = 1/2 sum_k |zeta_hat|^2 / K^2 (mean over the domain)
    zr = np.fft.rfft2(zeta.T).T
    with np.errstate(divide="ignore", invalid="ignore"):
        invK2 = np.where(K > 0, 1.0 / K ** 2, 0.0)
    w = np.full(nkr, 2.0)
    w[0] = 1.0
    if nx % 2 == 0:
        w[-1] = 1.0
    E = 0.5 * np.sum(w[:, None] * np.abs(zr) ** 2 * invK2) / (nx * ny) ** 2
    return np.asfortranarray(zeta * math.sqrt(E0 / E))


# ----------------------------------------------------------------------------------------
# ensembles
# ----------------------------------------------------------------------------------------
class EnsembleMember:
    """State, stepper buffers and coefficients of one ensemble problem (device arrays)."""

    def __init__(self, grid, nu, mu, dt, stepper, T, like=None):
        self.grid, self.nu, self.mu = grid, nu, mu
        Tf = np.dtype(T).type
        Ct = cxtype(T)
        shape = (grid.nkr, grid.ny)
        dev = grid.device
        self.sol = zeros(dev, Ct, shape)
        self.kind = stepper.replace("Filtered", "")
        nbuf = {"ETDRK4": 5, "RK4": 4, "LSRK54": 1}.get(self.kind)
        if nbuf is None:
            raise ValueError(f"the ensemble path supports ETDRK4, RK4 and LSRK54 (got {stepper})")
        self.bufs = [zeros(dev, Ct, shape) for _ in range(nbuf)]
        if like is not None:
            # same grid, nu, mu, dt and stepper: the read-only operator arrays are shared
            self.L, self.coefs, self.filter = like.L, like.coefs, like.filter
            return
        L = (-nu * grid.Krsq_host.astype(np.float64) - mu).astype(Tf)
        up = device_array(dev)
        self.L = up(L)
        if self.kind == "ETDRK4":
            dtT = Tf(dt)
            dtL = (dtT * L).astype(Tf)
            self.coefs = [up(np.exp(dtL).astype(Tf)), up(np.exp((dtL / Tf(2)).astype(Tf)).astype(Tf))]
            # zeta, alpha, beta, Gamma: the 32-point contour means evaluated in FP64 on the GPU
            zab = [zeros(dev, Tf, shape) for _ in range(4)]
            _lib.call("ff_etdrk4_coefficients", prec_of(self.L.dtype), self.L.numel(), ptr(self.L), float(dtT), 32,
                      1.0, ptr(zab[0]), ptr(zab[1]), ptr(zab[2]), ptr(zab[3]), stream_handle())
            self.coefs += zab
        else:
            self.coefs = [self.L]
        self.filter = None
        if stepper.startswith("Filtered"):
            from .domains import makefilter_host
            self.filter = up(makefilter_host(grid, shape, order=4, innerK=0.65).astype(Tf))


class Ensemble:
    """Independent 2D vorticity problems of (possibly) different sizes advanced together:
    every substep is three persistent launches over all members and a step is one CUDA
    graph replay.  ``members`` are (n, nu, seed) triples; grids of equal size share their
    wavenumber arrays, and members of equal size and viscosity share their operator and
    coefficient arrays (read-only).  ``value`` counters are problem-steps."""

    def __init__(self, members, mu=1e-2, dt=2e-3, stepper="ETDRK4", T=np.float32, Lx=2 * math.pi, E0=0.5,
                 k0=6.0, dev=None):
        from .timesteppers import _LSRK_A, _LSRK_B
        if len(members) == 0:
            raise ValueError("Ensemble: no members")
        dev = dev if dev is not None else GPU()
        self.T, self.dt, self.stepper = np.dtype(T).type, dt, stepper
        self.grids = {}
        self.members = []
        structs, keep = [], []
        shared = {}
        for (n, nu, seed) in members:
            g = self.grids.get(n)
            if g is None:
                g = TwoDGrid(dev, nx=n, Lx=Lx, T=T)
                self.grids[n] = g
            key = (n, float(nu))
            m = EnsembleMember(g, nu, mu, dt, stepper, T, like=shared.get(key))
            shared.setdefault(key, m)
            z0 = random_phase_vorticity(n, seed=seed, k0=k0, E0=E0)
            zd = device_array(dev)(z0.astype(self.T))
            mul_(m.sol, g.rfftplan, zd)
            m.seed = seed
            self.members.append(m)
            q = _vort_problem_struct(g, m.sol)
            for i, b in enumerate(m.bufs):
                q.buf[i] = ptr(b).value
            for i, c in enumerate(m.coefs):
                q.coef[i] = ptr(c).value
            if m.filter is not None:
                q.filter = ptr(m.filter).value
            Tf = self.T
            for i in range(5):
                q.lsrk_A[i] = float(Tf(float(_LSRK_A[i])))
                q.lsrk_B[i] = float(Tf(float(_LSRK_B[i])))
            structs.append(q)
            keep += [m, g]
        kind = stepper.replace("Filtered", "")
        self.fs = FusedStepper(kind, stepper.startswith("Filtered"), dt, prec_of(self.members[0].sol.dtype), structs,
                               keep)
        self.step = 0

    def stepforward_(self, nsteps=1, stream=None):
        self.fs.advance(nsteps, stream)
        self.step += nsteps

    @property
    def grid_points(self):
        return sum(m.grid.nx * m.grid.ny for m in self.members)

    def energies(self):
        out = []
        for m in self.members:
            g = m.grid
            out.append(0.5 * _weighted(m.sol, g, g.invKrsq) / (float(g.Lx) * float(g.Ly)))
        return out
