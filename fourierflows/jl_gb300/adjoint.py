"""Discrete adjoint of the 2D vorticity ETDRK4 step, with checkpointing.

``rrule_stepforward(prob, nsteps)`` is the analogue of a ChainRulesCore ``rrule`` for
``stepforward!(prob, nsteps)`` on a vorticity ETDRK4 problem: it advances the problem
(saving every ``checkpoint_every``-th state) and returns a pullback that maps the
gradient with respect to the final state to the gradients with respect to the initial
state and to the viscosity nu.

Gradients are taken with respect to the stored half spectrum read as a real vector of
its real and imaginary parts (inner product sum Re(conj(a) b)), the exact transpose of
the map the library computes; ``VorticityAdjoint.gradient`` converts the initial-state
gradient to one with respect to the physical initial field (F^T = nx ny irfft(. / w)).

The backward sweep recomputes each segment between checkpoints forward with the fused
stepper, then for every step recomputes the substep states a, b, c and N1..N4 with the
native calcN! and applies, in reverse order (src/timesteppers.jl:501-547 transposed):

    lam_s = E lam,  lam_N1 = alpha lam,  lam_N2 = lam_N3 = 2 beta lam,  lam_N4 = Gamma lam
    lam_c = J(c)^T lam_N4;  lam_a = E2 lam_c;  lam_N3 += 2 Z lam_c;  lam_N1 -= Z lam_c
    lam_b = J(b)^T lam_N3;  lam_s += E2 lam_b;  lam_N2 += Z lam_b
    lam_a += J(a)^T lam_N2;  lam_s += E2 lam_a;  lam_N1 += Z lam_a
    lam_s += J(s)^T lam_N1

with E = exp(L dt), E2 = exp(L dt/2), Z = zeta.  The viscosity gradient adds, per step,
the coefficient derivatives contracted with these adjoints (ff_vort_adj_nu_terms, FP64).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from . import vorticity as V
from .devices import GPU, device_array, fltype, prec_of, ptr, stream_handle, to_numpy, zeros
from .plans import ldiv_
from .timesteppers import ETDRK4TimeStepper, _coef


def etd_coefficient_derivatives(dt, L, dLdnu, ncirc=32, rcirc=1):
    """d/dnu of (expLdt, exp_half_Ldt, zeta, alpha, beta, Gamma) for L(nu), host FP64.

    With w_j = dt L + r exp(2 pi i (j + 1/2)/M) each contour coefficient is
    C = dt mean_j f(w_j), so dC/dnu = dt mean_j f'(w_j) dt dL/dnu, with the derivatives of
    the Kassam-Trefethen integrands f = (e^{w/2} - 1)/w and p(w)/w^3."""
    dtL = np.asarray(dt * L, dtype=np.float64)
    zp = np.asarray(dt * dLdnu, dtype=np.float64)
    circ = rcirc * np.exp(2j * math.pi / ncirc * (np.arange(ncirc) + 0.5))
    w = dtL[..., None].astype(np.complex128) + circ
    ew, ew2 = np.exp(w), np.exp(w / 2)
    fz = (0.5 * ew2 * w - (ew2 - 1)) / w ** 2
    pa = -4 - w + ew * (4 - 3 * w + w ** 2)
    pa1 = -1 + ew * (1 - w + w ** 2)
    pb = 2 + w + ew * (-2 + w)
    pb1 = 1 + ew * (-1 + w)
    pg = -4 - 3 * w - w ** 2 + ew * (4 - w)
    pg1 = -3 - 2 * w + ew * (3 - w)
    fa = pa1 / w ** 3 - 3 * pa / w ** 4
    fb = pb1 / w ** 3 - 3 * pb / w ** 4
    fg = pg1 / w ** 3 - 3 * pg / w ** 4
    d = [float(dt) * np.real(f.mean(axis=-1)) * zp for f in (fz, fa, fb, fg)]
    dE = np.exp(dtL) * zp
    dE2 = 0.5 * np.exp(dtL / 2) * zp
    return dE, dE2, d[0], d[1], d[2], d[3]


class VorticityAdjoint:
    """Adjoint machinery for one vorticity ETDRK4 problem (``vorticity.Problem``)."""

    def __init__(self, prob, checkpoint_every=50, graph=True):
        ts = prob.timestepper
        if not isinstance(ts, ETDRK4TimeStepper) or ts._filtered:
            raise NotImplementedError("the adjoint is implemented for the (unfiltered) ETDRK4 stepper")
        if not isinstance(prob.eqn.calcN, V.VorticityCalcN):
            raise NotImplementedError("the adjoint needs the native vorticity calcN!")
        self.prob, self.ts, self.K = prob, ts, int(checkpoint_every)
        g = prob.grid
        self.grid = g
        self.T = g.T
        dev = GPU()
        Ct = np.complex64 if self.T == np.float32 else np.complex128
        self.shape = (g.nkr, g.ny)
        self.n = g.nkr * g.ny
        self.prec = prec_of(prob.sol.dtype)
        self._h = C.c_void_p()
        nkd = g.kralias.start if g.kralias is not None else g.nkr
        la, lb = (g.lalias.start, g.lalias.stop) if g.lalias is not None else (0, 0)
        _lib.call("ff_vadj_create", self.prec, g.nx, g.ny, nkd, la, lb, ptr(g.kr), ptr(g.l), ptr(g.invKrsq),
                  C.byref(self._h))
        up = device_array(dev)
        Zh = to_numpy(ts.zeta)
        self.negZ = up((-Zh).astype(self.T))
        nu = prob.params.ν
        Krsq = g.Krsq_host.astype(np.float64)
        L = to_numpy(prob.eqn.L).astype(np.float64)
        derivs = etd_coefficient_derivatives(ts.dt, L, -Krsq)
        self.dE, self.dE2, self.dZ, self.dA, self.dB, self.dG = (up(x.astype(self.T)) for x in derivs)
        w = np.full(self.shape, 2.0)
        w[0, :] = 1.0
        w[-1, :] = 1.0
        self.w = w
        nxy = g.nx * g.ny
        self.c1, self.c2 = 1.0 / nxy ** 2, 0.5 / nxy ** 2
        self.W1 = up((2 * (self.c1 + self.c2) * w).astype(self.T))
        self.W2 = up((-2 * self.c1 * w).astype(self.T))
        self.Nw = up((nxy / w).astype(self.T))
        names = ("s", "a", "b", "c", "N1", "N2", "N3", "N4", "lam", "lam2", "lam_a", "lam_b", "lam_c", "lN1", "lN2",
                 "lN3", "lN4", "tmp")
        self.buf = {k: zeros(dev, Ct, self.shape) for k in names}
        import torch
        self.nu_acc = torch.zeros(1, dtype=torch.float64, device="cuda")
        self.checkpoints = {}
        self.nu = nu
        # the reverse step as two captured CUDA graphs (lam -> lam2 and lam2 -> lam), built
        # at the first pullback; the four calcN! of a step run from bound slots
        self.use_graph = bool(graph)
        self._graphs = None
        self._slots = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().ff_vadj_destroy(h)
            except Exception:
                pass
            self._h = None

    # ---- native building blocks -------------------------------------------------------
    def _axpby(self, out, c1, x, c2, y):
        """out = c1 x + c2 y (coefficients: scalars or real arrays), one native pass."""
        _lib.call("ff_etdrk4_substep12", self.prec, self.n, ptr(out), _coef(c1, self.n), ptr(x), _coef(c2, self.n),
                  ptr(y), stream_handle())

    def _N(self, out, x, slot=None):
        p = self.prob
        if slot is None:
            V.calcN_(out, x, 0.0, p.clock, p.vars, p.params, p.grid)
        else:
            V.calcN_._handle(p.grid, p.sol).calcN_slot(self._slots[slot])

    def _JT(self, out, s, lam):
        _lib.call("ff_vadj_apply", self._h, ptr(s), ptr(lam), ptr(out), stream_handle())

    def intermediates(self, s, bound=False):
        """a, b, c and N1..N4 of the ETDRK4 step from state s (the forward substeps); bound:
        s is buf["s"] and the calcN! run from the slots bound to these buffers."""
        B, ts, p = self.buf, self.ts, self.prec
        E2, Z = ts.exp_half_Ldt, ts.zeta
        self._N(B["N1"], s, 0 if bound else None)
        self._axpby(B["a"], E2, s, Z, B["N1"])
        self._N(B["N2"], B["a"], 1 if bound else None)
        self._axpby(B["b"], E2, s, Z, B["N2"])
        self._N(B["N3"], B["b"], 2 if bound else None)
        _lib.call("ff_etdrk4_substep3", p, self.n, ptr(B["c"]), _coef(E2, self.n), ptr(B["a"]), _coef(Z, self.n),
                  ptr(B["N1"]), ptr(B["N3"]), stream_handle())
        self._N(B["N4"], B["c"], 3 if bound else None)

    def adjoint_step(self, s, lam_in, lam_out, bound=False):
        """lam_out = (d step / d s)^T lam_in at state s; adds the step's viscosity terms."""
        B, ts = self.buf, self.ts
        E, E2, Z, al, be, ga = ts.expLdt, ts.exp_half_Ldt, ts.zeta, ts.alpha, ts.beta, ts.Gamma
        self.intermediates(s, bound)
        ax = self._axpby
        ax(B["lN4"], ga, lam_in, 0.0, lam_in)
        ax(B["lN1"], al, lam_in, 0.0, lam_in)
        ax(B["lN2"], be, lam_in, be, lam_in)
        ax(B["lN3"], be, lam_in, be, lam_in)
        ax(lam_out, E, lam_in, 0.0, lam_in)
        self._JT(B["lam_c"], B["c"], B["lN4"])
        ax(B["lam_a"], E2, B["lam_c"], 0.0, B["lam_c"])
        ax(B["lN3"], 1.0, B["lN3"], Z, B["lam_c"])
        ax(B["lN3"], 1.0, B["lN3"], Z, B["lam_c"])
        ax(B["lN1"], 1.0, B["lN1"], self.negZ, B["lam_c"])
        self._JT(B["lam_b"], B["b"], B["lN3"])
        ax(lam_out, 1.0, lam_out, E2, B["lam_b"])
        ax(B["lN2"], 1.0, B["lN2"], Z, B["lam_b"])
        self._JT(B["tmp"], B["a"], B["lN2"])
        ax(B["lam_a"], 1.0, B["lam_a"], 1.0, B["tmp"])
        ax(lam_out, 1.0, lam_out, E2, B["lam_a"])
        ax(B["lN1"], 1.0, B["lN1"], Z, B["lam_a"])
        args = _lib.ff_adj_nu(*[ptr(x).value for x in (lam_in, B["lam_a"], B["lam_b"], B["lam_c"], s, B["a"], B["N1"],
                                                         B["N2"], B["N3"], B["N4"], self.dE, self.dE2, self.dZ,
                                                         self.dA, self.dB, self.dG)])
        _lib.call("ff_vort_adj_nu_terms", self._h, C.byref(args), 1.0, C.c_void_p(self.nu_acc.data_ptr()),
                  stream_handle())
        self._JT(B["tmp"], s, B["lN1"])
        ax(lam_out, 1.0, lam_out, 1.0, B["tmp"])

    def _bind_slots(self):
        """Four calcN! slots of the grid's calcN! handle, bound to this object's buffers
        (slots are handed out once per handle and never rebound while a graph uses them);
        False when the handle has none left."""
        if self._slots is not None:
            return True
        p, B = self.prob, self.buf
        fs = V.calcN_._handle(p.grid, p.sol)
        first = getattr(fs, "_next_slot", 0)
        if first + 4 > _lib.FF_VORT_CALC_SLOTS:
            return False
        fs._next_slot = first + 4
        self._slots = tuple(range(first, first + 4))
        for slot, (N, x) in zip(self._slots, ((B["N1"], B["s"]), (B["N2"], B["a"]), (B["N3"], B["b"]),
                                              (B["N4"], B["c"]))):
            fs.calcN_bind(slot, N, x)
        self._slot_handle = fs  # the slots' device buffers live as long as the handle
        return True

    def _capture(self):
        """The reverse step as two CUDA graphs over fixed buffers: s = buf["s"], and lam ->
        lam2 or lam2 -> lam.  Each is run once eagerly first (lazy set-up stays out of the
        capture).  Leaves the scratch buffers and nu_acc modified."""
        import torch
        if not self._bind_slots():
            return None
        B = self.buf
        graphs = {}
        for lin, lout in (("lam", "lam2"), ("lam2", "lam")):
            self.adjoint_step(B["s"], B[lin], B[lout], bound=True)
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self.adjoint_step(B["s"], B[lin], B[lout], bound=True)
            graphs[lin] = g
        torch.cuda.synchronize()
        return graphs

    # ---- forward with checkpoints, backward sweep ---------------------------------------
    def _fused(self):
        p = self.prob
        return p.timestepper._native(p.eqn)

    def forward(self, nsteps):
        """Advance prob.sol nsteps steps, keeping every K-th state (and the initial one)."""
        p, fused = self.prob, self._fused()
        self.checkpoints = {0: p.sol.clone()}
        done = 0
        while done < nsteps:
            k = min(self.K, nsteps - done)
            fused.advance(p.sol, p.clock, k)
            done += k
            if done < nsteps:
                self.checkpoints[done] = p.sol.clone()
        for _ in range(nsteps):  # the clock arithmetic of stepforward!
            p.clock.t = p.clock.t + p.clock.dt
            p.clock.step += 1
        self.nsteps = nsteps
        self.final = p.sol.clone()
        return p.sol

    def loss(self, target_hat):
        """mean((zeta - zeta_target)^2) + 1/2 mean(zeta^2) of prob.sol (domain means, FP64)."""
        B = self.buf
        self._axpby(B["tmp"], 1.0, self.prob.sol, -1.0, target_hat)
        g = self.grid
        area = float(g.Lx) * float(g.Ly)
        from .utils import parsevalsum2
        return parsevalsum2(B["tmp"], g) / area + 0.5 * parsevalsum2(self.prob.sol, g) / area

    def loss_gradient(self, target_hat, out):
        """d loss / d sol (real-vector gradient of the half spectrum) into `out`."""
        self._axpby(out, self.W1, self.prob.sol, self.W2, target_hat)

    def pullback(self, lam_T):
        """Gradient at the initial state and d/dnu, given the gradient at the final state;
        forward() must have run."""
        p, fused, B = self.prob, self._fused(), self.buf
        if self.use_graph and self._graphs is None:
            self._graphs = self._capture() or False
        graphs = self._graphs or None
        self.nu_acc.zero_()
        lam = B["lam"]
        lam.copy_(lam_T)
        other = B["lam2"]
        starts = sorted(self.checkpoints)
        for si in reversed(range(len(starts))):
            st = starts[si]
            en = starts[si + 1] if si + 1 < len(starts) else self.nsteps
            # recompute the segment's states from its checkpoint (the fused stepper
            # advances prob.sol in place)
            states = [self.checkpoints[st]]
            p.sol.copy_(self.checkpoints[st])
            for _ in range(en - st - 1):
                fused.advance(p.sol, p.clock, 1)
                states.append(p.sol.clone())
            for s in reversed(states):
                if graphs is not None:
                    B["s"].copy_(s)
                    graphs["lam" if lam is B["lam"] else "lam2"].replay()
                else:
                    self.adjoint_step(s, lam, other)
                lam, other = other, lam
        p.sol.copy_(self.final)
        import torch
        torch.cuda.synchronize()
        return lam.clone(), float(self.nu_acc.item())

    def gradient(self, zeta0, target_hat, nsteps):
        """(loss, d loss/d zeta0 (physical field, device), d loss/d nu) for the problem
        started from the physical field zeta0."""
        p = self.prob
        V.set_zeta_(p, zeta0)
        p.clock.t, p.clock.step = 0, 0
        self.forward(nsteps)
        L = self.loss(target_hat)
        lamT = self.buf["lN4"]
        self.loss_gradient(target_hat, lamT)
        lam0, dnu = self.pullback(lamT.clone())
        y = self.buf["tmp"]
        self._axpby(y, self.Nw, lam0, 0.0, lam0)
        g = self.grid
        gz = zeros(GPU(), g.T, (g.nx, g.ny))
        ldiv_(gz, g.rfftplan, y)
        return L, gz, dnu


def rrule_stepforward(prob, nsteps, checkpoint_every=50):
    """Forward ``stepforward_(prob, nsteps)`` and its pullback, as a ChainRulesCore rrule:
    returns (prob.sol, pullback) with pullback(lam_T) -> (lam_0, d/dnu)."""
    adj = VorticityAdjoint(prob, checkpoint_every)
    adj.forward(nsteps)
    return prob.sol, adj.pullback
