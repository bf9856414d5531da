"""The discrete adjoint of the vorticity ETDRK4 step: against the oracle's forward-mode
tangent (dot-product identities), against central finite differences in FP64, and the
FP32 adjoint against FP64 differences."""
import math

import numpy as np
import pytest

from oracle import ff_oracle as orc

pytestmark = pytest.mark.gpu


def redot(a, b):
    return float(np.sum(np.real(np.conj(a) * b)))


def setup(ff, n, nu=1e-3, mu=1e-2, dt=2e-3, T=np.float64, ny=None, K=5):
    ny = n if ny is None else ny
    prob = ff.Vorticity.Problem(ff.GPU(), nx=n, ny=ny, Lx=2 * math.pi, nu=nu, mu=mu, dt=dt, stepper="ETDRK4", T=T)
    return prob, ff.Adjoint.VorticityAdjoint(prob, checkpoint_every=K)


@pytest.mark.parametrize("n,ny", [(32, 32), (64, 48)])
def test_adjoint_term_dot_identity(ff, cuda, n, ny):
    """<J(s)^T lam, d> = <lam, J(s) d> for random (non-Hermitian, unmasked) lam and d."""
    prob, adj = setup(ff, n, ny=ny)
    rng = np.random.default_rng(3)
    z = ff.Vorticity.random_phase_vorticity(n, ny, seed=4)
    s = orc.rfft(z)
    lam = rng.standard_normal(s.shape) + 1j * rng.standard_normal(s.shape)
    d = rng.standard_normal(s.shape) + 1j * rng.standard_normal(s.shape)
    g = orc.Grid(2, (n, ny), (2 * math.pi, 2 * math.pi))
    Jd = orc.vorticity_calcN_tangent(s, d, g)
    dev = ff.device_array(ff.GPU())
    out = ff.zeros(ff.GPU(), np.complex128, s.shape)
    adj._JT(out, dev(s), dev(lam))
    JTl = ff.to_numpy(out)
    lhs, rhs = redot(JTl, d), redot(lam, Jd)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))


def test_trajectory_gradient_vs_oracle_tangent(ff, cuda):
    """d loss along a physical direction: GPU adjoint vs the oracle's tangent propagated
    through 12 ETDRK4 steps (checkpoints every 5)."""
    n, nsteps = 64, 12
    prob, adj = setup(ff, n, K=5)
    z0 = ff.Vorticity.random_phase_vorticity(n, seed=8)
    zt = ff.Vorticity.random_phase_vorticity(n, seed=9)
    tgt = ff.rfft(ff.device_array(ff.GPU())(zt))
    L, gz, dnu = adj.gradient(z0, tgt, nsteps)
    delta = np.random.default_rng(5).standard_normal((n, n))
    dL_adj = float(np.sum(ff.to_numpy(gz) * delta))
    # oracle tangent
    op = orc.VorticityProblem(n, 2 * math.pi, 1e-3, 1e-2, 2e-3, "ETDRK4")
    s, ds = orc.rfft(z0), orc.rfft(delta)
    for _ in range(nsteps):
        s, ds = orc.etdrk4_vorticity_tangent_step(s, ds, op.timestepper, op.grid)
    t = orc.rfft(zt)
    w = np.full(s.shape, 2.0)
    w[0] = w[-1] = 1.0
    c1, c2 = 1.0 / (n * n) ** 2, 0.5 / (n * n) ** 2
    dLds = 2 * c1 * w * (s - t) + 2 * c2 * w * s
    dL_tan = redot(dLds, ds)
    assert abs(dL_adj - dL_tan) <= 1e-10 * abs(dL_tan)
    L_or = c1 * np.sum(w * np.abs(s - t) ** 2) + c2 * np.sum(w * np.abs(s) ** 2)
    assert abs(L - L_or) <= 1e-12 * L_or


def test_nu_gradient_vs_central_differences(ff, cuda):
    n, nsteps, nu, h = 64, 20, 1e-3, 1e-6
    z0 = ff.Vorticity.random_phase_vorticity(n, seed=10)
    zt = ff.Vorticity.random_phase_vorticity(n, seed=11)
    prob, adj = setup(ff, n, nu=nu, K=7)
    tgt = ff.rfft(ff.device_array(ff.GPU())(zt))
    _, _, dnu = adj.gradient(z0, tgt, nsteps)

    def loss(nu_):
        p, a = setup(ff, n, nu=nu_)
        ff.Vorticity.set_zeta_(p, z0)
        ff.stepforward_(p, nsteps)
        return a.loss(tgt)

    fd = (loss(nu + h) - loss(nu - h)) / (2 * h)
    assert abs(dnu - fd) <= 1e-6 * abs(fd), (dnu, fd)


def test_fp32_adjoint_vs_fp64_differences(ff, cuda):
    """FP32 forward and adjoint (FP64 reductions) against FP64 central differences."""
    n, nsteps = 128, 60
    z0 = ff.Vorticity.random_phase_vorticity(n, seed=12)
    zt = ff.Vorticity.random_phase_vorticity(n, seed=13)
    p32, a32 = setup(ff, n, T=np.float32, K=20)
    tgt32 = ff.rfft(ff.device_array(ff.GPU())(zt.astype(np.float32)))
    _, gz, _ = a32.gradient(z0, tgt32, nsteps)
    p64, a64 = setup(ff, n, T=np.float64)
    tgt64 = ff.rfft(ff.device_array(ff.GPU())(zt))
    rng = np.random.default_rng(14)
    for _ in range(2):
        d = rng.standard_normal((n, n))
        dL = float(np.sum(ff.to_numpy(gz).astype(np.float64) * d))
        vals = []
        for sgn in (1, -1):
            ff.Vorticity.set_zeta_(p64, z0 + sgn * 1e-4 * d)
            ff.stepforward_(p64, nsteps)
            vals.append(a64.loss(tgt64))
        fd = (vals[0] - vals[1]) / 2e-4
        assert abs(dL - fd) <= 1e-4 * abs(fd), (dL, fd)
