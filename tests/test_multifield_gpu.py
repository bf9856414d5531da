"""Multi-field states, user-written calcN!, complex-field Jacobians and the stacked 3D
diffusion ensemble on the GPU, against the CPU oracle."""
import math

import numpy as np
import pytest

from oracle import ff_oracle as orc

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


F, G, H, NU, NNU = 1.0, 1.0, 1.0, 1e-6, 2  # Coriolis, gravity, depth, hyperviscosity


def sw_calcN_torch(ff):
    """A user calcN! with a multi-field sol (nkr, 3) = (u, v, eta), the pattern of the
    reference's 1D linear shallow-water example: N_u = f v - i k g eta, N_v = -f u,
    N_eta = -i k H u, then dealias!."""
    def calcN(N, sol, t, clock, vars, params, grid):
        kr = grid.kr.reshape(-1)
        N[:, 0] = F * sol[:, 1] - 1j * kr * G * sol[:, 2]
        N[:, 1] = -F * sol[:, 0]
        N[:, 2] = -1j * kr * H * sol[:, 0]
        ff.dealias_(N, grid)
    return calcN


def sw_calcN_numpy(N, sol, t, clock, vars, params, grid):
    kr = grid.kr.reshape(-1)
    N[:, 0] = F * sol[:, 1] - 1j * kr * G * sol[:, 2]
    N[:, 1] = -F * sol[:, 0]
    N[:, 2] = -1j * kr * H * sol[:, 0]
    orc.dealias(N, grid)


@pytest.mark.parametrize("stepper", ["RK4", "ETDRK4", "FilteredETDRK4", "LSRK54", "AB3"])
def test_multifield_user_calcN(ff, cuda, stepper):
    nx, Lx, dt, nsteps = 128, 2 * math.pi, 0.01, 20
    g = ff.OneDGrid(ff.GPU(), nx=nx, Lx=Lx)
    og = orc.OneDGrid(nx, Lx)
    D = -NU * og.kr.reshape(-1) ** (2 * NNU)
    L = np.stack([D, D, D], axis=1)
    eq = ff.Equation(ff.device_array(ff.GPU())(np.asfortranarray(L)), sw_calcN_torch(ff), g)
    prob = ff.Problem(eq, stepper, dt, g)
    oprob = orc.Problem(orc.Equation(L, sw_calcN_numpy, og), stepper, dt, og)
    x = og.x
    eta0 = np.exp(-x ** 2 / (2 * 0.5 ** 2))
    s0 = np.zeros((og.nkr, 3), complex)
    s0[:, 2] = orc.rfft(eta0)
    s0 = orc.dealias(s0, og)
    prob.sol.copy_(ff.device_array(ff.GPU())(np.asfortranarray(s0)))
    oprob.sol[...] = s0
    ff.stepforward_(prob, nsteps)
    orc.stepforward(oprob, nsteps)
    assert prob.clock.step == nsteps
    assert rel(ff.to_numpy(prob.sol), oprob.sol) < 1e-12


def test_complex_jacobian_known_answer(ff, cuda):
    """J(exp1, exp2) = (k2 l1 - k1 l2) exp((k1 + k2) x + (l1 + l2) y) i (test/runtests.jl:265,280)."""
    g = ff.TwoDGrid(ff.GPU(), nx=64, Lx=2 * math.pi, ny=128, Ly=3 * math.pi)
    X, Y = np.meshgrid(g.x, g.y, indexing="ij")
    k0, l0 = 2 * math.pi / float(g.Lx), 2 * math.pi / float(g.Ly)
    k1, l1, k2, l2 = 2 * k0, 6 * l0, 3 * k0, -3 * l0
    e1 = np.exp(1j * (k1 * X + l1 * Y))
    e2 = np.exp(1j * (k2 * X + l2 * Y))
    J = (k2 * l1 - k1 * l2) * np.exp(1j * ((k1 + k2) * X + (l1 + l2) * Y))
    dev = ff.device_array(ff.GPU())
    got = ff.to_numpy(ff.jacobian(dev(e1), dev(e2), g))
    atol = g.nx * g.ny * 10 * np.finfo(float).eps
    assert np.linalg.norm(got - J) <= atol


def test_diffusion3d_ensemble_members_decay(ff, cuda):
    """Each member of the stacked 3D ensemble evolves as the ETDRK4 step of its own
    kappa: with N = 0 every mode is multiplied by exp(L dt) per step."""
    kappas = [1e-3, 5e-3, 1e-2]
    ens = ff.Diffusion.Ensemble3D(kappas, n=32, dt=2e-3, T=np.float64)
    s0 = ff.to_numpy(ens.prob.sol).copy()
    ens.stepforward_(10)
    s = ff.to_numpy(ens.prob.sol)
    Krsq = ens.grid.Krsq_host.astype(np.float64)
    for b, k in enumerate(kappas):
        expect = s0[..., b] * np.exp(-k * Krsq * 10 * 2e-3)
        assert rel(s[..., b], expect) < 1e-12
