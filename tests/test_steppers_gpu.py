"""Time steppers, Diffusion, diagnostics and utilities on the GPU, restating the
reference's tests (test/test_timesteppers.jl, test/test_diagnostics.jl,
test/test_utils.jl, test/runtests.jl:215-334) and checking against the CPU oracle."""
import math

import numpy as np
import pytest

from oracle import ff_oracle as orc

pytestmark = pytest.mark.gpu

RTOL_TIMESTEPPERS = 1e-12  # test/runtests.jl:24
RTOL_UTILS = 1e-13         # test/runtests.jl:23
STEPPERS = ["ForwardEuler", "RK4", "LSRK54", "ETDRK4", "AB3", "FilteredForwardEuler", "FilteredRK4",
            "FilteredLSRK54", "FilteredETDRK4", "FilteredAB3"]


def isapprox(a, b, rtol=1.4901161193847656e-08, atol=0.0):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm(a - b) <= max(atol, rtol * max(np.linalg.norm(a), np.linalg.norm(b)))


def gaussian(x, t, c0=0.01, sigma=0.2, kappa=1e-2):
    """gausian_solution, test/test_timesteppers.jl:1."""
    return c0 * sigma / np.sqrt(sigma ** 2 + 2 * kappa * t) * np.exp(-x ** 2 / (2 * (sigma ** 2 + 2 * kappa * t)))


NX, KAPPA = 128, 1e-2
DT = 1e-9 * 1 / KAPPA


def _diffusion(ff, stepper, kappa):
    return ff.Diffusion.Problem(ff.GPU(), nx=NX, Lx=2 * math.pi, κ=kappa, dt=DT, stepper=stepper)


@pytest.mark.parametrize("stepper", STEPPERS)
@pytest.mark.parametrize("varying", [False, True], ids=["constant", "varying"])
def test_diffusion_stepforward(ff, cuda, stepper, varying):
    """constantdiffusiontest_stepforward / varyingdiffusiontest_stepforward."""
    nsteps = 1000
    kappa = KAPPA * np.ones(NX) if varying else KAPPA
    prob = _diffusion(ff, stepper, kappa)
    x = prob.grid.x
    c_initial = gaussian(x, 0)
    c_final = gaussian(x, nsteps * float(prob.clock.dt))
    ff.Diffusion.set_c_(prob, c_initial)
    ff.stepforward_(prob, nsteps)
    ff.Diffusion.updatevars_(prob)
    c = ff.to_numpy(prob.vars.c)
    assert isapprox(c_final, c, rtol=prob.clock.step * RTOL_TIMESTEPPERS)
    # and against the oracle's restatement of the same steps
    oprob = orc.DiffusionProblem(nx=NX, Lx=2 * math.pi, kappa=kappa, dt=DT, stepper=stepper)
    orc.diffusion_set_c(oprob, c_initial)
    orc.stepforward(oprob, nsteps)
    orc.diffusion_updatevars(oprob)
    assert isapprox(c, oprob.vars.c, rtol=1e-12)


@pytest.mark.parametrize("stepper", STEPPERS)
def test_diffusion_step_until(ff, cuda, stepper):
    """constantdiffusiontest_step_until; ETDRK4 steppers must throw."""
    prob = _diffusion(ff, stepper, KAPPA)
    t_final = 1000 * DT + 1e-6 / math.pi
    x = prob.grid.x
    ff.Diffusion.set_c_(prob, gaussian(x, 0))
    if not ff.isexplicit(stepper):
        with pytest.raises(Exception):
            ff.step_until_(prob, t_final)
        return
    ff.step_until_(prob, t_final)
    ff.Diffusion.updatevars_(prob)
    assert isapprox(gaussian(x, t_final), ff.to_numpy(prob.vars.c), rtol=prob.clock.step * RTOL_TIMESTEPPERS)
    assert abs(float(prob.clock.t) - t_final) < 1e-15


@pytest.mark.parametrize("stepper", ["ETDRK4", "FilteredETDRK4", "RK4", "FilteredRK4"])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_linear_step_matches_generic_substeps(ff, cuda, stepper, T):
    """Constant kappa (N = 0): the one-pass step (ff_linear_step) gives the generic
    substeps' bits -- ETDRK4 is exactly exp(L dt) sol, RK4 its four linear stages in the
    generic kernels' order.  nx = 252 gives an odd mode count (nkr = 127: the vectorised
    FP32 pass handles the last mode apart); dt kappa kr_max^2 = 1.6 keeps RK4 stable."""
    x = None
    out = []
    for fused in (True, False):
        p = ff.Diffusion.Problem(ff.GPU(), nx=252, Lx=2 * math.pi, κ=1e-2, dt=0.01, stepper=stepper, T=T)
        if not fused:
            p.eqn.zero_N = False
        x = p.grid.x
        ff.Diffusion.set_c_(p, np.exp(-x ** 2 / (2 * 0.3 ** 2)) + 0.1 * np.sin(3 * x))
        assert (p.timestepper._native(p.eqn) is not None) == fused
        ff.stepforward_(p, 40)
        out.append(ff.to_numpy(p.sol))
        assert p.clock.step == 40
    assert np.all(np.isfinite(out[0]))
    assert np.array_equal(out[0], out[1])


def test_linear_step_3d_ensemble_vs_oracle(ff, cuda):
    """The stacked 3D constant-kappa ensemble on the one-pass step: every member against
    its own oracle run (ThreeDGrid, L = -kappa Krsq, N = 0)."""
    kappas = [1e-3, 4e-3, 1e-2]
    ens = ff.Diffusion.Ensemble3D(kappas, n=16, dt=2e-3, T=np.float64)
    assert ens.prob.timestepper._native(ens.prob.eqn) is not None
    s0 = ff.to_numpy(ens.prob.sol).copy()
    ens.stepforward_(25)
    got = ff.to_numpy(ens.prob.sol)
    for b, kappa in enumerate(kappas):
        op = orc.Diffusion3DProblem(16, 2 * math.pi, kappa, 2e-3, "ETDRK4")
        op.sol[...] = s0[..., b]
        orc.stepforward(op, 25)
        assert isapprox(got[..., b], op.sol, rtol=1e-13), b


def test_diffusion_config_case(ff, cuda):
    """The Diffusion problem on nx=128, Lx=2pi, kappa=1e-2, c0=exp(-x^2/(2 0.3^2)),
    RK4 and ETDRK4 with dt=0.01 for 500 steps: each Fourier mode decays as exp(-kappa k^2 t)."""
    for stepper in ("RK4", "ETDRK4"):
        prob = ff.Diffusion.Problem(ff.GPU(), nx=128, Lx=2 * math.pi, κ=1e-2, dt=0.01, stepper=stepper)
        x = prob.grid.x
        ff.Diffusion.set_c_(prob, np.exp(-x ** 2 / (2 * 0.3 ** 2)))
        s0 = ff.to_numpy(prob.sol).copy()
        ff.stepforward_(prob, 500)
        kr = prob.grid.kr_host.reshape(-1)
        expect = s0 * np.exp(-1e-2 * kr ** 2 * 500 * 0.01)
        assert isapprox(ff.to_numpy(prob.sol), expect, rtol=1e-9)


def test_diagnostic_steps(ff, cuda):
    """test_diagnosticsteps for freq 1, 2 and 9 (test/test_diagnostics.jl:1-9)."""
    for nsteps, freq, ndata in [(100, 1, None), (100, 2, None), (100, 9, 20)]:
        prob = ff.Diffusion.Problem(ff.GPU(), nx=6, Lx=2 * math.pi)
        d = ff.Diagnostic(lambda p: 1, prob, nsteps=nsteps, freq=freq, ndata=ndata)
        ff.stepforward_(prob, d, nsteps)
        assert d.steps[:d.i] == [0] + list(range(freq, nsteps + 1, freq))


def test_scalar_diagnostics(ff, cuda):
    """test_scalardiagnostics: the variance decays as 1/2 exp(-2 kappa k0^2 t)."""
    for freq in (1, 2):
        nx, Lx, kappa, nsteps = 6, 2 * math.pi, 1e-2, 100
        k0 = 2 * math.pi / Lx
        dt = 1e-2 / (kappa * k0 ** 2)
        prob = ff.Diffusion.Problem(ff.GPU(), nx=nx, Lx=Lx, κ=kappa, dt=dt, stepper="RK4")
        ff.Diffusion.set_c_(prob, np.sin(k0 * prob.grid.x))
        d = ff.Diagnostic(lambda p: ff.parsevalsum2(p.sol, p.grid) / Lx, prob, nsteps=nsteps, freq=freq)
        ff.stepforward_(prob, d, nsteps)
        t = np.array(d["t"])
        assert isapprox(np.array(d["data"]), 0.5 * np.exp(-kappa * k0 ** 2 * t) ** 2)


def test_diagnostic_increment_extend_getindex(ff, cuda):
    prob = ff.Diffusion.Problem(ff.GPU(), nx=6, Lx=2 * math.pi, κ=1e-2, dt=1.0, stepper="ETDRK4")
    d1 = ff.Diagnostic(lambda p: 2.0, prob, nsteps=10)
    d2 = ff.Diagnostic(lambda p: 2.0j, prob, nsteps=10)
    ff.increment_([d1, d2])
    assert d1.data[1] == 2.0 and d2.data[1] == 2.0j
    for _ in range(6):
        ff.increment_([d1, d2])
    assert d1[range(2, 6)] == [2.0] * 4 and d2[range(2, 6)] == [2.0j] * 4
    s1 = ff.Diagnostic(lambda p: p.sol, prob, nsteps=1)
    n1 = len(s1.t)
    ff.extend_(s1, 12)
    assert len(s1.t) == n1 + 12
    s2 = ff.Diagnostic(lambda p: p.sol, prob, nsteps=4)
    n2 = len(s2.t)
    ff.extend_(s2)
    assert len(s2.t) == 2 * n2


def test_parsevalsums(ff, cuda):
    """test_parsevalsums on analytic and random fields (test/runtests.jl:243-295)."""
    dev = ff.device_array(ff.GPU())
    g = ff.TwoDGrid(ff.GPU(), nx=64, Lx=2 * math.pi, ny=128, Ly=3 * math.pi)
    X, Y = np.meshgrid(g.x, g.y, indexing="ij")
    sigma = 0.5
    f1 = np.exp(-(X ** 2 + Y ** 2) / (2 * sigma ** 2))
    f3 = np.random.default_rng(1).standard_normal((g.nx, g.ny))
    for f in (f1, f3):
        integral = np.sum(np.abs(f) ** 2) * float(g.dx) * float(g.dy)
        fh = ff.rfft(dev(f))
        a2 = dev(np.abs(ff.to_numpy(fh)) ** 2 + 0j)
        assert isapprox(integral, ff.parsevalsum(a2, g), rtol=RTOL_UTILS)
        assert isapprox(integral, ff.parsevalsum2(fh, g), rtol=RTOL_UTILS)
        fc = ff.fft(dev(f.astype(complex)))
        assert isapprox(integral, ff.parsevalsum2(fc, g), rtol=RTOL_UTILS)
    g1 = ff.OneDGrid(ff.GPU(), nx=64, Lx=2 * math.pi)
    f = np.exp(-g1.x ** 2 / (2 * sigma ** 2))
    integral = np.sum(f ** 2) * float(g1.dx)
    assert isapprox(integral, ff.parsevalsum2(ff.rfft(dev(f)), g1), rtol=RTOL_UTILS)


def test_jacobian_known_answers(ff, cuda):
    """J(sin1, sin1) = 0 and J(sin1, sin2) analytic on a 64x128 grid (test/runtests.jl:244-280),
    atol = nx ny 10 eps."""
    g = ff.TwoDGrid(ff.GPU(), nx=64, Lx=2 * math.pi, ny=128, Ly=3 * math.pi)
    X, Y = np.meshgrid(g.x, g.y, indexing="ij")
    k0, l0 = 2 * math.pi / float(g.Lx), 2 * math.pi / float(g.Ly)
    k1, l1 = 2 * k0, 6 * l0
    k2, l2 = 3 * k0, -3 * l0
    s1 = np.sin(k1 * X + l1 * Y)
    s2 = np.sin(k2 * X + l2 * Y)
    J12 = (k1 * l2 - k2 * l1) * np.cos(k1 * X + l1 * Y) * np.cos(k2 * X + l2 * Y)
    dev = ff.device_array(ff.GPU())
    atol = g.nx * g.ny * 10 * np.finfo(float).eps
    assert isapprox(ff.to_numpy(ff.jacobian(dev(s1), dev(s1), g)), 0 * s1, atol=atol)
    assert isapprox(ff.to_numpy(ff.jacobian(dev(s1), dev(s2), g)), J12, atol=atol)


def test_dealias_masks(ff, cuda):
    """dealias_ on GPU arrays equals the oracle's index-range zeroing (and the reference
    test's mask criteria, test/test_grid.jl:80-133)."""
    dev = ff.device_array(ff.GPU())
    for g, og in [(ff.TwoDGrid(ff.GPU(), nx=6, Lx=2 * math.pi, ny=8, Ly=4 * math.pi),
                   orc.TwoDGrid(6, 2 * math.pi, 8, 4 * math.pi)),
                  (ff.ThreeDGrid(ff.GPU(), nx=16, Lx=2 * math.pi, ny=32, Ly=2 * math.pi, nz=34, Lz=2 * math.pi),
                   orc.ThreeDGrid(16, 2 * math.pi, 32, 2 * math.pi, 34, 2 * math.pi)),
                  (ff.OneDGrid(ff.GPU(), nx=16, Lx=2 * math.pi), orc.OneDGrid(16, 2 * math.pi))]:
        for shape in (og.spectral_shape, tuple([og.nx] + list(og.n[1:]))):
            fh = np.ones(shape, complex)
            d = dev(fh)
            ff.dealias_(d, g)
            assert np.array_equal(ff.to_numpy(d), orc.dealias(fh.copy(), og))
    g0 = ff.TwoDGrid(ff.GPU(), nx=8, Lx=2 * math.pi, aliased_fraction=0)
    d = dev(np.ones((5, 8), complex))
    assert ff.dealias_(d, g0) is None and np.all(ff.to_numpy(d) == 1)


def test_filter_kwargs_instantiation(ff, cuda):
    """instantiate_problem_with_filter_kwargs: innerK=0, outerK=1/16 gives filter[3] < 1e-16."""
    for stepper in [s for s in STEPPERS if s.startswith("Filtered")]:
        dummy = ff.Diffusion.Problem(ff.GPU(), nx=16, stepper=stepper)
        real = ff.Problem(dummy.eqn, stepper, 1.0, dummy.grid, dummy.vars, dummy.params, innerK=0.0,
                          outerK=1 / 16)
        assert float(ff.to_numpy(real.timestepper.filter)[2]) < 1e-16
    for stepper in STEPPERS:
        p = ff.Diffusion.Problem(ff.GPU(), nx=4, stepper=stepper)
        assert isinstance(p, ff.Problem)
