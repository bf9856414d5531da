"""Pin the CPU oracle to the reference's own known-answer tests (no GPU).

Each test restates a reference test (path:line in the FourierFlows.jl tree) against
oracle/ff_oracle.py; these are what make the oracle a trustworthy yardstick for the GPU
parity tests.
"""
import math

import numpy as np
import pytest

from oracle import ff_oracle as orc


def isapprox(a, b, rtol=1.4901161193847656e-08, atol=0.0):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm(a - b) <= max(atol, rtol * max(np.linalg.norm(a), np.linalg.norm(b)))


def test_fft_known_answers():
    """test/createffttestfunctions.jl:71-209 with rtol_fft = 1e-12."""
    g = orc.OneDGrid(32, 2 * math.pi)
    k0 = g.k[1]
    f = np.cos(5 * k0 * g.x + math.pi / 3)
    th = np.zeros(g.nkr, complex)
    for i in range(g.nkr):
        if abs(g.k[i]) == 5 * k0:
            th[i] = -np.exp(np.sign(g.kr[i]) * 1j * math.pi / 3) * g.nx / 2
    assert isapprox(orc.rfft(f), th, 1e-12)
    g2 = orc.TwoDGrid(32, 2 * math.pi, 64, 3 * math.pi)
    X, Y = np.meshgrid(g2.x, g2.y, indexing="ij")
    k0, l0 = g2.k[1, 0], g2.l[0, 1]
    f1 = np.cos(5 * k0 * X) * np.cos(2 * l0 * Y)
    th = np.zeros((g2.nkr, g2.nl), complex)
    kr, l = g2.kr.reshape(-1), g2.l.reshape(-1)
    for j in range(g2.nl):
        for i in range(g2.nkr):
            if abs(kr[i]) == 5 * k0 and abs(l[j]) == 2 * l0:
                th[i, j] = -g2.nx * g2.ny / 4
    assert isapprox(orc.rfft(f1), th, 1e-12)
    assert isapprox(orc.irfft(th, g2.nx), f1, 1e-12)
    g3 = orc.ThreeDGrid(32, 2 * math.pi, 30, 3 * math.pi, 16, 4.0)
    X, Y, Z = np.meshgrid(g3.x, g3.y, g3.z, indexing="ij")
    k0, l0, m0 = g3.k[1, 0, 0], g3.l[0, 1, 0], g3.m[0, 0, 1]
    f2 = np.sin(5 * k0 * X + 2 * l0 * Y + 3 * m0 * Z)
    th = np.zeros((g3.nkr, g3.nl, g3.nm), complex)
    kr, l, m = g3.kr.reshape(-1), g3.l.reshape(-1), g3.m.reshape(-1)
    for c in range(g3.nm):
        for j in range(g3.nl):
            for i in range(g3.nkr):
                if kr[i] == 5 * k0 and l[j] == 2 * l0 and m[c] == 3 * m0:
                    th[i, j, c] = g3.nx * g3.ny * g3.nz / 2
    assert isapprox(orc.rfft(f2), -1j * th, 1e-12)


@pytest.mark.parametrize("af", [0, 1 / 3, 1 / 2, 1 / 4])
def test_aliased_fraction_ranges(af):
    """test_aliased_fraction (test/test_grid.jl:203-227), 0-based half-open ranges."""
    nx, ny, nz = 16, 32, 34
    lower = lambda n: math.floor((1 - af) / 2 * n) + 1
    upper = lambda n: math.ceil((1 + af) / 2 * n)
    g3 = orc.ThreeDGrid(nx, 2 * math.pi, ny, 2 * math.pi, nz, 2 * math.pi, aliased_fraction=af)
    if af == 0:
        assert g3.kalias is None and g3.kralias is None
        return
    assert g3.kralias == (lower(nx) - 1, nx // 2 + 1)
    assert g3.kalias == (lower(nx) - 1, upper(nx))
    assert g3.lalias == (lower(ny) - 1, upper(ny))
    assert g3.malias == (lower(nz) - 1, upper(nz))


def test_two_thirds_ranges_at_1024():
    """The asymmetric 2/3 mask at n = 1024: kalias = 342:683, kralias = 342:513 (1-based)."""
    kal, kral = orc.getaliasedwavenumbers(1024, 513, 1 / 3)
    assert kal == (341, 683) and kral == (341, 513)


def test_dealias_mask_criteria():
    """testdealias (test/test_grid.jl:80-133): after dealias!, zeroing the kept modes
    (|kr| < 2/3 kmax, -lmax <= l < lmax) leaves nothing."""
    for g in [orc.OneDGrid(6, 2 * math.pi), orc.TwoDGrid(6, 2 * math.pi, 8, 4 * math.pi),
              orc.ThreeDGrid(6, 2 * math.pi, 8, 4 * math.pi, 10, 3.0)]:
        fh = orc.dealias(np.ones(g.spectral_shape, complex), g)
        kmax = round(g.kr.max() * 2 / 3)
        keep = g.kr.reshape((-1,) + (1,) * (g.ndim - 1)) < kmax
        if g.ndim >= 2:
            lmax = round(np.abs(g.l).max() * 2 / 3)
            keep = keep & (g.l < lmax) & (g.l >= -lmax)
        if g.ndim == 3:
            mmax = round(np.abs(g.m).max() * 2 / 3)
            keep = keep & (g.m < mmax) & (g.m >= -mmax)
        fh[np.broadcast_to(keep, fh.shape)] = 0
        assert np.abs(fh).sum() == 0


def test_makefilter_bounds():
    """testmakefilter (test/test_grid.jl:165-173): 1 below K=0.65, ~0 above K=0.999."""
    for g in [orc.OneDGrid(6, 2 * math.pi), orc.TwoDGrid(6, 2 * math.pi, 8, 4 * math.pi),
              orc.ThreeDGrid(6, 2 * math.pi, 8, 4 * math.pi, 10, 3.0)]:
        f = orc.makefilter(g)
        if g.ndim == 1:
            K = g.kr * g.dx / math.pi
        elif g.ndim == 2:
            K = np.sqrt((g.kr * g.dx / math.pi) ** 2 + (g.l * g.dy / math.pi) ** 2)
        else:
            K = np.sqrt((g.kr * g.dx / math.pi) ** 2 + (g.l * g.dy / math.pi) ** 2 + (g.m * g.dz / math.pi) ** 2)
        K = np.broadcast_to(K, f.shape)
        assert np.all(f[K < 0.65] == 1)
        assert np.all(np.abs(f[K > 0.999]) < 1e-12)


def gaussian(x, t, c0=0.01, sigma=0.2, kappa=1e-2):
    return c0 * sigma / np.sqrt(sigma ** 2 + 2 * kappa * t) * np.exp(-x ** 2 / (2 * (sigma ** 2 + 2 * kappa * t)))


STEPPERS = ["ForwardEuler", "RK4", "LSRK54", "ETDRK4", "AB3", "FilteredForwardEuler", "FilteredRK4",
            "FilteredLSRK54", "FilteredETDRK4", "FilteredAB3"]


@pytest.mark.parametrize("stepper", STEPPERS)
@pytest.mark.parametrize("varying", [False, True], ids=["constant", "varying"])
def test_gaussian_diffusion(stepper, varying):
    """constantdiffusiontest_stepforward / varyingdiffusiontest_stepforward
    (test/test_timesteppers.jl:39-59), rtol = step * 1e-12."""
    kappa, dt = 1e-2, 1e-7
    prob = orc.DiffusionProblem(nx=128, Lx=2 * math.pi, kappa=kappa * np.ones(128) if varying else kappa, dt=dt,
                                stepper=stepper)
    orc.diffusion_set_c(prob, gaussian(prob.grid.x, 0))
    orc.stepforward(prob, 1000)
    orc.diffusion_updatevars(prob)
    assert isapprox(gaussian(prob.grid.x, 1000 * dt), prob.vars.c, rtol=prob.clock.step * 1e-12)


@pytest.mark.parametrize("stepper", STEPPERS)
def test_step_until(stepper):
    """constantdiffusiontest_step_until (test/test_timesteppers.jl:61-70, runtests.jl:222-226)."""
    dt = 1e-7
    prob = orc.DiffusionProblem(nx=128, Lx=2 * math.pi, kappa=1e-2, dt=dt, stepper=stepper)
    t_final = 1000 * dt + 1e-6 / math.pi
    orc.diffusion_set_c(prob, gaussian(prob.grid.x, 0))
    if not orc.isexplicit(stepper):
        with pytest.raises(RuntimeError):
            orc.step_until(prob, t_final)
        return
    orc.step_until(prob, t_final)
    orc.diffusion_updatevars(prob)
    assert isapprox(gaussian(prob.grid.x, t_final), prob.vars.c, rtol=prob.clock.step * 1e-12)


def test_parseval_sums():
    """test_parsevalsums (test/test_utils.jl:309-323, rtol_utils = 1e-13)."""
    g = orc.TwoDGrid(64, 2 * math.pi, 128, 3 * math.pi)
    X, Y = np.meshgrid(g.x, g.y, indexing="ij")
    for f in (np.exp(-(X ** 2 + Y ** 2) / (2 * 0.25)), np.random.default_rng(0).standard_normal((64, 128))):
        integral = np.sum(f ** 2) * g.dx * g.dy
        assert isapprox(integral, orc.parsevalsum2(orc.rfft(f), g), 1e-13)
        assert isapprox(integral, orc.parsevalsum(np.abs(orc.rfft(f)) ** 2, g), 1e-13)
        assert isapprox(integral, orc.parsevalsum2(orc.fft(f), g), 1e-13)


def test_jacobian_known_answer():
    """test_jacobian (test/runtests.jl:263-280, test/test_utils.jl:329-330)."""
    g = orc.TwoDGrid(64, 2 * math.pi, 128, 3 * math.pi)
    X, Y = np.meshgrid(g.x, g.y, indexing="ij")
    k0, l0 = 2 * math.pi / g.Lx, 2 * math.pi / g.Ly
    k1, l1, k2, l2 = 2 * k0, 6 * l0, 3 * k0, -3 * l0
    s1, s2 = np.sin(k1 * X + l1 * Y), np.sin(k2 * X + l2 * Y)
    e1, e2 = np.exp(1j * (k1 * X + l1 * Y)), np.exp(1j * (k2 * X + l2 * Y))
    atol = g.nx * g.ny * 10 * np.finfo(float).eps
    assert isapprox(orc.jacobian(s1, s1, g), 0 * s1, atol=atol)
    assert isapprox(orc.jacobian(s1, s2, g), (k1 * l2 - k2 * l1) * np.cos(k1 * X + l1 * Y) * np.cos(k2 * X + l2 * Y),
                    atol=atol)
    assert isapprox(orc.jacobian(e1, e2, g), (k2 * l1 - k1 * l2) * np.exp(1j * ((k1 + k2) * X + (l1 + l2) * Y)),
                    atol=atol)


def test_vorticity_calcN_is_minus_dealiased_jacobianh():
    """The flux-form vorticity term equals -dealias(jacobianh(psi, zeta)) for a dealiased
    field: the 2/3 rule leaves no aliasing on the kept modes, so both forms agree."""
    g = orc.TwoDGrid(64, 2 * math.pi)
    zh = orc.dealias(orc.rfft(np.random.default_rng(4).standard_normal((64, 64))), g)
    N = np.zeros_like(zh)
    orc.vorticity_calcN(N, zh, 0.0, None, None, None, g)
    psi = orc.irfft(-zh * g.invKrsq, g.nx)
    zeta = orc.irfft(zh, g.nx)
    J = orc.dealias(orc.jacobianh(psi, zeta, g), g)
    assert np.linalg.norm(N + J) / np.linalg.norm(J) < 1e-13


def test_diagnostic_decay():
    """test_scalardiagnostics (test/test_diagnostics.jl:11-31)."""
    nx, Lx, kappa = 6, 2 * math.pi, 1e-2
    k0 = 2 * math.pi / Lx
    dt = 1e-2 / (kappa * k0 ** 2)
    prob = orc.DiffusionProblem(nx=nx, Lx=Lx, kappa=kappa, dt=dt, stepper="RK4")
    orc.diffusion_set_c(prob, np.sin(k0 * prob.grid.x))
    d = orc.Diagnostic(lambda p: orc.parsevalsum2(p.sol, p.grid) / Lx, prob, nsteps=100, freq=1)
    orc.stepforward(prob, 100, d)
    t = np.array(d.t[:d.i])
    assert isapprox(np.array(d.data[:d.i]), 0.5 * np.exp(-kappa * k0 ** 2 * t) ** 2)
    assert d.steps[:d.i] == list(range(101))


def test_show_strings_grid_values():
    """The numbers in the reference's show() strings (test/runtests.jl:118-122)."""
    g = orc.OneDGrid(6, 2 * math.pi)
    assert repr(float(g.dx)) == "1.0471975511965976"
    assert repr(float(g.x[0])) == "-3.141592653589793" and repr(float(g.x[-1])) == "2.094395102393195"
    g3 = orc.ThreeDGrid(6, 2 * math.pi, 8, 4 * math.pi, 10, 3.0)
    assert repr(float(g3.y[-1])) == "4.71238898038469" and repr(float(g3.z[0])) == "-1.5"
    assert repr(float(g3.z[-1])) == "1.2"


def test_vorticity_tangent_matches_central_differences():
    """The oracle's forward-mode tangent of an ETDRK4 step agrees with central differences
    of the oracle step (the reference CPU path the GPU adjoint is checked against)."""
    g_prob = orc.VorticityProblem(32, 2 * math.pi, 1e-3, 1e-2, 2e-3, "ETDRK4")
    ts, g = g_prob.timestepper, g_prob.grid
    rng = np.random.default_rng(2)
    s = orc.dealias(orc.rfft(rng.standard_normal((32, 32))), g)
    ds = orc.rfft(rng.standard_normal((32, 32)))
    _, tan = orc.etdrk4_vorticity_tangent_step(s, ds, ts, g)
    h = 1e-6
    sp, _ = orc.etdrk4_vorticity_tangent_step(s + h * ds, ds, ts, g)
    sm, _ = orc.etdrk4_vorticity_tangent_step(s - h * ds, ds, ts, g)
    fd = (sp - sm) / (2 * h)
    assert np.linalg.norm(fd - tan) / np.linalg.norm(tan) < 1e-8


# radialspectrum known answers (test/runtests.jl:297-307 via test/test_utils.jl:59-77):
# normalised difference to the analytic angular integral below atol 0.1 at refinement 16
def _radial_cases():
    d = 128 / 10
    iso = (lambda k, l: np.exp(-(k ** 2 + l ** 2) / (2 * d ** 2)), lambda r: 2 * np.pi * r * np.exp(-r ** 2 / (2 * d ** 2)))

    def ani_f(k, l):
        with np.errstate(invalid="ignore", divide="ignore"):
            return np.exp(-(k ** 2 + l ** 2) / (2 * d ** 2)) * k ** 2 / (k ** 2 + l ** 2)

    ani = (ani_f, lambda r: np.pi * r * np.exp(-r ** 2 / (2 * d ** 2)))
    return [("isotropic", *iso), ("anisotropic", *ani)]


@pytest.mark.parametrize("rfft_form", [False, True])
@pytest.mark.parametrize("case", [0, 1])
def test_pin_radialspectrum(rfft_form, case):
    name, f, fr = _radial_cases()[case]
    g = orc.Grid(2, (128, 128), (2 * math.pi, 2 * math.pi))
    K = g.kr if rfft_form else g.k
    ah = f(K + 0 * g.l, 0 * K + g.l).astype(np.float64)
    ah[0, 0] = 0.0
    rho, est = orc.radialspectrum(ah, g, refinement=16)
    assert np.sum(np.abs(fr(rho) - est)) / len(rho) < 0.1, name
