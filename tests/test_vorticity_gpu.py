"""The fused 2D vorticity path on the GPU against the CPU oracle.

Tolerances: FP64 relative L2 <= 1e-12 over short horizons (the bar for the plain FP64
path); FP32 state and transforms relative L2 <= 1e-5 against the FP64 oracle after
100 steps."""
import math

import numpy as np
import pytest

from oracle import ff_oracle as orc

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def make_pair(ff, n, stepper, T=np.float64, nu=1e-3, mu=1e-2, dt=2e-3, seed=3, af=1 / 3, ny=None, **kw):
    ny = n if ny is None else ny
    z0 = ff.Vorticity.random_phase_vorticity(n, ny, seed=seed, aliased_fraction=af if af > 0 else 1 / 3)
    prob = ff.Vorticity.Problem(ff.GPU(), nx=n, ny=ny, Lx=2 * math.pi, nu=nu, mu=mu, dt=dt, stepper=stepper, T=T,
                                aliased_fraction=af, **kw)
    ff.Vorticity.set_zeta_(prob, z0)
    g = orc.Grid(2, (n, ny), (2 * math.pi, 2 * math.pi), None, np.float64, af)
    Lop = (-nu * g.Krsq - mu).astype(np.float64)
    eq = orc.Equation(Lop, orc.vorticity_calcN, g)
    oprob = orc.Problem(eq, stepper, dt, g, None, orc.VorticityParams(nu, mu), **kw)
    oprob.sol[...] = orc.rfft(z0)
    return prob, oprob


@pytest.mark.parametrize("n,ny", [(32, 32), (64, 48), (128, 128), (48, 96)])
def test_calcN_vs_oracle(ff, cuda, n, ny):
    prob, oprob = make_pair(ff, n, "ETDRK4", ny=ny)
    N = ff.zeros(ff.GPU(), np.complex128, (n // 2 + 1, ny))
    ff.Vorticity.calcN_(N, prob.sol, 0.0, prob.clock, prob.vars, prob.params, prob.grid)
    No = np.zeros_like(oprob.sol)
    orc.vorticity_calcN(No, oprob.sol, 0.0, None, None, None, oprob.grid)
    assert rel(ff.to_numpy(N), No) < 1e-13
    # the input was not modified (the mask is applied on the fly)
    assert np.array_equal(ff.to_numpy(prob.sol), oprob.sol) or rel(ff.to_numpy(prob.sol), oprob.sol) < 1e-15


@pytest.mark.parametrize("stepper", ["ETDRK4", "FilteredETDRK4", "RK4", "FilteredRK4", "LSRK54", "FilteredLSRK54"])
def test_fused_steppers_vs_oracle_fp64(ff, cuda, stepper):
    prob, oprob = make_pair(ff, 64, stepper)
    assert prob.timestepper._native(prob.eqn) is not None, "expected the fused native stepper"
    ff.stepforward_(prob, 10)
    orc.stepforward(oprob, 10)
    assert prob.clock.step == 10
    assert rel(ff.to_numpy(prob.sol), oprob.sol) < 1e-12


@pytest.fixture(params=["register", "generic"])
def kernel_path(request, monkeypatch):
    """Run a test on the register-resident power-of-two kernels and on the generic ones."""
    if request.param == "generic":
        monkeypatch.setenv("FF_VORT_GENERIC", "1")
    else:
        monkeypatch.delenv("FF_VORT_GENERIC", raising=False)
    return request.param


@pytest.mark.parametrize("stepper", ["ETDRK4", "RK4", "FilteredLSRK54"])
@pytest.mark.parametrize("n,ny", [(32, 32), (128, 64), (64, 256)])
def test_fused_paths_vs_oracle(ff, cuda, kernel_path, stepper, n, ny):
    prob, oprob = make_pair(ff, n, stepper, ny=ny)
    ff.stepforward_(prob, 6)
    fs = prob.timestepper._native(prob.eqn).fs
    assert (fs.config()["radix_order"] == -1) == (kernel_path == "register")
    orc.stepforward(oprob, 6)
    assert rel(ff.to_numpy(prob.sol), oprob.sol) < 1e-12


@pytest.mark.parametrize("stepper", ["ETDRK4", "FilteredETDRK4", "RK4", "FilteredRK4", "LSRK54", "FilteredLSRK54"])
@pytest.mark.parametrize("n,ny", [(64, 64), (128, 256)])
def test_fp32_fused_steppers_vs_oracle(ff, cuda, stepper, n, ny):
    """FP32 register path, where pass C also runs the next substep's pass A: every stepper
    against the FP64 oracle after 20 steps."""
    prob, oprob = make_pair(ff, n, stepper, T=np.float32, ny=ny)
    ff.stepforward_(prob, 20)
    orc.stepforward(oprob, 20)
    assert rel(ff.to_numpy(prob.sol).astype(np.complex128), oprob.sol) < 1e-5


def test_calcN_register_path(ff, cuda):
    for n, ny in [(64, 64), (256, 128), (32, 512)]:
        prob, oprob = make_pair(ff, n, "ETDRK4", ny=ny)
        N = ff.zeros(ff.GPU(), np.complex128, (n // 2 + 1, ny))
        ff.Vorticity.calcN_(N, prob.sol, 0.0, prob.clock, prob.vars, prob.params, prob.grid)
        No = np.zeros_like(oprob.sol)
        orc.vorticity_calcN(No, oprob.sol, 0.0, None, None, None, oprob.grid)
        assert rel(ff.to_numpy(N), No) < 1e-13, (n, ny)


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_uneven_ensemble_vs_oracle(ff, cuda, T):
    """An ensemble of different sizes and viscosities advanced in one launch per pass: every
    member matches its own oracle run.  Two members of equal size and viscosity share
    their operator and coefficient arrays."""
    spec = [(32, 1e-3, 5), (128, 3e-4, 6), (64, 1e-4, 7), (128, 1e-5, 8), (256, 2e-4, 9), (128, 3e-4, 10)]
    ens = ff.Vorticity.Ensemble(spec, mu=1e-2, dt=2e-3, T=T)
    assert ens.members[5].coefs[0] is ens.members[1].coefs[0]
    assert ens.members[5].bufs[0].data_ptr() != ens.members[1].bufs[0].data_ptr()
    ens.stepforward_(8)
    tol = 1e-12 if T == np.float64 else 2e-5
    for (n, nu, seed), m in zip(spec, ens.members):
        z0 = ff.Vorticity.random_phase_vorticity(n, seed=seed)
        op = orc.VorticityProblem(n, 2 * math.pi, nu, 1e-2, 2e-3, "ETDRK4")
        op.sol[...] = orc.rfft(z0.astype(T).astype(np.float64))
        orc.stepforward(op, 8)
        assert rel(ff.to_numpy(m.sol).astype(np.complex128), op.sol) < tol, (n, nu)


@pytest.mark.parametrize("stepper", ["ForwardEuler", "AB3", "FilteredAB3"])
def test_generic_steppers_with_native_calcN(ff, cuda, stepper):
    """Steppers without a fused path call the native calcN! between native substeps."""
    prob, oprob = make_pair(ff, 32, stepper, dt=1e-3)
    assert prob.timestepper._native(prob.eqn) is None
    for _ in range(6):
        ff.stepforward_(prob)
    orc.stepforward(oprob, 6)
    assert rel(ff.to_numpy(prob.sol), oprob.sol) < 1e-12


def test_nonsquare_radix3_grid(ff, cuda):
    prob, oprob = make_pair(ff, 96, "ETDRK4", ny=48)
    ff.stepforward_(prob, 5)
    orc.stepforward(oprob, 5)
    assert rel(ff.to_numpy(prob.sol), oprob.sol) < 1e-12


def test_no_dealiasing(ff, cuda):
    prob, oprob = make_pair(ff, 32, "RK4", af=0)
    ff.stepforward_(prob, 4)
    orc.stepforward(oprob, 4)
    assert rel(ff.to_numpy(prob.sol), oprob.sol) < 1e-12


def test_fp32_vs_fp64_oracle_100_steps(ff, cuda):
    prob, oprob = make_pair(ff, 128, "ETDRK4", T=np.float32)
    ff.stepforward_(prob, 100)
    orc.stepforward(oprob, 100)
    e = rel(ff.to_numpy(prob.sol).astype(np.complex128), oprob.sol)
    assert e < 1e-5, e
    E = ff.Vorticity.energy(prob)
    Eo = orc.vorticity_energy(oprob.sol, oprob.grid)
    assert abs(E - Eo) / Eo < 1e-5


def test_energy_enstrophy_vs_oracle(ff, cuda):
    prob, oprob = make_pair(ff, 64, "ETDRK4")
    E, Z = ff.Vorticity.energy(prob), ff.Vorticity.enstrophy(prob)
    assert abs(E - 0.5) < 1e-12  # the initial condition is normalised to E = 0.5
    assert abs(E - orc.vorticity_energy(oprob.sol, oprob.grid)) < 1e-13
    assert abs(Z - orc.vorticity_enstrophy(oprob.sol, oprob.grid)) / Z < 1e-13


def test_updatevars(ff, cuda):
    prob, oprob = make_pair(ff, 32, "ETDRK4")
    ff.Vorticity.updatevars_(prob)
    g = oprob.grid
    zh = oprob.sol
    psih = -zh * g.invKrsq
    u = orc.irfft(-1j * g.l * psih, g.nx)
    v = orc.irfft(1j * g.kr * psih, g.nx)
    assert rel(ff.to_numpy(prob.vars.u), u) < 1e-13
    assert rel(ff.to_numpy(prob.vars.v), v) < 1e-13
    assert rel(ff.to_numpy(prob.vars.zeta), orc.irfft(zh, g.nx)) < 1e-13


def test_full_size_1024_fp64_short_horizon(ff, cuda):
    """The plain FP64 configuration (1024^2, nu=1e-4, mu=1e-2, dt=2e-3): 3 steps vs the oracle."""
    prob, oprob = make_pair(ff, 1024, "ETDRK4", nu=1e-4, mu=1e-2, dt=2e-3, seed=2024)
    ff.stepforward_(prob, 3)
    orc.stepforward(oprob, 3)
    assert rel(ff.to_numpy(prob.sol), oprob.sol) < 1e-12


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_precision_size_2048_two_steps(ff, cuda, T):
    """The 2048^2 grid of the precision form: two ETDRK4 steps against the FP64 oracle."""
    prob, oprob = make_pair(ff, 2048, "ETDRK4", T=T, nu=1e-4, mu=1e-2, dt=1e-3, seed=31)
    ff.stepforward_(prob, 2)
    orc.stepforward(oprob, 2)
    tol = 1e-12 if T == np.float64 else 2e-6
    assert rel(ff.to_numpy(prob.sol).astype(np.complex128), oprob.sol) < tol


def test_full_size_properties_1024(ff, cuda):
    """Size-independent properties at 1024^2: the state stays 2/3-dealiased, energy decays
    monotonically under viscosity + drag, and FP32 tracks FP64 on the GPU."""
    p64, _ = make_pair(ff, 1024, "ETDRK4", nu=1e-4, mu=1e-2, dt=2e-3, seed=9)
    p32, _ = make_pair(ff, 1024, "ETDRK4", T=np.float32, nu=1e-4, mu=1e-2, dt=2e-3, seed=9)
    # the initial field is dealiased to round-off; make it exact so the check below is too
    ff.dealias_(p64.sol, p64.grid)
    ff.dealias_(p32.sol, p32.grid)
    E = [ff.Vorticity.energy(p64)]
    for _ in range(5):
        ff.stepforward_(p64, 4)
        ff.stepforward_(p32, 4)
        E.append(ff.Vorticity.energy(p64))
    assert all(b < a for a, b in zip(E, E[1:]))
    s = ff.to_numpy(p64.sol)
    g = p64.grid
    assert np.abs(s[g.kralias.start:, :]).max() == 0
    assert np.abs(s[:, g.lalias.start:g.lalias.stop]).max() == 0
    assert rel(ff.to_numpy(p32.sol).astype(np.complex128), s) < 1e-5


def test_autotune_keeps_results(ff, cuda):
    """Every autotuner candidate computes the same step (tile shapes and radix orders
    only change the schedule); the chosen configuration reproduces the oracle."""
    prob, oprob = make_pair(ff, 64, "ETDRK4")
    bound = prob.timestepper._native(prob.eqn)
    fs = bound.ensure(prob.sol, prob.clock)
    start = prob.sol.clone()
    fs.autotune(steps_per_trial=1)
    prob.sol.copy_(start)
    ff.stepforward_(prob, 5)
    orc.stepforward(oprob, 5)
    assert rel(ff.to_numpy(prob.sol), oprob.sol) < 1e-12
    for cfg in [(1, 1, 1, 0), (4, 2, 4, 1), (2, 4, 2, 2)]:
        fs.set_config(*cfg)
        prob.sol.copy_(start)
        fs.advance(5)
        assert rel(ff.to_numpy(prob.sol), oprob.sol) < 1e-12, cfg


@pytest.mark.parametrize("stepper", ["ETDRK4", "FilteredETDRK4", "RK4", "LSRK54", "FilteredLSRK54"])
def test_split_pass_c_matches_unsplit(ff, cuda, stepper):
    """FP64 pass C split by field (two work items per kept column tile; the second to
    finish forms the flux from both transforms and runs the epilogue) against the unsplit
    form and the oracle, at one, two and four columns per tile (the last kept tile then
    also holds aliased columns).  The two forms' kernels may round the flux differently, so
    they are compared to rounding, not bit for bit.  Twenty graph replays from the same
    state give the same result each time: the arrival counters are reset by every launch."""
    prob, oprob = make_pair(ff, 128, stepper, ny=64)  # power-of-two lengths: the register path
    fs = prob.timestepper._native(prob.eqn).ensure(prob.sol, prob.clock)
    start = prob.sol.clone()
    orc.stepforward(oprob, 20)
    outs = {}
    for split in (0, 1):
        fs.set_split(split)
        for tiles in ((1, 1, 1), (2, 2, 2), (4, 4, 1)):
            fs.set_config(*tiles, 0)
            assert fs.config()["split_c"] == split
            prob.sol.copy_(start)
            fs.advance(20)
            got = ff.to_numpy(prob.sol)
            assert rel(got, oprob.sol) < 1e-12, (split, tiles)
            outs[(split, tiles)] = got
        prob.sol.copy_(start)
        fs.advance(20)
        assert np.array_equal(ff.to_numpy(prob.sol), outs[(split, (4, 4, 1))])
    assert rel(outs[(1, (1, 1, 1))], outs[(0, (1, 1, 1))]) < 1e-14
    # automatic choice: one small problem has few kept column tiles, so pass C is split
    fs.set_split(-1)
    assert fs.config()["split_c"] == 1


def test_split_pass_c_ensemble_and_fp32(ff, cuda):
    """The split pass C over an uneven FP64 ensemble (arrival counters per problem and
    tile) matches every member's oracle run; FP32, whose pass C runs the next pass A, never
    splits."""
    spec = [(32, 1e-3, 5), (128, 3e-4, 6), (64, 1e-4, 7), (256, 2e-4, 9)]
    ens = ff.Vorticity.Ensemble(spec, mu=1e-2, dt=2e-3, T=np.float64)
    ens.fs.set_split(1)
    assert ens.fs.config()["split_c"] == 1
    ens.stepforward_(8)
    for (n, nu, seed), m in zip(spec, ens.members):
        z0 = ff.Vorticity.random_phase_vorticity(n, seed=seed)
        op = orc.VorticityProblem(n, 2 * math.pi, nu, 1e-2, 2e-3, "ETDRK4")
        op.sol[...] = orc.rfft(z0)
        orc.stepforward(op, 8)
        assert rel(ff.to_numpy(m.sol), op.sol) < 1e-12, (n, nu)
    prob, _ = make_pair(ff, 64, "ETDRK4", T=np.float32)
    fs = prob.timestepper._native(prob.eqn).ensure(prob.sol, prob.clock)
    fs.set_split(1)
    assert fs.config()["split_c"] == 0


def test_bound_calcN_slots(ff, cuda):
    """calcN! from a bound slot equals the staged call bit for bit; a geometry change
    invalidates the slot until it is bound again; bad slots are rejected."""
    for T in (np.float64, np.float32):
        prob, oprob = make_pair(ff, 128, "ETDRK4", T=T, ny=64)
        g = prob.grid
        fs = ff.Vorticity.calcN_._handle(g, prob.sol)
        Ct = np.complex128 if T == np.float64 else np.complex64
        N0 = ff.zeros(ff.GPU(), Ct, (g.nkr, g.ny))
        N1 = ff.zeros(ff.GPU(), Ct, (g.nkr, g.ny))
        fs.calcN(N0, prob.sol)
        fs.calcN_bind(3, N1, prob.sol)
        fs.calcN_slot(3)
        assert np.array_equal(ff.to_numpy(N0), ff.to_numpy(N1))
        No = np.zeros_like(oprob.sol)
        orc.vorticity_calcN(No, oprob.sol, 0.0, None, None, None, oprob.grid)
        assert rel(ff.to_numpy(N1).astype(np.complex128), No) < (1e-13 if T == np.float64 else 1e-5)
        fs.set_config(2, 2, 2, 0)
        with pytest.raises(ValueError, match="bind it again"):
            fs.calcN_slot(3)
        N1.zero_()
        fs.calcN_bind(3, N1, prob.sol)
        fs.calcN_slot(3)
        fs.calcN(N0, prob.sol)
        assert np.array_equal(ff.to_numpy(N0), ff.to_numpy(N1))
        with pytest.raises(ValueError):
            fs.calcN_slot(7)  # never bound
        with pytest.raises(ValueError):
            fs.calcN_bind(ff._lib.FF_VORT_CALC_SLOTS, N1, prob.sol)


def test_long_horizon_energy_enstrophy_series_fp64(ff, cuda):
    """Over a long horizon (2000 ETDRK4 steps, t = 4, the plain configuration's ν, μ, dt at
    256²) the FP64 GPU path's energy and enstrophy series match the oracle's, every 100
    steps, to 1e-10 relative, and the states to 1e-9 (trajectories of this flow stay
    close in FP64 over this horizon)."""
    prob, oprob = make_pair(ff, 256, "ETDRK4", nu=1e-4, mu=1e-2, dt=2e-3, seed=2026)
    worst_E = worst_Z = 0.0
    for _ in range(20):
        ff.stepforward_(prob, 100)
        orc.stepforward(oprob, 100)
        E, Eo = ff.Vorticity.energy(prob), orc.vorticity_energy(oprob.sol, oprob.grid)
        Z, Zo = ff.Vorticity.enstrophy(prob), orc.vorticity_enstrophy(oprob.sol, oprob.grid)
        worst_E = max(worst_E, abs(E - Eo) / Eo)
        worst_Z = max(worst_Z, abs(Z - Zo) / Zo)
    assert prob.clock.step == 2000
    assert worst_E < 1e-10 and worst_Z < 1e-10, (worst_E, worst_Z)
    assert rel(ff.to_numpy(prob.sol), oprob.sol) < 1e-9


@pytest.mark.parametrize("n,ny", [(4096, 32), (32, 4096)])
def test_register_path_maximum_lengths(ff, cuda, n, ny):
    """The longest lines the register-resident kernels take: rows of nx/2 = 2048 and
    columns of ny = 4096, FP64, three ETDRK4 steps against the oracle."""
    prob, oprob = make_pair(ff, n, "ETDRK4", ny=ny, dt=1e-4)
    ff.stepforward_(prob, 3)
    assert prob.timestepper._native(prob.eqn).fs.config()["radix_order"] == -1
    orc.stepforward(oprob, 3)
    assert rel(ff.to_numpy(prob.sol), oprob.sol) < 1e-12


@pytest.mark.parametrize("stepper", ["ETDRK4", "FilteredETDRK4", "RK4", "FilteredRK4", "LSRK54"])
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_state_with_aliased_modes(ff, cuda, stepper, T):
    """A state with energy in the aliased modes (which the nonlinear term never sees and
    which evolve by the linear part alone): the fused ETDRK4 and RK4 paths skip the
    aliased columns and rows in the first three substeps and must still match the oracle
    everywhere."""
    n, ny = 128, 96
    prob, oprob = make_pair(ff, n, stepper, T=T, ny=ny)
    rng = np.random.default_rng(77)
    s0 = oprob.sol + 1e-2 * (rng.standard_normal(oprob.sol.shape) + 1j * rng.standard_normal(oprob.sol.shape))
    s0[0, 0] = 0
    oprob.sol[...] = s0.astype(np.complex64 if T == np.float32 else np.complex128)
    prob.sol.copy_(ff.device_array(ff.GPU())(oprob.sol))
    ff.stepforward_(prob, 10)
    orc.stepforward(oprob, 10)
    got = ff.to_numpy(prob.sol).astype(np.complex128)
    tol = 1e-12 if T == np.float64 else 1e-5
    assert rel(got, oprob.sol) < tol
    g = prob.grid
    # the aliased modes alone, against the oracle's
    assert rel(got[g.kralias.start:, :], oprob.sol[g.kralias.start:, :]) < tol
    assert rel(got[:g.kralias.start, g.lalias.start:g.lalias.stop],
               oprob.sol[:g.kralias.start, g.lalias.start:g.lalias.stop]) < tol


def test_profile_pass_times(ff, cuda):
    """ff_vort_profile on ETDRK4 and RK4 handles (state untouched); an LSRK54 stage would
    advance the state, so that handle is refused."""
    # 64^2: the register path (FP32: pass C fused with the next pass A); 48^2: the generic
    # shared-memory path (radix 3), where pass C runs over every column tile unfused
    cases = [(64, "ETDRK4", np.float64), (64, "ETDRK4", np.float32), (64, "RK4", np.float32),
             (64, "RK4", np.float64), (48, "ETDRK4", np.float64), (48, "RK4", np.float32)]
    for n, stepper, T in cases:
        prob, _ = make_pair(ff, n, stepper, T=T)
        ff.stepforward_(prob, 1)
        fs = prob.timestepper._native(prob.eqn).fs
        assert (fs.config()["radix_order"] == -1) == (n == 64)
        before = ff.to_numpy(prob.sol)
        ms = fs.profile(reps=2)
        assert len(ms) == 3 and all(t > 0 for t in ms), (n, stepper, T)
        assert np.array_equal(ff.to_numpy(prob.sol), before), (n, stepper, T)
    prob, _ = make_pair(ff, 64, "LSRK54")
    ff.stepforward_(prob, 1)
    with pytest.raises(Exception, match="ETDRK4 and RK4"):
        prob.timestepper._native(prob.eqn).fs.profile(reps=1)
