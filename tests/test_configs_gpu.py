"""The benchmark configurations at their stated sizes and horizons, against the CPU oracle.

* Plain FP64, 1024^2 (nu = 1e-4, mu = 1e-2, ETDRK4, dt = 2e-3): 100 steps, relative L2 of
  the state <= 1e-12 and energy / enstrophy within 1e-12 (the bar for the FP64 path over
  short horizons, before chaotic divergence).
* FP32 state and transforms on the same problem: 100 steps against the FP64 oracle,
  relative L2 <= 1e-5 and energy / enstrophy within 1e-5.
* A batched FP32 ensemble with 1024^2 and 512^2 members (and smaller ones, each with its
  own viscosity): 100 steps, every member against its own FP64 oracle run, <= 1e-5.
* The precision form's 2048^2 grid: FP32 ETDRK4 (dt = 1e-3) for 100 steps against the
  FP64 oracle, <= 1e-5.

The oracle is the numpy / scipy.fft restatement of the reference's ETDRK4 step
(src/timesteppers.jl:518-547) with the vorticity nonlinear term built on the reference's
Jacobian (src/utils.jl:190-205)."""
import math
import os

import numpy as np
import pytest

from oracle import ff_oracle as orc

pytestmark = pytest.mark.gpu

NU, MU, DT, SEED = 1e-4, 1e-2, 2e-3, 20260101


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.fixture(scope="module", autouse=True)
def oracle_threads():
    """scipy.fft threads for the oracle's large grids (restored afterwards)."""
    before = orc.WORKERS
    orc.set_workers(os.cpu_count() or 1)
    yield
    orc.set_workers(before)


def oracle_run(z0, n, nu, steps, dt=DT, stepper="ETDRK4", **kw):
    op = orc.VorticityProblem(n, 2 * math.pi, nu, MU, dt, stepper, **kw)
    op.sol[...] = orc.rfft(z0)
    orc.stepforward(op, steps)
    return op


@pytest.fixture(scope="module")
def oracle_1024_100(ff):
    """The FP64 oracle's 1024^2 run of the plain configuration: state after 100 steps."""
    z0 = ff.Vorticity.random_phase_vorticity(1024, seed=SEED)
    return z0, oracle_run(z0, 1024, NU, 100)


def test_plain_fp64_1024_100_steps(ff, cuda, oracle_1024_100):
    z0, op = oracle_1024_100
    prob = ff.Vorticity.Problem(ff.GPU(), nx=1024, Lx=2 * math.pi, nu=NU, mu=MU, dt=DT, stepper="ETDRK4")
    ff.Vorticity.set_zeta_(prob, z0)
    ff.stepforward_(prob, 100)
    assert prob.clock.step == 100
    e = rel(ff.to_numpy(prob.sol), op.sol)
    assert e < 1e-12, e
    E, Eo = ff.Vorticity.energy(prob), orc.vorticity_energy(op.sol, op.grid)
    Z, Zo = ff.Vorticity.enstrophy(prob), orc.vorticity_enstrophy(op.sol, op.grid)
    assert abs(E - Eo) / Eo < 1e-12 and abs(Z - Zo) / Zo < 1e-12, (E, Eo, Z, Zo)


def test_fp32_1024_100_steps_vs_fp64_oracle(ff, cuda, oracle_1024_100):
    z0, op = oracle_1024_100
    prob = ff.Vorticity.Problem(ff.GPU(), nx=1024, Lx=2 * math.pi, nu=NU, mu=MU, dt=DT, stepper="ETDRK4",
                                T=np.float32)
    ff.Vorticity.set_zeta_(prob, z0)
    ff.stepforward_(prob, 100)
    e = rel(ff.to_numpy(prob.sol).astype(np.complex128), op.sol)
    assert e < 1e-5, e
    E, Eo = ff.Vorticity.energy(prob), orc.vorticity_energy(op.sol, op.grid)
    Z, Zo = ff.Vorticity.enstrophy(prob), orc.vorticity_enstrophy(op.sol, op.grid)
    assert abs(E - Eo) / Eo < 1e-5 and abs(Z - Zo) / Zo < 1e-5, (E, Eo, Z, Zo)


def test_batched_fp32_ensemble_with_1024_and_512_members_100_steps(ff, cuda):
    """One persistent launch per pass over members of four sizes and five viscosities; two
    members share size and viscosity (and so their coefficient arrays)."""
    spec = [(1024, 1e-4, 11), (512, 3e-4, 12), (1024, 2e-5, 13), (256, 1e-4, 14), (512, 3e-4, 15),
            (128, 1e-3, 16)]
    ens = ff.Vorticity.Ensemble(spec, mu=MU, dt=DT, T=np.float32)
    assert ens.members[4].coefs[0] is ens.members[1].coefs[0]
    ens.stepforward_(100)
    for (n, nu, seed), m in zip(spec, ens.members):
        z0 = ff.Vorticity.random_phase_vorticity(n, seed=seed)
        op = oracle_run(z0.astype(np.float32).astype(np.float64), n, nu, 100)
        e = rel(ff.to_numpy(m.sol).astype(np.complex128), op.sol)
        assert e < 1e-5, (n, nu, e)


def test_precision_form_2048_fp32_100_steps_vs_fp64_oracle(ff, cuda):
    """FP32 ETDRK4 on the 2048^2 grid (dt = 1e-3) against the FP64 oracle after 100 steps."""
    n, dt = 2048, 1e-3
    z0 = ff.Vorticity.random_phase_vorticity(n, seed=SEED)
    prob = ff.Vorticity.Problem(ff.GPU(), nx=n, Lx=2 * math.pi, nu=NU, mu=MU, dt=dt, stepper="ETDRK4", T=np.float32)
    ff.Vorticity.set_zeta_(prob, z0)
    ff.stepforward_(prob, 100)
    op = oracle_run(z0, n, NU, 100, dt=dt)
    e = rel(ff.to_numpy(prob.sol).astype(np.complex128), op.sol)
    assert e < 1e-5, e
