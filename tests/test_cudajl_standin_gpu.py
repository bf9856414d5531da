"""The comparator arm: the unfused FP64 restatement of FourierFlows.jl's GPU path (one kernel
per broadcast, cuFFT plans; baseline/cudajl_standin) computes the same ETDRK4 step as the
oracle and as the library's fused path, so that bench.py times like against like."""
import math

import numpy as np
import pytest

from oracle import ff_oracle as orc

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.mark.parametrize("n", [64, 256])
def test_standin_matches_oracle_and_fused_path(ff, cuda, n):
    from baseline.cudajl_standin.standin import UnfusedETDRK4
    nu, mu, dt, steps = 1e-4, 1e-2, 2e-3, 10
    z0 = ff.Vorticity.random_phase_vorticity(n, seed=41)
    prob = ff.Vorticity.Problem(ff.GPU(), nx=n, Lx=2 * math.pi, nu=nu, mu=mu, dt=dt, stepper="ETDRK4")
    ff.Vorticity.set_zeta_(prob, z0)
    state = prob.sol.clone()
    u = UnfusedETDRK4(prob)
    u.step(state, steps)
    ff.stepforward_(prob, steps)
    cuda.cuda.synchronize()
    op = orc.VorticityProblem(n, 2 * math.pi, nu, mu, dt, "ETDRK4")
    op.sol[...] = orc.rfft(z0)
    orc.stepforward(op, steps)
    got = ff.to_numpy(state)
    assert rel(got, op.sol) < 1e-12
    assert rel(got, ff.to_numpy(prob.sol)) < 1e-12
    # 4 calcN! of 18 launches (cuFFT executions counted once each) + 4 ETDRK4 broadcasts
    assert u.launches_per_step == 76
