"""Why the precision form runs its 2048^2 grid at dt = 1e-3 rather than 2e-3 (CPU).

At 2048^2 the kept wavenumbers reach k_max = 682 and the initial velocity |u|_max ~ 2.8,
so dt = 2e-3 gives an advective number k_max |u|_max dt ~ 3.8, past the interval of the
imaginary axis inside ETDRK4's (and RK4's) stability region (~2.8).  The FP64 oracle
itself, the restatement of the reference's ETDRK4 step (src/timesteppers.jl:518-547),
blows up there within 20 steps; at 1024^2 (k_max = 341) the same dt is stable.  The GPU
paths are compared against the oracle at dt = 1e-3 (tests/test_configs_gpu.py)."""
import math
import os

import numpy as np

from oracle import ff_oracle as orc


def test_oracle_2048_blows_up_at_dt_2e_3():
    import fourierflows.jl_gb300.vorticity as vort
    before = orc.WORKERS
    orc.set_workers(os.cpu_count() or 1)
    try:
        n = 2048
        z0 = vort.random_phase_vorticity(n, seed=20260101)
        op = orc.VorticityProblem(n, 2 * math.pi, 1e-4, 1e-2, 2e-3, "ETDRK4")
        op.sol[...] = orc.rfft(z0)
        E0 = orc.vorticity_energy(op.sol, op.grid)
        series = []
        with np.errstate(over="ignore", invalid="ignore"):
            for _ in range(20):
                orc.stepforward(op, 1)
                series.append(orc.vorticity_energy(op.sol, op.grid))
                if not np.isfinite(series[-1]) or series[-1] > 10 * E0:
                    break
    finally:
        orc.set_workers(before)
    # the first steps decay as the viscous, damped flow should ...
    assert all(b < a for a, b in zip([E0] + series[:10], series[:10]))
    # ... then the kept modes past the stability limit take over within 20 steps
    assert not np.isfinite(series[-1]) or series[-1] > 10 * E0, series
    assert len(series) <= 20
