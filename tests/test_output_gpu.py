"""saveoutput from a stepping GPU problem: the asynchronous device -> pinned host -> file
path stores each snapshot as it was when saveoutput was called, while stepping goes on."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_saveoutput_snapshots_while_stepping(ff, cuda, tmp_path):
    prob = ff.Diffusion.Problem(ff.GPU(), nx=128, Lx=2 * math.pi, kappa=1e-2, dt=1e-2, stepper="ETDRK4")
    x = ff.to_numpy(prob.grid.x) if hasattr(prob.grid.x, "device") else np.asarray(prob.grid.x)
    ff.Diffusion.set_c_(prob, np.exp(-x ** 2 / (2 * 0.3 ** 2)))
    out = ff.Output(prob, str(tmp_path / "diffusion.jld2"), ("sol", lambda p: p.sol), ("c", lambda p: p.vars.c))
    ff.saveproblem(out)
    expected = {}
    for k in range(5):
        ff.Diffusion.updatevars_(prob)
        ff.saveoutput(out)  # returns at once; the next steps overwrite sol while it is written
        expected[prob.clock.step] = (ff.to_numpy(prob.sol), ff.to_numpy(prob.vars.c), prob.clock.t)
        ff.stepforward_(prob, 7)
    out.flush()
    f = ff.openoutput(out.path)
    assert sorted(int(s) for s in f["snapshots"]["sol"]) == sorted(expected)
    for step, (sol, c, t) in expected.items():
        assert np.array_equal(f["snapshots"]["sol"][str(step)], sol)
        assert np.array_equal(f["snapshots"]["c"][str(step)], c)
        assert f["snapshots"]["t"][str(step)] == t
    assert np.array_equal(f["eqn"]["L"], ff.to_numpy(prob.eqn.L))
    assert f["grid"]["nx"] == 128
