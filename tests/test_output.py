"""Output / saveoutput / saveproblem / savediagnostic (src/output.jl), after the reference's
test/test_output.jl: path handling and the stored keys, on host arrays (no GPU)."""
import math
import os

import numpy as np
import pytest


def test_withoutjld2(ff):
    assert ff.withoutjld2("blahblah.jld2") == "blahblah"
    assert ff.withoutjld2("blahblah") == "blahblah"


def test_uniquepath(ff, tmp_path):
    path = str(tmp_path / "foo.jld2")
    open(path, "w").close()
    assert ff.uniquepath(path) == str(tmp_path / "foo_1.jld2")
    open(str(tmp_path / "foo_1.jld2"), "w").close()
    assert ff.uniquepath(path) == str(tmp_path / "foo_2.jld2")


class _Clock:
    def __init__(self):
        self.t, self.step, self.dt = 0.0, 0, 1e-7


class _Eqn:
    def __init__(self, n):
        self.L = -1e-2 * np.arange(n // 2 + 1, dtype=np.float64) ** 2
        self.dims = (n // 2 + 1,)
        self.T = np.complex128


class _Params:
    def __init__(self):
        self.kappa = 1e-2
        self.func = math.sin  # functions are not stored (forbidden_output_types)


class _Prob:
    """A host stand-in for a OneDGrid Diffusion problem."""

    def __init__(self, ff, n=32):
        self.grid = ff.OneDGrid(ff.CPU(), nx=n, Lx=2 * math.pi)
        self.clock, self.eqn, self.params = _Clock(), _Eqn(n), _Params()
        self.c = np.zeros(n)
        self.c[2] = math.pi


def test_output_constructor_and_getindex(ff, tmp_path):
    prob = _Prob(ff)
    out1 = ff.Output(prob, str(tmp_path / "testoutput.jld2"), ("c", lambda p: p.c))
    out2 = ff.Output(prob, str(tmp_path / "testoutput.jld2"), {"c": lambda p: p.c, "sol": lambda p: 2 * p.c})
    assert out1.path.endswith("testoutput.npz") and list(out2.fields) == ["c", "sol"]
    assert np.array_equal(out1["c"], prob.c) and np.array_equal(out2[":sol"], 2 * prob.c)
    assert repr(out1).startswith("Output\n  ├──── prob: _Prob\n")


def test_saveproblem_saveoutput_savediagnostic(ff, tmp_path):
    prob = _Prob(ff)
    out = ff.Output(prob, str(tmp_path / "testoutput.jld2"), ("c", lambda p: p.c.copy()))
    ff.saveproblem(out)
    for step in range(3):
        prob.clock.step, prob.clock.t = step, step * prob.clock.dt
        prob.c[3] = step
        ff.saveoutput(out)

    class _Diag:
        i = 3
        steps = [0, 2, 4, 6]
        t = [0.0, 0.2, 0.4, 0.6]
        data = [np.ones(2) * k for k in range(4)]

    ff.savediagnostic(_Diag(), "mydiagnostic", out.path)
    f = ff.openoutput(out.path)
    assert os.path.isfile(out.path)
    assert f["grid"]["Lx"] == pytest.approx(2 * math.pi) and np.array_equal(f["grid"]["x"], prob.grid.x)
    assert np.array_equal(f["eqn"]["L"], prob.eqn.L) and tuple(f["eqn"]["dims"]) == (17,)
    assert f["clock"]["dt"] == 1e-7 and f["params"]["kappa"] == 1e-2 and "func" not in f["params"]
    for step in range(3):
        assert f["snapshots"]["c"][str(step)][3] == step and f["snapshots"]["c"][str(step)][2] == math.pi
        assert f["snapshots"]["t"][str(step)] == step * 1e-7
    d = f["diagnostics"]["mydiagnostic"]
    assert list(d["steps"]) == [0, 2, 4] and d["data"].shape == (3, 2)
