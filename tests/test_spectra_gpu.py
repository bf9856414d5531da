"""radialspectrum on the GPU (one native binned reduction) against the oracle and against
the reference's own known answers (test/runtests.jl:297-307)."""
import math

import numpy as np
import pytest

from oracle import ff_oracle as orc

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.mark.parametrize("rfft_form", [True, False])
@pytest.mark.parametrize("complex_input", [True, False])
@pytest.mark.parametrize("T", [np.float64, np.float32])
@pytest.mark.parametrize("nx,ny,Ly", [(64, 64, 2 * math.pi), (96, 48, 3.0)])
def test_radialspectrum_vs_oracle(ff, cuda, rfft_form, complex_input, T, nx, ny, Ly):
    grid = ff.TwoDGrid(ff.GPU(), nx=nx, ny=ny, Lx=2 * math.pi, Ly=Ly, T=T)
    g = orc.Grid(2, (nx, ny), (float(grid.Lx), float(grid.Ly)))  # the grid's own (FP32-rounded) lengths
    rng = np.random.default_rng(nx + ny)
    shape = (nx // 2 + 1 if rfft_form else nx, ny)
    fh = rng.standard_normal(shape) + (1j * rng.standard_normal(shape) if complex_input else 0)
    ctype = (np.complex128 if T == np.float64 else np.complex64) if complex_input else T
    fh = fh.astype(ctype)
    rho, out = ff.radialspectrum(ff.device_array(ff.GPU())(fh), grid, refinement=3)
    rho_o, out_o = orc.radialspectrum(fh.astype(np.complex128 if complex_input else np.float64), g, refinement=3)
    assert np.allclose(rho, rho_o, rtol=1e-15, atol=0)
    got = ff.to_numpy(out)
    assert got.dtype == ctype
    tol = 1e-12 if T == np.float64 else 1e-6
    assert rel(got, out_o) < tol
    assert got[0] == fh[0, 0]


@pytest.mark.parametrize("rfft_form", [True, False])
def test_radialspectrum_known_answers(ff, cuda, rfft_form):
    """The reference's isotropic and anisotropic Gaussian spectra at n = 128, refinement 16."""
    n, d = 128, 128 / 10
    grid = ff.TwoDGrid(ff.GPU(), nx=n, Lx=2 * math.pi)
    g = orc.Grid(2, (n, n), (2 * math.pi, 2 * math.pi))
    K = g.kr if rfft_form else g.k
    kk, ll = K + 0 * g.l, 0 * K + g.l
    with np.errstate(invalid="ignore", divide="ignore"):
        cases = [(np.exp(-(kk ** 2 + ll ** 2) / (2 * d ** 2)), lambda r: 2 * np.pi * r * np.exp(-r ** 2 / (2 * d ** 2))),
                 (np.exp(-(kk ** 2 + ll ** 2) / (2 * d ** 2)) * kk ** 2 / (kk ** 2 + ll ** 2),
                  lambda r: np.pi * r * np.exp(-r ** 2 / (2 * d ** 2)))]
    for ah, ar in cases:
        ah = np.asfortranarray(ah.astype(np.float64))
        ah[0, 0] = 0.0
        rho, est = ff.radialspectrum(ff.device_array(ff.GPU())(ah), grid, refinement=16)
        est = ff.to_numpy(est)
        assert np.sum(np.abs(ar(rho) - est)) / len(rho) < 0.1
        _, est_o = orc.radialspectrum(ah, g, refinement=16)
        assert rel(est, est_o) < 1e-12


def test_radialspectrum_rejects_bad_shapes(ff, cuda):
    grid = ff.TwoDGrid(ff.GPU(), nx=32, Lx=2 * math.pi)
    bad = ff.zeros(ff.GPU(), np.complex128, (20, 32))
    with pytest.raises(ValueError):
        ff.radialspectrum(bad, grid)
