"""ff_parsevalsum2_noalloc: the Parseval sum for callers that cannot call cudaMalloc
(their device memory belongs to another allocator).  It must agree with the allocating
ff_parsevalsum2 on consecutive calls, so that the shared static scratch never leaks one
call's partial sums into the next.  This file is collected last on purpose."""
import ctypes as C
import math

import numpy as np
import pytest


def _noalloc(ff, code, uh, n0, nrest, rfft_form, norm, out):
    ff._lib.call("ff_parsevalsum2_noalloc", code, C.c_void_p(uh.data_ptr()), n0, nrest, rfft_form, norm,
                 C.c_void_p(out.data_ptr()), ff.devices.stream_handle())


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_noalloc_parseval_matches_allocating_version(ff, cuda, prec):
    """Two calls in a row (the second on a larger input), each against the allocating
    ff_parsevalsum2 and against the oracle's parsevalsum2 (src/utils.jl:113-139) on the
    host copy of the same values.  n0 = nkr = 257 is odd."""
    from oracle import ff_oracle as orc
    torch = cuda
    T = np.float64 if prec == "f64" else np.float32
    cdt = torch.complex128 if prec == "f64" else torch.complex64
    code = ff._lib.FF_F64 if prec == "f64" else ff._lib.FF_F32
    tol = 1e-13 if prec == "f64" else 1e-6
    g = ff.TwoDGrid(ff.GPU(), nx=512, Lx=2 * math.pi, ny=384, Ly=3.0, T=T)
    og = orc.TwoDGrid(512, 2 * math.pi, 384, 3.0)
    norm = float(g.Lx) * float(g.Ly) / (g.nx ** 2 * g.ny ** 2)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(17)
    for shape in [(g.nkr, g.ny), (g.nkr, g.ny, 3)]:
        x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        uh = ff.device_array(ff.GPU())(x.astype(np.complex128 if prec == "f64" else np.complex64))
        assert uh.dtype == cdt
        n0, nrest = shape[0], int(np.prod(shape[1:]))
        _noalloc(ff, code, uh, n0, nrest, 1, norm, out)
        torch.cuda.synchronize()
        got = float(out.item())
        ref = C.c_double()
        ff._lib.call("ff_parsevalsum2", code, C.c_void_p(uh.data_ptr()), n0, nrest, 1, norm, C.byref(ref),
                     ff.devices.stream_handle())
        assert abs(got - ref.value) <= tol * abs(ref.value), (shape, got, ref.value)
        host = ff.to_numpy(uh).astype(np.complex128)
        want = orc.parsevalsum2(host.reshape(n0, -1), og)
        assert abs(got - want) <= tol * abs(want), (shape, got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("n0,nrest", [(96, 40), (75, 33)])
def test_noalloc_parseval_full_spectrum_form(ff, cuda, n0, nrest):
    """rfft_form = 0 (a full complex spectrum: every row counted once), even and odd n0,
    against the oracle's plain sum of |u|^2."""
    from oracle import ff_oracle as orc
    torch = cuda
    # any grid whose nkr differs from n0 sends the oracle down its full-spectrum branch; its
    # normalisation is divided out below
    og = orc.TwoDGrid(2 * n0, 2 * math.pi, nrest + nrest % 2, 2 * math.pi)
    assert og.nkr != n0
    norm = 0.37
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    x = np.random.default_rng(n0).standard_normal((n0, nrest)) + 1j * np.random.default_rng(nrest).standard_normal(
        (n0, nrest))
    uh = ff.device_array(ff.GPU())(x)
    for _ in range(2):
        _noalloc(ff, ff._lib.FF_F64, uh, n0, nrest, 0, norm, out)
        torch.cuda.synchronize()
        got = float(out.item())
        want = float(np.sum(np.abs(x) ** 2)) * norm
        assert abs(got - want) <= 1e-13 * want
        oracle_sum = orc.parsevalsum2(x, og) / (og.Lx * og.Ly / (og.nx ** 2 * og.ny ** 2))
        assert abs(got - oracle_sum * norm) <= 1e-13 * want


def test_noalloc_parseval_rejects_oversized_input(ff):
    """The size check precedes any CUDA call, so this runs without a GPU."""
    out = C.c_double()
    with pytest.raises(ValueError) as e:
        ff._lib.call("ff_parsevalsum2_noalloc", ff._lib.FF_F64, C.c_void_p(16), 8193, 4096, 1, 1.0, C.byref(out),
                     None)
    assert "exceed the maximum" in str(e.value)
