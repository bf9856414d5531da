"""FFT plans on the GPU: the reference's analytic known-answer tests
(test/createffttestfunctions.jl, test/test_fft.jl, test/test_ifft.jl; rtol_fft = 1e-12,
test/runtests.jl:21) and random-field parity against the CPU oracle."""
import math

import numpy as np
import pytest

from oracle import ff_oracle as orc

pytestmark = pytest.mark.gpu

RTOL_FFT = 1e-12


def isapprox(a, b, rtol=1e-8, atol=0.0):
    """Julia's isapprox for arrays: norm(a - b) <= max(atol, rtol * max(norm(a), norm(b)))."""
    a, b = np.asarray(a), np.asarray(b)
    d = np.linalg.norm(a - b)
    return d <= max(atol, rtol * max(np.linalg.norm(a), np.linalg.norm(b)))


def _grid(ff, ndim, n, L, T=np.float64):
    if ndim == 1:
        return ff.OneDGrid(ff.GPU(), nx=n[0], Lx=L[0], T=T)
    if ndim == 2:
        return ff.TwoDGrid(ff.GPU(), nx=n[0], Lx=L[0], ny=n[1], Ly=L[1], T=T)
    return ff.ThreeDGrid(ff.GPU(), nx=n[0], Lx=L[0], ny=n[1], Ly=L[1], nz=n[2], Lz=L[2], T=T)


def _testfuncs(g):
    """The analytic functions and transforms of test/createffttestfunctions.jl:71-209."""
    if g.ndim == 1:
        m, phi = 5, math.pi / 3
        k0 = g.k_host[1]
        x = g.x
        f1 = np.cos(m * k0 * x + phi)
        kk = g.k_host.reshape(-1)
        f1h = np.zeros(g.nx, complex)
        f1hr = np.zeros(g.nkr, complex)
        for i in range(g.nk):
            if abs(kk[i]) == m * k0:
                f1h[i] = -np.exp(np.sign(kk[i]) * 1j * phi) * g.nx / 2
        krr = g.kr_host.reshape(-1)
        for i in range(g.nkr):
            if abs(kk[i]) == m * k0:
                f1hr[i] = -np.exp(np.sign(krr[i]) * 1j * phi) * g.nx / 2
        return [(f1, f1h, f1hr)]
    if g.ndim == 2:
        m, n = 5, 2
        k0, l0 = g.k_host[1, 0], g.l_host[0, 1]
        X, Y = np.meshgrid(g.x, g.y, indexing="ij")
        f1 = np.cos(m * k0 * X) * np.cos(n * l0 * Y)
        f2 = np.sin(m * k0 * X + n * l0 * Y)
        k, l, kr = g.k_host.reshape(-1), g.l_host.reshape(-1), g.kr_host.reshape(-1)
        f1h = np.zeros((g.nk, g.nl), complex)
        f2h = np.zeros((g.nk, g.nl), complex)
        f1hr = np.zeros((g.nkr, g.nl), complex)
        f2hr = np.zeros((g.nkr, g.nl), complex)
        nx, ny = g.nx, g.ny
        for j in range(g.nl):
            for i in range(g.nk):
                if abs(k[i]) == m * k0 and abs(l[j]) == n * l0:
                    f1h[i, j] = -nx * ny / 4
                if k[i] == m * k0 and l[j] == n * l0:
                    f2h[i, j] = -nx * ny / 2
                elif k[i] == -m * k0 and l[j] == -n * l0:
                    f2h[i, j] = nx * ny / 2
            for i in range(g.nkr):
                if abs(kr[i]) == m * k0 and abs(l[j]) == n * l0:
                    f1hr[i, j] = -nx * ny / 4
                if kr[i] == m * k0 and l[j] == n * l0:
                    f2hr[i, j] = -nx * ny / 2
        return [(f1, f1h, f1hr), (f2, -1j * f2h, -1j * f2hr)]
    mx, my, mz = 5, 2, 3
    k0, l0, m0 = g.k_host[1, 0, 0], g.l_host[0, 1, 0], g.m_host[0, 0, 1]
    X, Y, Z = np.meshgrid(g.x, g.y, g.z, indexing="ij")
    f1 = np.cos(mx * k0 * X) * np.cos(my * l0 * Y) * np.cos(mz * m0 * Z)
    f2 = np.sin(mx * k0 * X + my * l0 * Y + mz * m0 * Z)
    k, l, mm, kr = g.k_host.reshape(-1), g.l_host.reshape(-1), g.m_host.reshape(-1), g.kr_host.reshape(-1)
    N = g.nx * g.ny * g.nz
    f1h = np.zeros((g.nk, g.nl, g.nm), complex)
    f2h = np.zeros_like(f1h)
    f1hr = np.zeros((g.nkr, g.nl, g.nm), complex)
    f2hr = np.zeros_like(f1hr)
    for c in range(g.nm):
        for j in range(g.nl):
            for i in range(g.nk):
                if abs(k[i]) == mx * k0 and abs(l[j]) == my * l0 and abs(mm[c]) == mz * m0:
                    f1h[i, j, c] = N / 8
                if k[i] == mx * k0 and l[j] == my * l0 and mm[c] == mz * m0:
                    f2h[i, j, c] = N / 2
                elif k[i] == -mx * k0 and l[j] == -my * l0 and mm[c] == -mz * m0:
                    f2h[i, j, c] = -N / 2
            for i in range(g.nkr):
                if abs(kr[i]) == mx * k0 and abs(l[j]) == my * l0 and abs(mm[c]) == mz * m0:
                    f1hr[i, j, c] = N / 8
                if kr[i] == mx * k0 and l[j] == my * l0 and mm[c] == mz * m0:
                    f2hr[i, j, c] = N / 2
    return [(f1, f1h, f1hr), (f2, -1j * f2h, -1j * f2hr)]


CASES = [(1, (32,), (2 * math.pi,)), (2, (32, 64), (2 * math.pi, 3 * math.pi)),
         (3, (32, 30, 16), (2 * math.pi, 3 * math.pi, 4.0))]


@pytest.mark.parametrize("ndim,n,L", CASES)
def test_known_answer_transforms(ff, cuda, ndim, n, L):
    """test_fft_*, test_rfft_*, test_rfft_mul_*, test_ifft_*, test_irfft_*, test_irfft_mul_*."""
    g = _grid(ff, ndim, n, L)
    dev = ff.device_array(ff.GPU())
    for f, fh_th, fhr_th in _testfuncs(g):
        fd = dev(f)
        fhr = ff.to_numpy(ff.rfft(fd))
        assert isapprox(fhr, fhr_th, RTOL_FFT)
        out = ff.zeros(ff.GPU(), np.complex128, g.spectral_shape)
        ff.mul_(out, g.rfftplan, fd)
        assert isapprox(ff.to_numpy(out), fhr_th, RTOL_FFT)
        fh = ff.to_numpy(ff.fft(dev(f.astype(complex))))
        assert isapprox(fh, fh_th, RTOL_FFT)
        # inverses of the analytic spectra (the reference inverts its computed ones)
        back = ff.zeros(ff.GPU(), np.float64, g.physical_shape)
        src = dev(fhr_th)
        ff.ldiv_(back, g.rfftplan, src)
        assert isapprox(ff.to_numpy(back), f, RTOL_FFT)
        assert np.array_equal(ff.to_numpy(src), fhr_th), "ldiv_ must not modify its input"
        assert isapprox(ff.to_numpy(ff.irfft(dev(fhr), g.nx)), f, RTOL_FFT)
        assert isapprox(np.real(ff.to_numpy(ff.ifft(dev(fh)))), f, RTOL_FFT)


SIZES = [(2,), (4,), (6,), (8,), (10,), (16,), (34,), (48,), (128,), (1024,), (4096,), (6, 8), (8, 8), (16, 32),
         (32, 30), (64, 128), (24, 40), (128, 128), (256, 512), (1024, 1024), (6, 8, 10), (16, 32, 34), (32, 30, 16),
         (8, 12, 20)]


@pytest.mark.parametrize("shape", SIZES, ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_random_rfft_vs_oracle(ff, cuda, shape, prec):
    T = np.float64 if prec == "f64" else np.float32
    tol = 1e-13 if prec == "f64" else 2e-6
    rng = np.random.default_rng(sum(shape) * 7 + len(shape))
    x = rng.standard_normal(shape)
    ref = orc.rfft(x)
    dev = ff.device_array(ff.GPU())
    plan = ff.RFFTPlan(shape, T)
    xd = dev(x.astype(T))
    out = ff.zeros(ff.GPU(), np.complex128 if prec == "f64" else np.complex64, (shape[0] // 2 + 1,) + shape[1:])
    ff.mul_(out, plan, xd)
    got = ff.to_numpy(out)
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() / scale < tol
    back = ff.zeros(ff.GPU(), T, shape)
    ff.ldiv_(back, plan, out)
    assert np.abs(ff.to_numpy(back) - x).max() < 10 * tol * max(1.0, np.abs(x).max())
    assert np.array_equal(ff.to_numpy(xd), x.astype(T))


@pytest.mark.parametrize("shape", [(8,), (30,), (16, 12), (32, 30, 16), (64, 64)], ids=str)
def test_random_complex_fft_vs_oracle(ff, cuda, shape):
    rng = np.random.default_rng(3)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    dev = ff.device_array(ff.GPU())
    got = ff.to_numpy(ff.fft(dev(x)))
    ref = orc.fft(x)
    assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-13
    back = ff.to_numpy(ff.ifft(dev(ref)))
    assert np.abs(back - x).max() < 1e-13
    # in place
    plan = ff.FFTPlan(shape, np.float64)
    xd = dev(x)
    ff.mul_(xd, plan, xd)
    assert np.abs(ff.to_numpy(xd) - ref).max() / np.abs(ref).max() < 1e-13


def test_batched_plan_trailing_dims(ff, cuda):
    """A plan applied to arrays with trailing field dimensions transforms each field."""
    rng = np.random.default_rng(5)
    x = rng.standard_normal((32, 16, 3))
    dev = ff.device_array(ff.GPU())
    g = ff.TwoDGrid(ff.GPU(), nx=32, Lx=2 * math.pi, ny=16, Ly=2 * math.pi)
    out = ff.zeros(ff.GPU(), np.complex128, (17, 16, 3))
    ff.mul_(out, g.rfftplan, dev(x))
    got = ff.to_numpy(out)
    for f in range(3):
        assert np.abs(got[..., f] - orc.rfft(x[..., f])).max() < 1e-12


def test_linearity_and_parseval_at_2048(ff, cuda):
    """Size-independent properties at the precision-form size (2048^2, FP32)."""
    rng = np.random.default_rng(11)
    n = 2048
    a = rng.standard_normal((n, n)).astype(np.float32)
    b = rng.standard_normal((n, n)).astype(np.float32)
    dev = ff.device_array(ff.GPU())
    plan = ff.RFFTPlan((n, n), np.float32)
    A = ff.zeros(ff.GPU(), np.complex64, (n // 2 + 1, n))
    B = ff.zeros(ff.GPU(), np.complex64, (n // 2 + 1, n))
    C = ff.zeros(ff.GPU(), np.complex64, (n // 2 + 1, n))
    ff.mul_(A, plan, dev(a))
    ff.mul_(B, plan, dev(b))
    ff.mul_(C, plan, dev(2 * a - b))
    lin = ff.to_numpy(C) - (2 * ff.to_numpy(A) - ff.to_numpy(B))
    assert np.abs(lin).max() / np.abs(ff.to_numpy(C)).max() < 1e-5
    g = ff.TwoDGrid(ff.GPU(), nx=n, Lx=2 * math.pi, T=np.float32)
    s2 = ff.parsevalsum2(A, g)
    integral = float(np.sum(a.astype(np.float64) ** 2)) * float(g.dx) * float(g.dy)
    assert abs(s2 - integral) / integral < 1e-5


def test_plan_errors(ff, cuda):
    with pytest.raises(ValueError):
        ff.RFFTPlan((7,), np.float64)
    with pytest.raises(NotImplementedError):
        ff.RFFTPlan((2 * 37,), np.float64)  # prime factor 37 > 31
    plan = ff.RFFTPlan((16,), np.float64)
    dev = ff.device_array(ff.GPU())
    with pytest.raises(ValueError):
        ff.mul_(ff.zeros(ff.GPU(), np.complex128, (9,)), plan, dev(np.zeros(12)))


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("n", [(64,), (4096,), (32, 64), (512, 256), (16, 4096), (2048, 16), (16, 32, 8)])
def test_register_and_generic_plan_kernels_agree(ff, cuda, monkeypatch, prec, n):
    """Power-of-two lengths run the register-resident plan kernels (ff_plan_reg.cu);
    FF_PLAN_GENERIC=1 sends the same plans through the shared-memory Stockham kernels.
    rfft, irfft, fft and ifft agree between the two paths and with the oracle."""
    T = np.float64 if prec == "f64" else np.float32
    tol = 1e-12 if prec == "f64" else 2e-6
    rng = np.random.default_rng(sum(n))
    x = rng.standard_normal(n).astype(T)
    z = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex128 if prec == "f64" else np.complex64)
    dev = ff.device_array(ff.GPU())
    res = {}
    for path in ("register", "generic"):
        monkeypatch.setenv("FF_PLAN_GENERIC", "1" if path == "generic" else "0")
        xh = ff.rfft(dev(x))
        back = ff.irfft(xh, n[0])
        zh = ff.fft(dev(z))
        zb = ff.ifft(zh)
        res[path] = [ff.to_numpy(a) for a in (xh, back, zh, zb)]
    want = [orc.rfft(x.astype(np.float64)), x.astype(np.float64), orc.fft(z.astype(np.complex128)),
            z.astype(np.complex128)]
    for a, b, w in zip(res["register"], res["generic"], want):
        a, b = a.astype(w.dtype), b.astype(w.dtype)
        assert isapprox(a, b, rtol=tol), (n, prec)
        assert isapprox(a, w, rtol=tol), (n, prec)
