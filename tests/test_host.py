"""Host-side logic of the product (no GPU): grid set-up, alias ranges, filters, ETDRK4
coefficients, initial conditions, the C ABI's exports and its argument checks."""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import ff_oracle as orc


def test_library_exports_every_header_symbol(ff):
    syms = ff._lib.header_symbols()
    assert len(syms) >= 30
    lib = ff._lib.lib()
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) == set(ff._lib.SIGNATURES), "ctypes signatures must cover the header exactly"
    assert lib.ff_version() == (0 << 16) | (1 << 8)


def test_calcN_slot_count_and_argument_errors(ff):
    """The slot count mirrored in Python is the header's, and the bound-calcN! entry points
    reject bad arguments before any CUDA call."""
    import os
    import re
    hdr = os.path.join(os.path.dirname(__file__), "..", "include", "fourierflows_gb300.h")
    m = re.search(r"#define FF_VORT_CALC_SLOTS (\d+)", open(hdr).read())
    assert m and int(m.group(1)) == ff._lib.FF_VORT_CALC_SLOTS
    with pytest.raises(ValueError):
        ff._lib.call("ff_vort_calcN_bind", None, 0, 0, None, None)
    with pytest.raises(ValueError):
        ff._lib.call("ff_vort_calcN_slot", None, 0, None)
    with pytest.raises(ValueError):
        ff._lib.call("ff_vort_set_split", None, 0)


def test_argument_errors_without_a_gpu(ff):
    """Shape/argument validation happens before any CUDA call, so it is testable here."""
    h = C.c_void_p()
    n = ff._lib.i64_array([8, 1, 1])
    with pytest.raises(ValueError):
        ff._lib.call("ff_plan_create", 0, n, ff._lib.FF_F64, 1, C.byref(h))
    with pytest.raises(ValueError):
        ff._lib.call("ff_plan_create", 1, ff._lib.i64_array([7, 1, 1]), ff._lib.FF_F64, 1, C.byref(h))
    with pytest.raises(NotImplementedError):
        ff._lib.call("ff_plan_create", 1, ff._lib.i64_array([74, 1, 1]), ff._lib.FF_F64, 1, C.byref(h))
    with pytest.raises(ValueError):
        ff._lib.call("ff_plan_create", 2, ff._lib.i64_array([8, 9000, 1]), 7, 1, C.byref(h))
    with pytest.raises(ValueError):
        ff._lib.call("ff_euler_update", ff._lib.FF_F64, 4, None, None, ff._lib.ff_coef(), 0.1, None, None)
    assert "null" in ff._lib.last_error()
    q = ff._lib.ff_vort_problem()
    q.nx, q.ny, q.nkd = 7, 8, 3
    arr = (ff._lib.ff_vort_problem * 1)(q)
    with pytest.raises(ValueError):
        ff._lib.call("ff_vort_create", ff._lib.FF_F64, 0, 0, 0.1, 1, C.cast(arr, C.c_void_p), C.byref(h))


def test_grids_match_oracle(ff):
    for args, og in [(dict(nx=6, Lx=2 * math.pi), orc.OneDGrid(6, 2 * math.pi)),
                     (dict(nx=32, Lx=2 * math.pi, ny=30, Ly=3 * math.pi), orc.TwoDGrid(32, 2 * math.pi, 30, 3 * math.pi)),
                     (dict(nx=16, Lx=2 * math.pi, ny=32, Ly=2 * math.pi, nz=34, Lz=2 * math.pi),
                      orc.ThreeDGrid(16, 2 * math.pi, 32, 2 * math.pi, 34, 2 * math.pi))]:
        cls = {1: ff.OneDGrid, 2: ff.TwoDGrid, 3: ff.ThreeDGrid}[og.ndim]
        g = cls(ff.CPU(), **args)
        assert np.array_equal(g.x, og.x)
        assert np.array_equal(g.k_host.reshape(-1), og.k.reshape(-1))
        assert np.array_equal(g.kr_host.reshape(-1), og.kr.reshape(-1))
        for name in ("kalias", "kralias", "lalias", "malias"):
            r = getattr(g, name, None)
            o = getattr(og, name, None)
            assert (r is None and o is None) or (r.start, r.stop) == o, name
        if og.ndim >= 2:
            assert np.array_equal(g.invKrsq, og.invKrsq)
        assert g.rfftplan is None  # CPU grids carry no transforms


def test_grid_wavenumber_layout(ff):
    """testk/testkr/testdk (test/test_grid.jl:31-48)."""
    g = ff.TwoDGrid(ff.CPU(), nx=6, Lx=2 * math.pi, ny=8, Ly=4 * math.pi)
    k, kr, l = g.k_host.reshape(-1), g.kr_host.reshape(-1), g.l_host.reshape(-1)
    assert math.isclose(k[1], 2 * math.pi / float(g.Lx)) and math.isclose(l[1], 2 * math.pi / float(g.Ly))
    mid = g.nx // 2
    assert np.allclose(k[1:mid], -k[mid + 1:][::-1])
    assert np.allclose(np.concatenate([k[:g.nkr - 1], [abs(k[g.nkr - 1])]]), kr)
    assert math.isclose(g.x[-1] - g.x[0], float(g.Lx - g.dx))


def test_odd_sizes_raise_domain_error(ff):
    """test/runtests.jl:133-138."""
    with pytest.raises(ff.DomainError):
        ff.OneDGrid(ff.CPU(), nx=5, Lx=1)
    with pytest.raises(ff.DomainError):
        ff.TwoDGrid(ff.CPU(), nx=4, Lx=1, ny=5, Ly=2)
    with pytest.raises(ff.DomainError):
        ff.ThreeDGrid(ff.CPU(), nx=4, Lx=1, ny=6, Ly=2, nz=5, Lz=3)


def test_show_strings(ff):
    """repr of the grids equals the reference's show() (test/runtests.jl:118-122)."""
    g1 = ff.OneDGrid(ff.CPU(), nx=6, Lx=2 * math.pi)
    assert repr(g1) == ("OneDimensionalGrid\n  ├─────────── Device: CPU\n  ├──────── FloatType: Float64\n"
                        "  ├────────── size Lx: 6.283185307179586\n  ├──── resolution nx: 6\n"
                        "  ├── grid spacing dx: 1.0471975511965976\n"
                        "  ├─────────── domain: x ∈ [-3.141592653589793, 2.094395102393195]\n"
                        "  └─ aliased fraction: 0.3333333333333333")
    g2 = ff.TwoDGrid(ff.CPU(), nx=6, Lx=2 * math.pi, ny=8, Ly=4 * math.pi)
    assert repr(g2) == ("TwoDimensionalGrid\n  ├───────────────── Device: CPU\n  ├────────────── FloatType: Float64\n"
                        "  ├────────── size (Lx, Ly): (6.283185307179586, 12.566370614359172)\n"
                        "  ├──── resolution (nx, ny): (6, 8)\n"
                        "  ├── grid spacing (dx, dy): (1.0471975511965976, 1.5707963267948966)\n"
                        "  ├───────────────── domain: x ∈ [-3.141592653589793, 2.094395102393195]\n"
                        "  |                          y ∈ [-6.283185307179586, 4.71238898038469]\n"
                        "  └─ aliased fraction: 0.3333333333333333")
    g3 = ff.ThreeDGrid(ff.CPU(), nx=6, Lx=2 * math.pi, ny=8, Ly=4 * math.pi, nz=10, Lz=3.0)
    assert "(6.283185307179586, 12.566370614359172, 3.0)" in repr(g3)
    assert "z ∈ [-1.5, 1.2]" in repr(g3)
    c = ff.Clock(0.01, 0, 0)
    assert repr(c) == "Clock\n  ├─── timestep dt: 0.01\n  ├────────── step: 0\n  └──────── time t: 0.0"


@pytest.mark.parametrize("af", [0, 1 / 3, 1 / 2, 1 / 4])
def test_aliased_fraction(ff, af):
    g = ff.ThreeDGrid(ff.CPU(), nx=16, Lx=2 * math.pi, ny=32, Ly=2 * math.pi, nz=34, Lz=2 * math.pi,
                      aliased_fraction=af)
    og = orc.ThreeDGrid(16, 2 * math.pi, 32, 2 * math.pi, 34, 2 * math.pi, aliased_fraction=af)
    assert float(g.aliased_fraction) == af
    for name in ("kalias", "kralias", "lalias", "malias"):
        r, o = getattr(g, name), getattr(og, name)
        assert (r is None and o is None) or (r.start, r.stop) == o


def test_makefilter_matches_oracle(ff):
    from fourierflows.jl_gb300.domains import makefilter_host
    g = ff.TwoDGrid(ff.CPU(), nx=32, Lx=2 * math.pi, ny=24, Ly=3.0)
    og = orc.TwoDGrid(32, 2 * math.pi, 24, 3.0)
    for kw in ({}, dict(order=4, innerK=0.65), dict(innerK=0.0, outerK=1 / 16)):
        assert np.array_equal(makefilter_host(g, (17, 24), **kw), orc.makefilter(og, **kw))


def test_etdrk4_coefficients_match_oracle(ff):
    og = orc.TwoDGrid(32, 2 * math.pi)
    L = (-1e-3 * og.Krsq - 1e-2)
    for dt in (2e-3, 0.5):
        got = ff.getetdcoeffs(np.float64(dt), L)
        ref = orc.getetdcoeffs(np.float64(dt), L)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
    # Kassam-Trefethen limits: zeta -> dt/2, alpha, gamma -> dt/6, beta -> dt/6 as L -> 0
    z, a, b, c = ff.getetdcoeffs(np.float64(0.1), np.zeros((2, 2)))
    assert np.allclose(z, 0.05, rtol=1e-14) and np.allclose(a, 0.1 / 6, rtol=1e-13)
    assert np.allclose(b, 0.1 / 6, rtol=1e-13) and np.allclose(c, 0.1 / 6, rtol=1e-13)


def test_lsrk54_coefficients(ff):
    """Carpenter-Kennedy (5,4) 2N-storage table (src/timesteppers.jl:335-350): consistency."""
    from fourierflows.jl_gb300.timesteppers import _LSRK_A, _LSRK_B, _LSRK_C
    assert _LSRK_A[0] == 0 and _LSRK_C[0] == 0
    assert float(_LSRK_C[1]) == float(_LSRK_B[0])


def test_random_phase_ic(ff):
    z = ff.Vorticity.random_phase_vorticity(64, seed=11)
    g = orc.TwoDGrid(64, 2 * math.pi)
    zh = orc.rfft(z)
    assert abs(orc.vorticity_energy(zh, g) - 0.5) < 1e-12
    assert np.abs(zh[g.kralias[0]:, :]).max() < 1e-9 * np.abs(zh).max()
    assert np.array_equal(z, ff.Vorticity.random_phase_vorticity(64, seed=11))
    assert not np.array_equal(z, ff.Vorticity.random_phase_vorticity(64, seed=12))
    u = ff.Vorticity.uniform01(5, 1000)
    assert u.min() >= 0 and u.max() < 1 and abs(u.mean() - 0.5) < 0.05


def test_cpu_device_refuses_compute(ff):
    g = ff.OneDGrid(ff.CPU(), nx=8, Lx=2 * math.pi)
    with pytest.raises(NotImplementedError):
        ff.mul_(np.zeros(5, complex), g.rfftplan, np.zeros(8))
    with pytest.raises(NotImplementedError):
        ff.ForwardEulerTimeStepper(ff.Equation(np.zeros(5), None, g), ff.CPU())


def test_stepper_dispatch_names(ff):
    assert ff.isexplicit("RK4") and ff.isexplicit("FilteredAB3") and not ff.isexplicit("ETDRK4")
    g = ff.OneDGrid(ff.CPU(), nx=8, Lx=2 * math.pi)
    with pytest.raises(ValueError):
        ff.TimeStepper("Nope", ff.Equation(np.zeros(5), None, g), 0.1, ff.CPU())


def test_empty_ensemble_rejected(ff):
    with pytest.raises(ValueError):
        ff.Vorticity.Ensemble([])
