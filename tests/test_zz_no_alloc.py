"""ff_parsevalsum2_noalloc: the Parseval sum for callers that cannot call cudaMalloc
(their device memory belongs to another allocator).  It must agree with the allocating
ff_parsevalsum2 on consecutive calls, so that the shared static scratch never leaks one
call's partial sums into the next.  This file is collected last on purpose."""
import ctypes as C
import math

import numpy as np
import pytest


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_noalloc_parseval_matches_allocating_version(ff, cuda, prec):
    torch = cuda
    T = np.float64 if prec == "f64" else np.float32
    cdt = torch.complex128 if prec == "f64" else torch.complex64
    code = ff._lib.FF_F64 if prec == "f64" else ff._lib.FF_F32
    tol = 1e-13 if prec == "f64" else 1e-6
    g = ff.TwoDGrid(ff.GPU(), nx=512, Lx=2 * math.pi, ny=384, Ly=3.0, T=T)
    norm = float(g.Lx) * float(g.Ly) / (g.nx ** 2 * g.ny ** 2)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(17)
    # two calls in a row on different inputs (the second one larger than the first)
    for shape in [(g.nkr, g.ny), (g.nkr, g.ny, 3)]:
        x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        uh = ff.device_array(ff.GPU())(x.astype(np.complex128 if prec == "f64" else np.complex64))
        assert uh.dtype == cdt
        n0, nrest = shape[0], int(np.prod(shape[1:]))
        ff._lib.call("ff_parsevalsum2_noalloc", code, C.c_void_p(uh.data_ptr()), n0, nrest, 1, norm,
                     C.c_void_p(out.data_ptr()), ff.devices.stream_handle())
        torch.cuda.synchronize()
        got = float(out.item())
        ref = C.c_double()
        ff._lib.call("ff_parsevalsum2", code, C.c_void_p(uh.data_ptr()), n0, nrest, 1, norm, C.byref(ref),
                     ff.devices.stream_handle())
        assert abs(got - ref.value) <= tol * abs(ref.value), (shape, got, ref.value)


def test_noalloc_parseval_rejects_oversized_input(ff):
    """The size check precedes any CUDA call, so this runs without a GPU."""
    out = C.c_double()
    with pytest.raises(ValueError) as e:
        ff._lib.call("ff_parsevalsum2_noalloc", ff._lib.FF_F64, C.c_void_p(16), 8193, 4096, 1, 1.0, C.byref(out),
                     None)
    assert "exceed the maximum" in str(e.value)
