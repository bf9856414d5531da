"""bench.py's byte and flop bookkeeping (no GPU): the per-step byte models quoted with the
measurements, and the FP64 roofline counts' consistency."""
import importlib.util
import os

import pytest

ROOT = os.path.join(os.path.dirname(__file__), "..")


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_unfused_step_model(bench):
    # 20 (C + R) + 21 C with C = (n/2+1) n 2 s, R = n^2 s: 1024^2 in FP32 and FP64
    assert bench.model_step_bytes(1024, 4) == 256_188_416
    assert bench.model_step_bytes(1024, 8) == 512_376_832
    n, s = 128, 4
    C, R = (n // 2 + 1) * n * 2 * s, n * n * s
    assert bench.model_step_bytes(n, s) == 20 * (C + R) + 21 * C


def test_fused_pass_bytes(bench):
    fp32 = bench.pass_bytes(1024, 8, fused_a=True)
    fp64 = bench.pass_bytes(1024, 16, fused_a=False)
    assert fp32["step"] == 154_803_800 and fp64["step"] == 331_933_552
    # the step is the sum of its launches: pass A once (fused into pass C) or four times,
    # pass B four times, the four pass C epilogues; and it moves less than the unfused model
    for b, fused, s in ((fp32, True, 4), (fp64, False, 8)):
        total = b["A"] * (1 if fused else 4) + 4 * b["B"] + b["C1"] + b["C2"] + b["C3"] + b["C4"]
        assert total == b["step"]
        assert b["step"] < bench.model_step_bytes(1024, s)


def test_fp64_roofline_counts(bench):
    flops, inst = bench.fp64_counts("B")
    c = bench.NCU["fp64_1024"]["B"]
    assert inst == c["dadd"] + c["dmul"] + c["dfma"]
    assert flops == inst + c["dfma"]
    # a full pipe reaches flops / (2 inst) of the FMA-counted peak: at most 1
    assert 0.5 <= flops / (2 * inst) <= 1.0
