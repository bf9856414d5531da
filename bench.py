#!/usr/bin/env python
"""ETDRK4 steps/s of the 2D vorticity problem on one GB300 (and N independent replicas).

Workload (the plain FP64 configuration): TwoDGrid 1024 x 1024, Lx = Ly = 2 pi, Float64,
L = -nu |k|^2 - mu with nu = 1e-4, mu = 1e-2, N = -J(psi, zeta) with 2/3 dealiasing,
random-phase initial vorticity (seeded) with E(k) ~ k^4 exp(-2 (k/6)^2) and energy 0.5,
ETDRK4 with dt = 2e-3.  A "step" is one ETDRK4 step of that problem.

  value          steps/s with the state resident in HBM (device time, CUDA events around
                 each step, L2 flushed between steps by writing a 256 MiB buffer)
  e2e            steps/s through the public API (stepforward_) with the state copied from
                 pinned host memory before every step and the energy read back after it
  roofline       the dominant pass's algorithmic bytes (and FP64 flops) per launch over its
                 event-timed duration, against the measured copy bandwidth (and FP64 rate)
  cpu_baseline   the CPU oracle (numpy / scipy.fft, all host cores) on a bounded sample
  forms          FP32 on the same problem, FP32 batched (32 problems of 1024^2 in one
                 launch per pass) and the uneven ensemble (384 problems 128^2 .. 1024^2),
                 with the FP32-vs-FP64 relative L2 error after 100 steps

--impl reference times the CPU oracle of the same step (FourierFlows.jl itself is Julia,
absent here) with every host thread.  Multi-GPU runs are independent replicas: each rank
steps its own problem, there is no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N, LX, NU, MU, DT, SEED = 1024, 2 * math.pi, 1e-4, 1e-2, 2e-3, 20260101
METRIC = "ETDRK4 steps/s, 2D 1024²: FP32+batched vs FP64 plain @≤1e-5 rel L2; HBM GB/s"
WORKLOAD = "2D vorticity ETDRK4, TwoDGrid 1024x1024 FP64, nu=1e-4, mu=1e-2, dt=2e-3, 2/3 dealiasing"


def args_():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--no-forms", action="store_true", help="skip the FP32 / batched / ensemble forms")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    p.add_argument("--no-adjoint", action="store_true", help="skip the differentiation form")
    p.add_argument("--profile-case", default="",
                   help="run only a small case for ncu (fp64|fp32|batch|fft|steppers|adjoint|spectra)")
    p.add_argument("--tiles", default="", help="profile case: tile_a,tile_c,rows_b (default: the library's)")
    return p.parse_args()


# ----------------------------------------------------------------------------------------
# helpers
# ----------------------------------------------------------------------------------------
def replica_time(total_ms, world, device):
    """The job's timed-region duration: the MAX over ranks of each replica's own (every rank
    advances an independent problem; no collective on the data path)."""
    if world == 1:
        return total_ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ms_per_step, world):
    """Whole-job steps/s: every rank's problem-steps over the slowest rank's time."""
    return world * 1e3 / ms_per_step


def dist_init(gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def pass_bytes(n, es, fused_a, filtered=False):
    """Algorithmic bytes of each launch of one fused ETDRK4 step of an n^2 problem (es bytes
    per complex value, es/2 per real): every operand a launch reads counted once and every
    result it writes once, over the modes its kernels touch.

      A    kept zeta_hat and kept 1/K^2 in; W (u, v, zeta: nkd kept columns x n) out
      B    W in; Q (u zeta, v zeta) out
      Ck   Q in, then substep k's epilogue.  Substeps 1-3 touch only the kept modes
           (nkd columns x lrows rows); substep 4 also advances the aliased modes by
           exp(L dt) alone (sol and exp(L dt) in, sol out).  fused_a (FP32): pass C of
           substeps 1-3 also runs the next substep's pass A (kept 1/K^2 in, W out), so A
           runs apart only in substep 1, and the intermediate states sol1 / sol2 pass to it
           in registers instead of through HBM (substep 3 rebuilds sol1 from sol and N1)."""
    from fourierflows.jl_gb300.domains import getaliasedwavenumbers
    nkr = n // 2 + 1
    lal, kral = getaliasedwavenumbers(n, nkr, 1 / 3)
    nkd, lrows = kral.start, n - len(lal)
    rs = es // 2
    K, M = nkd * lrows, nkr * n
    Wd = nkd * n * es
    a_in, a_out = K * (es + rs), 3 * Wd
    b = 5 * Wd
    fl = rs if filtered else 0
    if fused_a:  # sol (+ N1) and e_half, zeta in; N_k out
        epi = {1: K * (2 * es + 2 * rs), 2: K * (2 * es + 2 * rs), 3: K * (3 * es + 2 * rs)}
    else:        # the input state (+ N1) and e_half, zeta in; N_k and the next state out
        epi = {1: K * (3 * es + 2 * rs), 2: K * (3 * es + 2 * rs), 3: K * (4 * es + 2 * rs)}
    epi[4] = K * (5 * es + 4 * rs + fl) + (M - K) * (2 * es + rs + fl)
    c = {k: 2 * Wd + epi[k] + ((K * rs + a_out) if fused_a and k < 4 else 0) for k in (1, 2, 3, 4)}
    step = (a_in + a_out) * (1 if fused_a else 4) + 4 * b + sum(c.values())
    return {"A": a_in + a_out, "B": b, "C1": c[1], "C2": c[2], "C3": c[3], "C4": c[4], "step": step}


def model_step_bytes(n, s):
    """Bytes of an unfused ETDRK4 step of the vorticity problem: 20 (C + R) + 21 C with
    C = (n/2+1) n 2 s and R = n^2 s (one read and one write per 2D FFT, the operands of the
    four combinations read once)."""
    C = (n // 2 + 1) * n * 2 * s
    R = n * n * s
    return 20 * (C + R) + 21 * C


# Per-launch counters from ncu captures (one launch, cold L2; the summaries of these captures,
# with the commands that made them, are kept with the profiles).  FP64 counts are thread instructions (DFMA = 2 flops); DRAM bytes
# are read + write and miss the outputs still in L2 when the kernel ends.
NCU = {
    "fp64_1024": {
        "capture": "ncu --metrics (FP64 instruction counts, DRAM bytes) on bench.py --profile-case fp64 "
                   "--steps 3 --tiles 1,1,1: 1024^2 FP64, k_vort_b_r<double>, step 2, substep 1",
        "B": {"dadd": 36.62e6, "dmul": 4.99e6, "dfma": 37.11e6, "dram_bytes": 17.16e6},
    },
    "fp32_batch4_1024": {
        "capture": "ncu --set full on bench.py --profile-case batch --tiles 4,4,1: 4 x 1024^2 FP32, "
                   "passes A, B and C of step 2",
        "A": {"dram_bytes": 9.13e6}, "B": {"dram_bytes": 33.83e6}, "C": {"dram_bytes": 35.35e6},
    },
}


def fp64_counts(kernel="B"):
    c = NCU["fp64_1024"][kernel]
    return c["dadd"] + c["dmul"] + 2 * c["dfma"], c["dadd"] + c["dmul"] + c["dfma"]


# ----------------------------------------------------------------------------------------
# the reference arm: the CPU oracle of the same step
# ----------------------------------------------------------------------------------------
def cpu_oracle_rate(steps, warmup, budget_s, cores):
    import numpy as np
    from oracle import ff_oracle as orc
    import fourierflows.jl_gb300.vorticity as vort
    orc.set_workers(cores)
    z0 = vort.random_phase_vorticity(N, seed=SEED)
    prob = orc.VorticityProblem(N, LX, NU, MU, DT, "ETDRK4")
    prob.sol[...] = orc.rfft(z0)
    orc.stepforward(prob, max(1, warmup))
    done, t0 = 0, time.perf_counter()
    while done < steps:
        orc.stepforward(prob, 1)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return done / dt, done, dt


def reference_arm(a):
    rank, world, _ = dist_init(a.gpus)
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    rate, done, secs = cpu_oracle_rate(a.steps, a.warmup, 150.0, cores)
    line = {"metric": METRIC, "value": rate, "unit": "steps/s", "n_gpus": a.gpus, "steps": done, "warmup": a.warmup,
            "ms_per_step": 1e3 / rate, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "parallelism": "cpu", "l2": "n/a"},
            "cpu_baseline": {"value": rate, "unit": "steps/s", "cores": cores, "kind": "port",
                             "sample": f"{done} ETDRK4 steps of the 1024^2 FP64 problem in {secs:.1f} s "
                                       "(numpy/scipy.fft restatement of the reference; FourierFlows.jl is Julia, "
                                       "absent on this box)"},
            "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ----------------------------------------------------------------------------------------
# our arm
# ----------------------------------------------------------------------------------------
def make_problem(ff, T):
    import numpy as np
    prob = ff.Vorticity.Problem(ff.GPU(), nx=N, Lx=LX, nu=NU, mu=MU, dt=DT, stepper="ETDRK4", T=T)
    ff.Vorticity.set_zeta_(prob, ff.Vorticity.random_phase_vorticity(N, seed=SEED))
    fs = prob.timestepper._native(prob.eqn).ensure(prob.sol, prob.clock)
    return prob, fs


def timed_steps(torch, fs, steps, flush):
    """Sum of per-step device times (ms), L2 flushed before each step (not timed)."""
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for e0, e1 in ev:
        flush.add_(1.0)
        e0.record()
        fs.advance(1)
        e1.record()
    torch.cuda.synchronize()
    return sum(e0.elapsed_time(e1) for e0, e1 in ev)


def autotune(torch, fs, sol):
    saved = sol.clone()
    fs.autotune(steps_per_trial=2)
    sol.copy_(saved)
    torch.cuda.synchronize()
    return fs.config()


def fp64_roofline(ff, tA, tB, tC, steps_per_s, hbm, peak_src):
    """The FP64 step is bound by the FP64 pipe, not HBM: the dominant pass (B) against the
    FP64 rate measured in this run (ff_fp64_peak: FMA chains, 2 flops per FMA).  achieved =
    the flops pass B executes (DADD + DMUL + 2 DFMA, counted by ncu on the same launch:
    NCU["fp64_1024"]) over its event-timed duration.  A DADD or DMUL fills an FMA slot with
    one flop, so at a full pipe this mix reaches attainable_frac of the FMA peak; pipe_frac =
    FP64 instructions issued per second over the pipe's rate (peak / 2)."""
    fp64 = ctypes_peak(ff)
    flops, inst = fp64_counts("B")
    byts = pass_bytes(N, 16, fused_a=False)
    t = tB * 1e-3
    achieved = flops / t / 1e12
    hbm_gbs = byts["B"] / t / 1e9
    out = {"bound": "fp64", "achieved": achieved, "peak": fp64, "unit": "TFLOP/s",
           "frac": achieved / fp64 if fp64 else None,
           "traffic": NCU["fp64_1024"]["B"]["dram_bytes"],
           "traffic_note": "ncu dram bytes (read + write) of one launch, cold L2: the inputs; outputs still in "
                           "L2 at the kernel's end are not in it",
           "kernel": "k_vort_b_r<double> (pass B: 3 C2R rows, products, 2 R2C rows)",
           "peak_source": "ff_fp64_peak in this run (FP64 is not in MEASURED_PEAKS.json)",
           "counts_source": NCU["fp64_1024"]["capture"],
           "flops_per_launch": flops, "fp64_inst_per_launch": inst,
           "pipe_frac": (inst / t) / (fp64 * 1e12 / 2) if fp64 else None,
           "attainable_frac": flops / inst / 2,
           "pass_ms": {"A": tA, "B": tB, "C": tC},
           "hbm": {"achieved": hbm_gbs, "peak": hbm, "unit": "GB/s", "frac": hbm_gbs / hbm,
                   "peak_source": peak_src, "bytes_per_launch": byts["B"]},
           "step_bytes": byts["step"], "step_hbm_frac": byts["step"] * steps_per_s / 1e9 / hbm,
           "step_model_bytes": model_step_bytes(N, 8),
           "step_model_frac": model_step_bytes(N, 8) * steps_per_s / 1e9 / hbm}
    return out


def our_arm(a):
    import numpy as np
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import fourierflows.jl_gb300 as ff

    rank, world, local = dist_init(a.gpus)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    pk = peaks()
    hbm = pk.get("hbm_gbs", 6800.0)
    peak_src = "of measured" if "hbm_gbs" in pk else "of fallback"

    prob, fs = make_problem(ff, np.float64)
    cfg64 = autotune(torch, fs, prob.sol)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2
    fs.advance(a.warmup)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    total_ms = timed_steps(torch, fs, a.steps, flush)
    torch.cuda.synchronize()
    total_ms = replica_time(total_ms, world, "cuda")
    clk = clocks.stop()
    ms_per_step = total_ms / a.steps
    value = replica_value(ms_per_step, world)
    launches = a.steps * 12

    # per-pass device times (events inside the library) and the roofline of the dominant pass
    tA, tB, tC = fs.profile(reps=20)
    roofline = fp64_roofline(ff, tA, tB, tC, value / world, hbm, peak_src)

    # end to end through the public API: pinned host state in, energy out, every step
    host = torch.empty(prob.sol.shape[::-1], dtype=prob.sol.dtype, pin_memory=True).t()
    host.copy_(prob.sol)
    torch.cuda.synchronize()
    e2e_steps = max(10, min(a.steps, 100))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        prob.sol.copy_(host, non_blocking=True)
        ff.stepforward_(prob)
        ff.Vorticity.energy(prob)  # device -> host read (8 bytes) and synchronisation
    torch.cuda.synchronize()
    e2e = world * e2e_steps / (time.perf_counter() - t0)
    h2d = prob.sol.numel() * prob.sol.element_size()

    # the precision / batching / differentiation forms are single-GPU measurements
    forms = {} if (a.no_forms or world > 1) else run_forms(torch, ff, a, hbm, peak_src, value)

    cpu = None
    if rank == 0 and not a.no_cpu:
        cores = os.cpu_count() or 1
        rate, done, secs = cpu_oracle_rate(400, 1, 10.0, cores)  # about 10 s of CPU work
        cpu = {"value": rate, "unit": "steps/s", "cores": cores, "kind": "port",
               "sample": f"{done} ETDRK4 steps of the same 1024^2 FP64 problem in {secs:.1f} s (numpy/scipy.fft "
                         "oracle, scipy workers = all host cores)"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random-phase vorticity)",
                "config": {"workload": WORKLOAD, "global_batch": world, "parallelism": f"replicas{world}",
                           "l2": "flushed between steps (256 MiB write)", "tiles": cfg64,
                           "algorithmic_bytes_per_step": roofline["step_bytes"],
                           "model_bytes_per_step": model_step_bytes(N, 8)},
                "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 8},
                "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
                "forms": forms}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def ctypes_peak(ff):
    import ctypes as C
    v = C.c_double()
    try:
        ff._lib.call("ff_fp64_peak", C.byref(v), None)
        return v.value
    except Exception:
        return None


def run_forms(torch, ff, a, hbm, peak_src, fused_fp64):
    import numpy as np
    out = {}
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    out["cudajl_standin_fp64_1024"] = cudajl_standin(torch, ff, a, fused_fp64, flush)
    steps = max(20, min(a.steps, 200))
    # FP32 single problem and its accuracy against FP64 after 100 steps
    p32, f32 = make_problem(ff, np.float32)
    p64, f64s = make_problem(ff, np.float64)
    f32.advance(100)
    f64s.advance(100)
    torch.cuda.synchronize()
    s64 = ff.to_numpy(p64.sol)
    s32 = ff.to_numpy(p32.sol).astype(np.complex128)
    relL2 = float(np.linalg.norm(s32 - s64) / np.linalg.norm(s64))
    E64, E32 = ff.Vorticity.energy(p64), ff.Vorticity.energy(p32)
    Z64, Z32 = ff.Vorticity.enstrophy(p64), ff.Vorticity.enstrophy(p32)
    del p64, f64s
    cfg32 = autotune(torch, f32, p32.sol)
    f32.advance(a.warmup)
    ms32 = timed_steps(torch, f32, steps, flush) / steps
    out["fp32_1024"] = {"value": 1e3 / ms32, "unit": "steps/s", "ms_per_step": ms32, "tiles": cfg32,
                        "rel_l2_vs_fp64_after_100": relL2, "energy_rel_err": abs(E32 - E64) / E64,
                        "enstrophy_rel_err": abs(Z32 - Z64) / Z64}
    del p32, f32
    # FP32 batched: 32 problems of 1024^2 advanced together
    B = 32
    members = [(N, NU, SEED + i) for i in range(B)]
    ens = ff.Vorticity.Ensemble(members, mu=MU, dt=DT, T=np.float32)
    saved = [m.sol.clone() for m in ens.members]
    acc = batched_accuracy(torch, ff, ens, members, 100)
    for m, s in zip(ens.members, saved):
        m.sol.copy_(s)
    ens.fs.autotune(steps_per_trial=1)
    for m, s in zip(ens.members, saved):
        m.sol.copy_(s)
    ens.fs.advance(a.warmup)
    bsteps = max(10, min(a.steps, 50))
    msb = timed_steps(torch, ens.fs, bsteps, flush) / bsteps
    tA, tB, tC = ens.fs.profile(reps=5)
    bts = pass_bytes(N, 8, fused_a=True)
    # pass C as profiled: substep 1's, fused with substep 2's pass A
    passes = {"A": (tA, B * bts["A"]), "B": (tB, B * bts["B"]), "C": (tC, B * bts["C1"])}
    dom = max(passes, key=lambda k: passes[k][0])
    ach = passes[dom][1] / (passes[dom][0] * 1e-3) / 1e9
    step_ach = B * bts["step"] / (msb * 1e-3) / 1e9
    step_md = B * model_step_bytes(N, 4) / (msb * 1e-3) / 1e9
    cap = NCU["fp32_batch4_1024"]
    out["fp32_batched_1024x32"] = {
        "value": B * 1e3 / msb, "unit": "problem-steps/s (1024^2 ETDRK4)", "ms_per_step": msb,
        "tiles": ens.fs.config(), "l2": "working set 1.8 GB > L2; flushed between steps",
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                     "traffic": cap[dom]["dram_bytes"] * B / 4 if dom in cap else None,
                     "traffic_note": "ncu dram bytes of one launch on 4 problems, scaled to 32 (per-problem "
                                     "traffic is size-independent); cold L2, outputs still in L2 at the end "
                                     "are not in it; " + cap["capture"],
                     "kernel": f"k_vort_{dom.lower()}_r<float> (pass {dom})", "peak_source": peak_src,
                     "bytes_per_launch": passes[dom][1], "pass_ms": {"A": tA, "B": tB, "C": tC}},
        "step_bytes_per_problem": bts["step"], "step_algorithmic_gbs": step_ach, "step_frac": step_ach / hbm,
        "step_model_bytes_per_problem": model_step_bytes(N, 4),
        "step_model_gbs": step_md, "step_model_frac": step_md / hbm, **acc}
    del ens, saved
    # the uneven ensemble: 128 x 128^2, 128 x 256^2, 96 x 512^2, 32 x 1024^2, nu log-uniform
    u = ff.Vorticity.uniform01(99, 384)
    nus = 10 ** (-5 + 2 * u)
    spec = [(128, nus[i], 1000 + i) for i in range(128)] + [(256, nus[128 + i], 2000 + i) for i in range(128)]
    spec += [(512, nus[256 + i], 3000 + i) for i in range(96)] + [(1024, nus[352 + i], 4000 + i) for i in range(32)]
    ens = ff.Vorticity.Ensemble(spec, mu=MU, dt=DT, T=np.float32)
    saved = [m.sol.clone() for m in ens.members]
    ens.fs.autotune(steps_per_trial=1)
    for m, s in zip(ens.members, saved):
        m.sol.copy_(s)
    del saved
    ens.fs.advance(a.warmup)
    msu = timed_steps(torch, ens.fs, bsteps, flush) / bsteps
    gp = ens.grid_points
    ubytes = sum(pass_bytes(n, 8, fused_a=True)["step"] for n, _, _ in spec)
    umodel = sum(model_step_bytes(n, 4) for n, _, _ in spec)
    ugbs = ubytes / (msu * 1e-3) / 1e9
    out["ensemble_uneven_384"] = {"value": 384 * 1e3 / msu, "unit": "problem-steps/s", "ms_per_step": msu,
                                  "tiles": ens.fs.config(),
                                  "grid_point_steps_per_s": gp * 1e3 / msu, "problems": 384,
                                  "sizes": "128x128^2 + 128x256^2 + 96x512^2 + 32x1024^2", "dtype": "f32",
                                  "roofline": {"bound": "hbm", "achieved": ugbs, "peak": hbm, "unit": "GB/s",
                                               "frac": ugbs / hbm, "kernel": "whole step (9 launches)",
                                               "bytes_per_step": ubytes, "peak_source": peak_src,
                                               "model_bytes_per_step": umodel,
                                               "model_frac": umodel / (msu * 1e-3) / 1e9 / hbm}}
    del ens
    out["diffusion3d_64x128^3"] = diffusion3d_ensemble(torch, ff, a, hbm, peak_src, flush)
    out["precision_2048"] = precision_2048(torch, ff)
    if not a.no_adjoint:
        out["adjoint_512"] = adjoint_512(torch, ff)
    return out


def batched_accuracy(torch, ff, ens, members, steps):
    """The batched FP32 members against the same members advanced in FP64 (the FP64 path is
    itself pinned to the CPU oracle at 1e-12): relative L2 of each member's state after
    `steps` steps from the same seeded initial conditions; the FP32 ensemble is left advanced."""
    import numpy as np
    e64 = ff.Vorticity.Ensemble(members, mu=MU, dt=DT, T=np.float64)
    e64.stepforward_(steps)
    ens.stepforward_(steps)
    torch.cuda.synchronize()
    errs = []
    for m32, m64 in zip(ens.members, e64.members):
        a, b = ff.to_numpy(m32.sol).astype(np.complex128), ff.to_numpy(m64.sol)
        errs.append(float(np.linalg.norm(a - b) / np.linalg.norm(b)))
    del e64
    return {"rel_l2_vs_fp64_after_100_max": max(errs), "rel_l2_vs_fp64_after_100_mean": float(np.mean(errs)),
            "members_checked": len(errs)}


def cudajl_standin(torch, ff, a, fused_steps_per_s, flush):
    """The reference's own GPU design, restated: the same FP64 1024^2 ETDRK4 step unfused,
    one kernel per Julia broadcast and cuFFT plans for the transforms, launched one by one
    from the host (baseline/cudajl_standin; FourierFlows.jl + CUDA.jl cannot run here).
    Same L2 flush between steps as the headline; its state after the timed steps is checked
    against the fused path's."""
    import numpy as np
    from baseline.cudajl_standin.standin import UnfusedETDRK4
    prob, fs = make_problem(ff, np.float64)
    u = UnfusedETDRK4(prob)
    state = prob.sol.clone()
    u.step(state, a.warmup)
    fs.advance(a.warmup)
    steps = max(10, min(a.steps, 50))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for e0, e1 in ev:
        flush.add_(1.0)
        e0.record()
        u.step(state, 1)
        e1.record()
    torch.cuda.synchronize()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev) / steps
    fs.advance(steps)
    torch.cuda.synchronize()
    ref = ff.to_numpy(prob.sol)
    err = float(np.linalg.norm(ff.to_numpy(state) - ref) / np.linalg.norm(ref))
    return {"value": 1e3 / ms, "unit": "steps/s", "ms_per_step": ms, "launches_per_step": u.launches_per_step,
            "what": "unfused FP64 restatement of FourierFlows.jl's GPU path: one kernel per broadcast "
                    "(src/timesteppers.jl:501-547, src/domains.jl:457-458), cuFFT D2Z/Z2D plans + scaling "
                    "(src/domains.jl:5), host-launched one by one",
            "rel_l2_vs_fused_after_steps": err, "steps_compared": a.warmup + steps,
            "fused_speedup": fused_steps_per_s / (1e3 / ms),
            "l2": "flushed between steps (256 MiB write)"}


def precision_2048(torch, ff):
    """FP32 state and transforms against the FP64 run of the same 2048^2 problem, for ETDRK4
    and FilteredRK4 (order 4, innerK 0.65): relative L2 of zeta at steps 100 and 1000 and
    the largest relative energy / enstrophy deviation over the series sampled every 100 steps;
    the FP32 rate from CUDA events around steps 101-1000."""
    import numpy as np
    n = 2048
    # dt = 2e-3 puts the kept modes past the advective stability limit at 2048^2
    # (k_max u_max dt = 681 * 2.78 * 2e-3 = 3.8 > 2.83 for RK4 and ETDRK4: both precisions
    # blow up); dt = 1e-3 keeps the CFL number of the 1024^2 configuration (1.9)
    dt = 1e-3
    z0 = ff.Vorticity.random_phase_vorticity(n, seed=SEED)
    out = {"dt": dt}
    for stepper, kw in (("ETDRK4", {}), ("FilteredRK4", {"order": 4, "innerK": 0.65})):
        probs = {}
        for T in (np.float64, np.float32):
            p = ff.Vorticity.Problem(ff.GPU(), nx=n, Lx=LX, nu=NU, mu=MU, dt=dt, stepper=stepper, T=T, **kw)
            ff.Vorticity.set_zeta_(p, z0)
            probs[T] = p
        p64, p32 = probs[np.float64], probs[np.float32]
        res, eE, eZ, t32 = {}, 0.0, 0.0, 0.0
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for chunk in range(10):
            ff.stepforward_(p64, 100)
            torch.cuda.synchronize()
            ev0.record()
            ff.stepforward_(p32, 100)
            ev1.record()
            torch.cuda.synchronize()
            if chunk > 0:  # the first chunk also captures the step's CUDA graph
                t32 += ev0.elapsed_time(ev1) * 1e-3
            E64, E32 = ff.Vorticity.energy(p64), ff.Vorticity.energy(p32)
            Z64, Z32 = ff.Vorticity.enstrophy(p64), ff.Vorticity.enstrophy(p32)
            eE, eZ = max(eE, abs(E32 - E64) / E64), max(eZ, abs(Z32 - Z64) / Z64)
            if chunk in (0, 9):
                s64 = ff.to_numpy(p64.sol)
                s32 = ff.to_numpy(p32.sol).astype(np.complex128)
                res[f"rel_l2_step{100 * (chunk + 1)}"] = float(np.linalg.norm(s32 - s64) / np.linalg.norm(s64))
        res.update({"energy_max_rel_err": eE, "enstrophy_max_rel_err": eZ, "energy_final": E64,
                    "fp32_steps_per_s": 900 / t32, "finite": bool(np.isfinite(E64) and np.isfinite(E32))})
        out[stepper] = res
        del probs, p64, p32
    return out


def diffusion3d_ensemble(torch, ff, a, hbm, peak_src, flush):
    """64 constant-kappa diffusion problems on ThreeDGrid 128^3 (kappa uniform in [1e-3, 1e-2],
    Gaussian blobs), FP32 ETDRK4 dt = 2e-3, stacked so each step is one native pass."""
    import numpy as np
    B, n = 64, 128
    kappas = 1e-3 + 9e-3 * ff.Vorticity.uniform01(77, B)
    ens = ff.Diffusion.Ensemble3D(kappas, n=n, dt=DT, T=np.float32)
    ens.stepforward_(a.warmup)
    steps = max(5, min(a.steps, 30))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for e0, e1 in ev:
        flush.add_(1.0)
        e0.record()
        ens.stepforward_(1)
        e1.record()
    torch.cuda.synchronize()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev) / steps
    C = (n // 2 + 1) * n * n * B * 8  # one complex state array
    R = C // 2                         # one real coefficient array
    # N = 0 (constant kappa): a step is sol = exp(L dt) sol, one pass (ff_linear_step):
    # sol and exp(L dt) read, sol written
    byts = 2 * C + R
    gbs = byts / (ms * 1e-3) / 1e9
    return {"value": B * 1e3 / ms, "unit": "problem-steps/s", "ms_per_step": ms, "problems": B,
            "grid_point_steps_per_s": ens.grid_points * 1e3 / ms, "dtype": "f32",
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                         "kernel": "k_linear_etd_f32x2 (one pass per step)", "bytes_per_step": byts,
                         "peak_source": peak_src},
            "kernels_per_step": 1,
            "note": "constant kappa gives N = 0 (src/diffusion.jl:129-133), so the ETDRK4 step is exactly "
                    "sol = exp(L dt) sol; the stepper's N fills and substep passes are skipped"}


def fp32_adjoint_segment_check(torch, ff, n=512, K=50):
    """Is the FP32 adjoint the transpose of its own map?  One checkpoint segment (K steps at
    n^2): the FP32 adjoint's directional derivative against an FP64 tangent-linear sweep
    along the FP32 forward states, with the FP32-rounded ETDRK4 coefficients.  The tangent
    of the nonlinear term comes from the library's FP64 calcN! by polarisation: N is
    bilinear, so J(s) d = (N(s + l d) - N(s) - N(l d)) / l, with l = |s| / |d|."""
    import numpy as np
    dev = ff.device_array(ff.GPU())
    p32 = ff.Vorticity.Problem(ff.GPU(), nx=n, Lx=LX, nu=NU, mu=MU, dt=DT, stepper="ETDRK4", T=np.float32)
    a32 = ff.Adjoint.VorticityAdjoint(p32, checkpoint_every=K)
    z0 = ff.Vorticity.random_phase_vorticity(n, seed=SEED + 22)
    zt = ff.Vorticity.random_phase_vorticity(n, seed=SEED + 23).astype(np.float32)
    tgt = ff.rfft(dev(zt))
    _, gz, _ = a32.gradient(z0, tgt, K)
    # the FP32 forward states of the segment
    ff.Vorticity.set_zeta_(p32, z0)
    states = [p32.sol.clone()]
    for _ in range(K):
        ff.stepforward_(p32)
        states.append(p32.sol.clone())
    p64 = ff.Vorticity.Problem(ff.GPU(), nx=n, Lx=LX, nu=NU, mu=MU, dt=DT, stepper="ETDRK4")
    ts = p32.timestepper
    E, E2, Z, A, B, G = (c.double() for c in (ts.expLdt, ts.exp_half_Ldt, ts.zeta, ts.alpha, ts.beta, ts.Gamma))

    def N(x):
        out = torch.empty_like(x)
        ff.Vorticity.calcN_(out, x, 0.0, p64.clock, p64.vars, p64.params, p64.grid)
        return out

    def J(x, d):
        lam = float(torch.linalg.vector_norm(x) / torch.linalg.vector_norm(d))
        return (N(x + lam * d) - N(x) - N(lam * d)) / lam

    delta = np.random.default_rng(SEED + 24).standard_normal((n, n)).astype(np.float32)
    ds = ff.rfft(dev(delta.astype(np.float64)))
    for k in range(K):
        s = states[k].to(torch.complex128)
        N1 = N(s)
        a = E2 * s + Z * N1
        N2 = N(a)
        b = E2 * s + Z * N2
        N3 = N(b)
        c = E2 * a + Z * (2 * N3 - N1)
        dN1 = J(s, ds)
        da = E2 * ds + Z * dN1
        dN2 = J(a, da)
        db = E2 * ds + Z * dN2
        dN3 = J(b, db)
        dc = E2 * da + Z * (2 * dN3 - dN1)
        dN4 = J(c, dc)
        ds = E * ds + A * dN1 + 2 * B * (dN2 + dN3) + G * dN4
    sT, t = states[K].to(torch.complex128), tgt.to(torch.complex128)
    w = torch.full(sT.shape, 2.0, dtype=torch.float64, device=sT.device)
    w[0] = 1.0
    w[-1] = 1.0
    c1, c2 = 1.0 / (n * n) ** 2, 0.5 / (n * n) ** 2
    g = 2 * c1 * w * (sT - t) + 2 * c2 * w * sT
    dL_tan = float(torch.sum((torch.conj(g) * ds).real))
    dL_adj = float(np.sum(ff.to_numpy(gz).astype(np.float64) * delta.astype(np.float64)))
    return {"steps": K, "grid": f"{n}^2", "dL_adjoint_fp32": dL_adj, "dL_tangent_fp64_on_fp32_states": dL_tan,
            "rel_err": abs(dL_adj - dL_tan) / abs(dL_tan)}


def adjoint_512(torch, ff, ndir=8, nsteps=2000):
    """Discrete adjoint of 512^2 ETDRK4 (dt 2e-3, 2000 steps, checkpoint every 50): FP32
    forward and adjoint with FP64 gradient reductions; loss = mean((zeta_T - zeta_target)^2)
    + enstrophy(zeta_T); directional derivatives along seeded random directions against
    FP64 central differences with h in {1e-3, 1e-4, 1e-5}, and d/dnu likewise."""
    import numpy as np
    n, nu, mu, dt = 512, NU, MU, DT
    z0 = ff.Vorticity.random_phase_vorticity(n, seed=SEED + 5)
    zt = ff.Vorticity.random_phase_vorticity(n, seed=SEED + 6)
    dev = ff.device_array(ff.GPU())
    out = {"grid": "512^2", "steps": nsteps, "checkpoint_every": 50, "directions": ndir}
    res = {}
    for T, name in ((np.float32, "fp32"), (np.float64, "fp64")):
        p = ff.Vorticity.Problem(ff.GPU(), nx=n, Lx=LX, nu=nu, mu=mu, dt=dt, stepper="ETDRK4", T=T)
        adj = ff.Adjoint.VorticityAdjoint(p, checkpoint_every=50)
        tgt = ff.rfft(dev(zt.astype(T)))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        L, gz, dnu = adj.gradient(z0, tgt, nsteps)
        torch.cuda.synchronize()
        res[name] = {"loss": L, "grad": ff.to_numpy(gz).astype(np.float64), "dnu": dnu,
                     "seconds": time.perf_counter() - t0,
                     "final": ff.to_numpy(p.sol).astype(np.complex128)}
        del adj, p
    p64 = ff.Vorticity.Problem(ff.GPU(), nx=n, Lx=LX, nu=nu, mu=mu, dt=dt, stepper="ETDRK4", T=np.float64)
    a64 = ff.Adjoint.VorticityAdjoint(p64)
    tgt64 = ff.rfft(dev(zt))

    def loss_at(z, prob=p64, ad=a64):
        ff.Vorticity.set_zeta_(prob, z)
        ff.stepforward_(prob, nsteps)
        return ad.loss(tgt64)

    rng = np.random.default_rng(SEED + 7)
    worst = {name: {h: 0.0 for h in (1e-3, 1e-4, 1e-5)} for name in res}
    for _ in range(ndir):
        d = rng.standard_normal((n, n))
        for h in (1e-3, 1e-4, 1e-5):
            fd = (loss_at(z0 + h * d) - loss_at(z0 - h * d)) / (2 * h)
            for name in res:
                dl = float(np.sum(res[name]["grad"] * d))
                worst[name][h] = max(worst[name][h], abs(dl - fd) / abs(fd))
    nu_rel = {}
    for h in (1e-7, 1e-8):
        vals = []
        for sgn in (1, -1):
            pn = ff.Vorticity.Problem(ff.GPU(), nx=n, Lx=LX, nu=nu + sgn * h, mu=mu, dt=dt, stepper="ETDRK4",
                                      T=np.float64)
            an = ff.Adjoint.VorticityAdjoint(pn)
            vals.append(loss_at(z0, pn, an))
            del an, pn
        fd = (vals[0] - vals[1]) / (2 * h)
        nu_rel[f"h={h:g}"] = {name: abs(res[name]["dnu"] - fd) / abs(fd) for name in res}
    for name in res:
        out[name] = {"loss": res[name]["loss"], "d_loss_d_nu": res[name]["dnu"],
                     "gradient_seconds": res[name]["seconds"],
                     "adjoint_steps_per_s": nsteps / res[name]["seconds"],
                     "max_rel_err_vs_fp64_fd": {f"h={h:g}": v for h, v in worst[name].items()}}
    out["nu_rel_err_vs_fp64_fd"] = nu_rel
    # the FP32 adjoint against a tangent of its own map over one checkpoint segment
    out["fp32"]["segment_vs_tangent_of_fp32_map"] = fp32_adjoint_segment_check(torch, ff)
    # what bounds the FP32 figures: the FP32 forward map itself drifts from the FP64 one
    g32, g64 = res["fp32"]["grad"], res["fp64"]["grad"]
    f32, f64 = res["fp32"]["final"], res["fp64"]["final"]
    out["fp32_vs_fp64"] = {"grad_rel_l2": float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64)),
                           "final_zeta_rel_l2": float(np.linalg.norm(f32 - f64) / np.linalg.norm(f64)),
                           "loss_rel": abs(res["fp32"]["loss"] - res["fp64"]["loss"]) / abs(res["fp64"]["loss"])}
    return out


def profile_case(a):
    """Small cases for ncu, one kernel family each (a few GB on the device at most, inputs
    larger than L2 where the family's real workloads are):

      fp64 / fp32 / batch  the fused vorticity step: 1024^2 FP64 or FP32, or 4 x 1024^2 FP32
      fft        generic transforms (k_r2c_rows, k_cols, k_c2r_rows, k_c2c_rows): 2D rfft and
                 irfft of 4096^2 FP64 and FP32 fields, and a complex fft/ifft of 2048^2 FP64
      steppers   generic substep kernels (N fills, k_etd12 / k_etd3 / k_etd_update, k_rk4_*,
                 k_lsrk54, k_ab3) on a 4 x 128^3 FP32 diffusion stack run as if N were not
                 zero, then the one-pass linear step (k_linear_etd_f32x2) on the same stack
      adjoint    the vorticity adjoint (k_adj_*, ff_vadj_apply) on 512^2 FP32: a 4-step
                 gradient
      spectra    reductions: parsevalsum2 (k_parseval_partial) and radialspectrum on a
                 4096^2 FP64 half spectrum"""
    import numpy as np
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import fourierflows.jl_gb300 as ff
    torch.cuda.set_device(0)
    case = a.profile_case
    dev = ff.device_array(ff.GPU())
    rng = np.random.default_rng(5)
    if case in ("fp64", "fp32", "batch"):
        if case == "batch":
            ens = ff.Vorticity.Ensemble([(N, NU, SEED + i) for i in range(4)], mu=MU, dt=DT, T=np.float32)
            fs = ens.fs
        else:
            T = np.float64 if case == "fp64" else np.float32
            prob, fs = make_problem(ff, T)
        if a.tiles:
            fs.set_config(*[int(x) for x in a.tiles.split(",")])
        fs.advance(a.steps)
    elif case == "fft":
        for n, T in ((4096, np.float64), (4096, np.float32)):
            x = dev(rng.standard_normal((n, n)).astype(T))
            for _ in range(a.steps):
                xh = ff.rfft(x)
                x = ff.irfft(xh, n)
            del x, xh
        z = dev((rng.standard_normal((2048, 2048)) + 1j * rng.standard_normal((2048, 2048))))
        for _ in range(a.steps):
            z = ff.ifft(ff.fft(z))
    elif case == "steppers":
        kappas = 1e-3 + 9e-3 * ff.Vorticity.uniform01(77, 4)
        for stepper in ("ETDRK4", "RK4", "LSRK54", "AB3"):
            ens = ff.Diffusion.Ensemble3D(kappas, n=128, dt=DT, stepper=stepper, T=np.float32)
            ens.prob.eqn.zero_N = False  # the generic substeps, as for a nonlinear calcN!
            ens.stepforward_(a.steps)
            del ens
        ens = ff.Diffusion.Ensemble3D(kappas, n=128, dt=DT, stepper="ETDRK4", T=np.float32)
        ens.stepforward_(a.steps)
    elif case == "adjoint":
        n = 512
        p = ff.Vorticity.Problem(ff.GPU(), nx=n, Lx=LX, nu=NU, mu=MU, dt=DT, stepper="ETDRK4", T=np.float32)
        adj = ff.Adjoint.VorticityAdjoint(p, checkpoint_every=2)
        z0 = ff.Vorticity.random_phase_vorticity(n, seed=SEED + 5)
        tgt = ff.rfft(dev(ff.Vorticity.random_phase_vorticity(n, seed=SEED + 6).astype(np.float32)))
        adj.gradient(z0, tgt, max(4, a.steps))
    elif case == "spectra":
        g = ff.TwoDGrid(ff.GPU(), nx=4096, Lx=LX)
        uh = dev(rng.standard_normal((g.nkr, g.ny)) + 1j * rng.standard_normal((g.nkr, g.ny)))
        for _ in range(a.steps):
            ff.parsevalsum2(uh, g)
        ff.radialspectrum(uh, g)
    else:
        raise SystemExit(f"unknown profile case {case}")
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": case, "steps": a.steps}))


if __name__ == "__main__":
    A = args_()
    if A.profile_case:
        profile_case(A)
    elif A.impl == "reference":
        reference_arm(A)
    else:
        our_arm(A)
