"""Benchmark: pair interactions/s of the StePS direct-summation force
evaluation on one GB300, mixed precision against the plain FP64 kernel, with
the p50/p99/max relative force error of mixed against FP64.

Workload (default): compactified R^3, N = 2^20 particles (R_max = 1000 Mpc,
seeded Gaussian clustering displacement), positions FP64, masses and
softening FP32 on the device -- one full force evaluation per step
(N^2 = 1.10e12 pair interactions, self pair included as in the reference).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU implementation (the
plain-C oracle restating StePS/src/forces.cc, OpenMP over all host cores) on
a bounded i-subset sample of the same workload.

With --gpus N > 1 (torchrun) every rank evaluates its own independent
realisation (seed 1 + rank): weak scaling, no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pair interactions/s (mixed FP32-pair/FP64-accumulate force kernel), p99 force err <= 1e-5 vs FP64"
UNIT = "pairs/s"
FLOPS_PER_PAIR = 20  # R^3 convention: 3 sub, 5 r^2, 1 rsqrt, 2+1 mul, 6 acc, 1 beta add, 1 compare


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1 << 20, help="particles (default: the 2^20 workload)")
    ap.add_argument("--fp64-sample", type=int, default=16384, help="i particles timed with the FP64 kernel")
    ap.add_argument("--cpu-sample", type=int, default=1024, help="i particles in the CPU baseline sample")
    ap.add_argument("--e2e-steps", type=int, default=3)
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, v: float) -> float:
    if dist is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([c.strip() for c in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 5 + k and "Active" in r[5 + k]
                          and "Not" not in r[5 + k]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_baseline(ps, sample: int, threads: int):
    """The reference algorithm on the host cores: the plain-C oracle
    (OpenMP over i, sequential j, per-pair atomics as StePS/src/forces.cc)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    port = pyoracle.Port(threads=threads)
    s = port.system(0, ps.m, ps.eps, pyoracle.make_params())
    lo = ps.n // 2
    hi = min(ps.n - 1, lo + sample - 1)
    port.forces(s, ps.x, lo, min(hi, lo + 31))  # warm
    t0 = time.perf_counter()
    port.forces(s, ps.x, lo, hi)
    dt = time.perf_counter() - t0
    pairs = (hi - lo + 1) * ps.n
    return pairs / dt, dt, pairs, hi - lo + 1


def run_reference(args, ws, rank):
    from steps_gb300 import workloads as W

    if rank != 0:
        return
    ps = W.r3_compactified(args.n, 1000.0, seed=1, displace=True)
    threads = os.cpu_count() or 1
    rates = []
    for _ in range(max(args.warmup, 0)):
        cpu_baseline(ps, max(64, args.cpu_sample // 8), threads)
    for _ in range(args.steps):
        r, dt, pairs, ni = cpu_baseline(ps, args.cpu_sample, threads)
        rates.append(r)
    v = float(np.median(rates))
    sample = f"{args.cpu_sample} i particles x all {ps.n} j per step (force cost is linear in the i range)"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(args.cpu_sample * ps.n / v * 1e3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": f"R3 compactified N={ps.n} R_max=1000 Mpc, clustered, CPU sample"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local, dist):
    import steps_gb300 as S
    from steps_gb300 import workloads as W

    ps = W.r3_compactified(args.n, 1000.0, seed=1 + rank, displace=True)
    n = ps.n
    eng = S.Engine(local)
    eng.set_particles(ps.m, ps.eps)
    eng.upload_positions(ps.x)
    p = S.params(S.R3)
    f32_peak, f64_peak = eng.measure_peaks()

    for _ in range(args.warmup):
        eng.forces_resident(p, S.MIXED)
    eng.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    barrier(dist)
    eng.synchronize()
    launches0 = eng.launch_count()
    step_ms, kernel_ms = [], []
    for _ in range(args.steps):
        eng.flush_l2(512 << 20)  # evict L2 (129 MB) between steps; outside the step's events
        eng.mark(0)
        eng.forces_resident(p, S.MIXED)
        eng.mark(1)
        step_ms.append(eng.elapsed_ms(0, 1))
        kernel_ms.append(eng.phase_ms(1))
    eng.synchronize()
    launches = eng.launch_count() - launches0  # our kernels only (the L2 flush is a memset)
    barrier(dist)
    clk = clocks.stop()
    total_ms = allmax(dist, float(sum(step_ms)))
    pairs_step = float(n) * float(n)
    value = ws * pairs_step * args.steps / (total_ms * 1e-3)
    kern_ms = float(np.mean(kernel_ms))
    kern_rate = pairs_step / (kern_ms * 1e-3)
    Fmixed = eng.download_forces(n)

    # e2e through the host-buffer C-ABI call (H2D positions, D2H forces inside).
    F_host = np.empty((n, 3))
    e2e_s = []
    for _ in range(args.e2e_steps):
        barrier(dist)
        t0 = time.perf_counter()
        F_host = eng.forces(ps.x, p, S.MIXED)
        e2e_s.append(time.perf_counter() - t0)
    e2e_t = allmax(dist, float(np.mean(e2e_s)))
    e2e_value = ws * pairs_step / e2e_t

    # FP64 kernel on an i subset (cost is linear in the i range) + accuracy.
    lo = n // 2 - args.fp64_sample // 2
    hi = lo + args.fp64_sample - 1
    eng.forces_resident(p, S.FP64, lo, hi)
    eng.synchronize()
    f64_ms = eng.phase_ms(1)
    f64_total_ms = eng.phase_ms(0) + eng.phase_ms(1) + eng.phase_ms(2)
    F64 = eng.download_forces(hi - lo + 1)
    f64_rate = args.fp64_sample * n / (f64_ms * 1e-3)
    rel = np.linalg.norm(Fmixed[lo:hi + 1] - F64, axis=1) / np.linalg.norm(F64, axis=1)
    acc = {"p50": float(np.percentile(rel, 50)), "p99": float(np.percentile(rel, 99)), "max": float(rel.max()),
           "sample": f"{args.fp64_sample} i particles vs the FP64 kernel"}
    mixed_f64_rel = np.linalg.norm(F_host - Fmixed, axis=1).max()

    achieved = kern_rate * FLOPS_PER_PAIR / 1e12
    nominal = 152 * 128 * 2 * 2070e6 / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.mean(step_ms)), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 pairs / f64 accumulate (positions f64)", "data": "synthetic (seeded; no public dataset)",
        "config": {"workload": f"R3 compactified N={n} R_max=1000 Mpc, clustered (sigma=0.5 spacing), one full "
                               f"force evaluation per step", "n": n, "pairs_per_step": pairs_step,
                   "parallelism": "one independent realisation per GPU" if ws > 1 else "1 GPU",
                   "l2": "512 MB flush between steps", "precision": "mixed"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(ps.x.nbytes),
                "d2h_bytes_per_step": int(F_host.nbytes), "ms_per_step": e2e_t * 1e3},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": f32_peak / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / (f32_peak / 1e12), "traffic": None,
                     "peak_kind": "FP32 FMA issue peak measured in this process (dependent-FMA-chain kernel)",
                     "nominal_peak_at_max_clock": nominal, "frac_of_nominal": achieved / nominal,
                     "flops_per_pair": FLOPS_PER_PAIR, "kernel_ms": kern_ms},
        "fp64": {"pairs_per_s": f64_rate, "kernel_ms": f64_ms, "sample_i": args.fp64_sample,
                 "frac_of_fp64_peak": f64_rate * FLOPS_PER_PAIR / f64_peak, "fp64_peak_tflops": f64_peak / 1e12},
        "speedup_vs_fp64": kern_rate / f64_rate,
        "accuracy_mixed_vs_fp64": acc,
        "e2e_vs_resident_max_abs_diff": float(mixed_f64_rel),
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    return line


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    dist = dist_init(ws)
    line = run_ours(args, ws, rank, local, dist)
    if rank == 0:
        from steps_gb300 import workloads as W

        threads = os.cpu_count() or 1
        psb = W.r3_compactified(args.n, 1000.0, seed=1, displace=True)
        rate, dt, pairs, ni = cpu_baseline(psb, args.cpu_sample, threads)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{ni} i particles x all {psb.n} j ({dt:.1f} s of CPU work)"}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
