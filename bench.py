"""Benchmark: pair interactions/s of the StePS direct-summation force
evaluation on one GB300, mixed precision against the plain FP64 kernel, with
the p50/p99/max relative force error of mixed against FP64.

Default workload (the headline): compactified R^3, N = 2^20 particles
(R_max = 1000 Mpc, seeded Gaussian clustering displacement), positions FP64,
masses and softening FP32 on the device -- one full force evaluation per
step (N^2 = 1.10e12 pair interactions, self pair included as in the
reference). Other workloads (--workload):
  cfg0  R^3 compactified, N = 32768, R_max = 480 Mpc
  cfg2  S1xR2, N = 2^21, L_z = 200 Mpc, R_max = 600 Mpc, 7 periodic images (IS_PERIODIC = 2)
  cfg3  T^3, N = 2^19, L = 100 Mpc, clumpy, Ewald table Ng = 63 (trilinear; --order 4 tricubic)
  cfg4  64 independent R^3 realisations of uneven N, 1 force + 10 KDK steps in one CUDA graph

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload cfg1]

--impl reference times the reference algorithm's CPU implementation (the
plain-C oracle restating StePS/src/forces.cc, OpenMP over all host cores) on
a bounded i-subset sample of the same workload. With --ref-device gpu it
times instead the reference's own CUDA kernels (StePS/src/forces_cuda.cu,
compiled unmodified into oracle/_ref/*.cubin) with the reference's launch
shape, in its FP32 and FP64 builds, on one full wave of i particles against a
j subset sized to about --ref-seconds per launch.

The default run (cfg1 at one GPU) also measures every other workload in a
`configs` block of the same JSON line -- cfg0 (one force evaluation per
step, and as specified: one force + 4 KDK steps, mixed and FP64), cfg2 with
the image sum and with the (rho, z) table at orders 0/2/4, cfg3 at orders 2/4
and on the IS_PERIODIC = 3 table (Ng = 127), cfg4 as one persistent kernel
against a per-phase graph and plain launches -- each
with its pair rate, issue-roofline fraction, FP64 rate, p50/p99/max against
FP64 and a short CPU baseline; and a `ref_gpu` block timing the reference's
own CUDA kernels (FP32 and FP64 builds) on the R^3, T^3 and S1xR2 workloads.
--no-configs skips both.

With --gpus N > 1 (torchrun) every rank evaluates its own independent
realisation (seed + rank): weak scaling, no collective on the data path.
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

# Ewald table of the T^3 workload: Ng = 63, alpha = 2/L, real images |r+nL| <= 2L
# (index radius 3), k vectors |k| <= 5 (2 pi / L) (index radius 6).
T3_NG = 63
LOOPS = ["fp32", "fp32x2", "fp32x2 (768 threads/SM)", "fp32x2 (1024 threads/SM)", "fp32x2, bulk-copy mbarrier pipeline"]
# DRAM bytes (read + write) of one launch of the pair kernel, from one-pass ncu
# captures of dram__bytes_read.sum + dram__bytes_write.sum, keyed by
# (workload, N, threads, ipt, pair-loop variant): the traffic is reported only
# for the shape that was timed, else null.
# N = 2^20 R^3 (cfg1), one launch each (-s 1 -c 1, after the warm-up launch):
# about 110 MB read (particles, tiles) and 1.6 GB written (the FP64 partial
# sums of 64 j chunks per i particle).
NCU_TRAFFIC = {("cfg1", 1 << 20, 128, 2, 1): 110.01e6 + 1.60e9,
               ("cfg1", 1 << 20, 128, 2, 4): 111.90e6 + 1.60e9,
               ("cfg1", 1 << 20, 256, 1, 2): 107.21e6 + 1.59e9}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ref-device", default="cpu", choices=["cpu", "gpu"],
                    help="--impl reference: the reference's CPU path (default) or its own CUDA kernels")
    ap.add_argument("--ref-seconds", type=float, default=1.0, help="--ref-device gpu: target time of one launch")
    ap.add_argument("--workload", default="cfg1", choices=["cfg0", "cfg1", "cfg2", "cfg3", "cfg4"])
    ap.add_argument("--batch-scale", type=float, default=1.0, help="cfg4: scale every N_k (small test runs)")
    ap.add_argument("--order", type=int, default=2,
                    help="T^3 interpolation order (2 or 4); S1xR2 table order (0, 2 or 4)")
    ap.add_argument("--s1-table", action="store_true",
                    help="cfg2 with the (rho, z) correction table instead of the image sum")
    ap.add_argument("--n", type=int, default=0, help="override the particle count (small profiling cases)")
    ap.add_argument("--fp64-sample", type=int, default=16384, help="i particles timed with the FP64 kernel")
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="i particles in the CPU baseline sample (0: sized for --cpu-seconds)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="target CPU time of one baseline sample")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--variant", type=int, default=-1,
                    help="R^3 pair loop without autotuning: 0 fp32, 1 fp32x2, 2/3 fp32x2 at 768/1024 threads per SM, "
                         "4 fp32x2 with the bulk-copy pipeline")
    ap.add_argument("--shape", default="", help="kernel shape THREADSxIPT without autotuning, e.g. 128x1")
    ap.add_argument("--t3-level", type=int, default=0,
                    help="cfg3: Ewald table of the reference's IS_PERIODIC level 3 (Ng = 127, rel_cut 3.6, rec_cut 10) "
                         "instead of the workload's Ng = 63 table")
    ap.add_argument("--no-configs", action="store_true", help="skip the configs and ref_gpu blocks")
    return ap.parse_args()


def workload(args, rank=0):
    """Particles, parameters, the flop convention of one pair, a description
    and (T^3) the Ewald table arguments."""
    import steps_gb300 as S
    from steps_gb300 import workloads as W

    w = args.workload
    if w in ("cfg0", "cfg1"):
        n = args.n or (32768 if w == "cfg0" else 1 << 20)
        rmax = 480.0 if w == "cfg0" else 1000.0
        ps = W.r3_compactified(n, rmax, seed=(0 if w == "cfg0" else 1) + rank, displace=(w == "cfg1"))
        desc = f"R3 compactified N={n} R_max={rmax:g} Mpc" + (", clustered (sigma=0.5 spacing)" if w == "cfg1" else "")
        return ps, S.params(S.R3), 20, desc, None
    if w == "cfg4":
        # The reference arms time the ensemble's force path on its largest
        # realisation: the per-pair cost does not depend on N.
        sets = W.r3_ensemble(64, scale=args.batch_scale)
        k = int(np.argmax([s.n for s in sets]))
        desc = (f"batched ensemble of {len(sets)} R3 realisations (N_k log-uniform [8192, 262144]), "
                f"timed on its largest, realisation {k} (N={sets[k].n})")
        return sets[k], S.params(S.R3), 20, desc, None
    if w == "cfg2":
        n = args.n or (1 << 21)
        ps = W.s1r2_cylindrical(n, 200.0, 600.0, seed=2 + rank)
        if args.s1_table:
            # The (rho, z) table with the reference's IS_PERIODIC = 2 settings
            # (StePS/src/main.cc:569-602): N_z = 128, N_rho = floor(N_z 2.25 Rsim / L),
            # alpha L = 0.787875, n_max = 4, m_max = 10; interpolation order --order.
            nz = 128
            nrho = int(math.floor(nz * 2.25 * 600.0 / 200.0))
            p = S.params(S.S1R2, is_periodic=2, L=200.0, rsim=600.0, s1r2_images=0, ewald_order=args.order)
            table = {"kind": "s1", "args": (nrho, nz, 2.25 * 600.0, 200.0, 0.787875 / 200.0, 4, 10)}
            flops = 33 + {0: 2, 2: 24, 4: 56}[args.order]  # pair part as T^3 + NGP / CIC / TSC taps
            return ps, p, flops, (f"S1xR2 N={n} L_z=200 Mpc R_max=600 Mpc, (rho, z) correction table "
                                           f"{nrho}x{nz} order {args.order} (IS_PERIODIC=2)"), table
        p = S.params(S.S1R2, is_periodic=2, L=200.0, rsim=600.0, s1r2_images=1)
        return ps, p, 11 + 11 * 7, f"S1xR2 N={n} L_z=200 Mpc R_max=600 Mpc, 7 z images (IS_PERIODIC=2)", None
    n = args.n or (1 << 19)
    ps = W.t3_clumpy(n, 100.0, seed=3 + rank)
    flops = 33 + (494 if args.order == 4 else 62)
    if getattr(args, "t3_level", 0) == 3:
        # The reference's IS_PERIODIC = 3 table (StePS/src/main.cc:433-440):
        # Ng = 127, alpha = 2/L, rel_cut 3.6, rec_cut 10 over ewald_space(rel_cut + 1)
        # and ewald_space(rec_cut + 2).
        p = S.params(S.T3, is_periodic=3, L=100.0, rsim=50.0, ewald_order=args.order)
        table = {"kind": "t3", "args": (127, 100.0, 2.0 / 100.0, 3.6, 10.0, 4.6, 12.0)}
        return ps, p, flops, (f"T3 N={n} L=100 Mpc clumpy, IS_PERIODIC=3 Ewald table Ng=127 (rel_cut 3.6, rec_cut 10) "
                              f"order {args.order}"), table
    p = S.params(S.T3, is_periodic=2, L=100.0, rsim=50.0, ewald_order=args.order)
    table = {"kind": "t3", "args": (T3_NG, 100.0, 2.0 / 100.0, 2.0, 5.0 * 2.0 * math.pi / 100.0, 3.0, 6.0)}
    return ps, p, flops, f"T3 N={n} L=100 Mpc clumpy, Ewald table Ng={T3_NG} order {args.order}", table


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
        pw = [float(r[3]) for r in self.rows if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 5 + k and "Active" in r[5 + k]
                          and "Not" not in r[5 + k]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_median": float(np.median(pw)) if pw else None, "reasons": reasons,
                "samples": len(self.rows)}


def cpu_baseline(ps, p, sample: int, threads: int, table=None, seconds: float = 10.0):
    """The reference algorithm on the host cores: the plain-C oracle (OpenMP
    over i, sequential j, per-pair atomics, as StePS/src/forces.cc) built with
    the reference's release flags (-O3 -ffast-math), timed on the i range
    [N/2, N/2 + sample) against all N j. sample <= 0 sizes the range from a
    short calibration run so that it takes about `seconds`."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    port = pyoracle.Port(threads=threads, release=True)
    tp = {0: 0, 1: 1, 2: 3 if p.s1r2_images else 2}[p.topology]
    tab, ng, nrho, nz = table if table else (None, 0, 0, 0)
    s = port.system(tp, ps.m, ps.eps, pyoracle.make_params(p.is_periodic, p.L, p.rsim), table=tab, ngrid=ng,
                    nrho=nrho, nz=nz, order=p.ewald_order)
    lo = ps.n // 2
    probe = min(max(threads, 8), ps.n - lo)
    port.forces(s, ps.x, lo, lo + probe - 1)  # warm-up: threads, pages
    target = min(1.0, seconds / 4)
    while True:  # calibration: grow the probe until it takes `target` seconds
        t0 = time.perf_counter()
        port.forces(s, ps.x, lo, lo + probe - 1)
        dt = time.perf_counter() - t0
        if dt >= target or probe >= ps.n - lo:
            break
        probe = min(max(2 * probe, int(probe * target / max(dt, 1e-9))), ps.n - lo)
    if sample <= 0:
        sample = int(probe * seconds / max(dt, 1e-9))
    # whole rounds of the thread team, at least 4 i per thread (OpenMP static schedule)
    sample = max(4 * threads, -(-sample // threads) * threads)
    sample = max(8, min(sample, ps.n - lo))
    hi = lo + sample - 1
    t0 = time.perf_counter()
    port.forces(s, ps.x, lo, hi)
    dt = time.perf_counter() - t0
    pairs = (hi - lo + 1) * ps.n
    return pairs / dt, dt, pairs, hi - lo + 1


def host_table(table, eng=None):
    """The workload's Ewald table for the CPU baseline as (table, ngrid, nrho, nz):
    the GPU-built table when an engine holds it (the builders match the
    reference's to 1e-13), else the oracle's builder on the host."""
    if table is None:
        return None
    if table["kind"] == "t3":
        ng = table["args"][0]
        if eng is not None:
            return eng.get_table_t3(ng), ng, 0, 0
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle

        return pyoracle.Port().t3_table(*table["args"]), ng, 0, 0
    nrho, nz = table["args"][:2]
    if eng is not None:
        return eng.get_table_s1r2(nrho, nz), 0, nrho, nz
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    return pyoracle.Port().s1r2_table(*table["args"]), 0, nrho, nz


def run_reference(args, ws, rank):
    if rank != 0:
        return
    ps, p, flops, desc, table = workload(args)
    tab = host_table(table)
    threads = os.cpu_count() or 1
    for _ in range(max(args.warmup, 0)):
        cpu_baseline(ps, p, 0, threads, tab, seconds=args.cpu_seconds / 8)
    runs = [cpu_baseline(ps, p, args.cpu_sample, threads, tab, seconds=args.cpu_seconds)
            for _ in range(args.steps)]
    v = float(np.median([r[0] for r in runs]))
    sample = runs[0][3]
    smp = (f"{sample} i particles x all {ps.n} j per step, about {args.cpu_seconds:g} s of CPU work each "
           "(force cost is linear in the i range)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(sample * ps.n / v * 1e3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": desc + ", CPU sample"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": smp,
                             "build": "oracle port, -O3 -ffast-math (the reference's release flags)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def set_ref_table(k, tab):
    """Hands host_table()'s (table, ngrid, nrho, nz) to a reference kernel."""
    if tab is None:
        return
    if tab[1]:
        k.set_table_t3(tab[0], tab[1])
    else:
        k.set_table_s1r2(tab[0], tab[2], tab[3])


def ref_gpu_measure(args, ps, p, flops, desc, table, seconds, steps, warmup):
    """The reference's CUDA kernels (oracle/refgpu.py) on one workload: FP32
    build (USE_SINGLE_PRECISION) and FP64 build, kernel time only, with the
    FP32 build's error against the FP64 build on the same sample. None when the
    cubins were not built."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import refgpu

    base = {0: "r3", 1: "t3", 2: "s1nl"}[p.topology]
    if p.topology == 1:
        flops = 33 + 494  # the reference GPU kernel interpolates T^3 tricubically only
    if table and table["kind"] == "s1":
        base = f"s1o{p.ewald_order}"
    if not (refgpu.available(base) and refgpu.available(base + "sp")):
        return None
    kw = {}
    if p.topology == 1:
        kw = {"is_periodic": p.is_periodic, "L": p.L}
    elif p.topology == 2:
        kw = {"is_periodic": p.is_periodic, "L": p.L, "rsim": p.rsim}
    tab = host_table(table)
    res = {}
    for v in (base + "sp", base):
        k = refgpu.RefKernel(v)
        k.set_particles(ps.x, ps.m, ps.eps)
        set_ref_table(k, tab)
        ni = min(ps.n, k.wave())
        nj = min(ps.n, 1024)
        ms, _ = k.time(0, ni - 1, nj, steps=1, warmup=1, **kw)  # calibration
        nj = int(min(ps.n, max(nj, nj * seconds * 1e3 / max(ms, 1e-3))))
        ms, F = k.time(0, ni - 1, nj, steps=steps, warmup=warmup, **kw)
        res[v] = {"pairs_per_s": ni * nj / (ms * 1e-3), "kernel_ms": ms, "i": ni, "j": nj, "F": F,
                  "registers": k.registers, "blocks_per_sm": k.blocks_per_sm}
    a, b = res[base + "sp"], res[base]
    Fb = b["F"]
    if a["j"] == b["j"]:
        Fa = a["F"]
    else:  # the FP32 build on the FP64 build's sample for the error figures
        k = refgpu.RefKernel(base + "sp")
        k.set_particles(ps.x, ps.m, ps.eps)
        set_ref_table(k, tab)
        Fa = k.forces(0, b["i"] - 1, b["j"], **kw)
    rel = np.linalg.norm(Fa - Fb, axis=1) / np.maximum(np.linalg.norm(Fb, axis=1), 1e-300)
    interp = ", tricubic (the reference GPU kernel's only T^3 interpolation)" if p.topology == 1 else ""
    return {"workload": desc + interp, "kernel": base, "flops_per_pair": flops,
            "sample": f"i = one full wave of resident blocks ({a['i']}), j = the first {a['j']} particles "
                      f"(FP64 build: {b['j']}); pair cost does not depend on N",
            "fp32_build": {k_: a[k_] for k_ in ("pairs_per_s", "kernel_ms", "i", "j", "registers", "blocks_per_sm")},
            "fp64_build": {k_: b[k_] for k_ in ("pairs_per_s", "kernel_ms", "i", "j", "registers", "blocks_per_sm")},
            "accuracy_fp32_vs_fp64": {"p50": float(np.percentile(rel, 50)), "p99": float(np.percentile(rel, 99)),
                                      "max": float(rel.max()), "sample": f"{b['i']} i x {b['j']} j"}}


def run_reference_gpu(args, ws, rank):
    """--impl reference --ref-device gpu: the reference's CUDA kernels on the
    chosen workload, as its own JSON line."""
    if rank != 0:
        return
    ps, p, flops, desc, table = workload(args)
    r = ref_gpu_measure(args, ps, p, flops, desc, table, args.ref_seconds, args.steps, args.warmup)
    if r is None:
        print(json.dumps({"impl": "reference", "device": "gpu", "unavailable":
                          "oracle/_ref/forces_cuda_*.cubin not built (needs the reference tree at build time)"}),
              flush=True)
        return
    a = r["fp32_build"]
    v = a["pairs_per_s"]
    line = {"impl": "reference", "device": "gpu", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": a["kernel_ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (the reference's USE_SINGLE_PRECISION build)",
            "data": "synthetic (seeded)",
            "config": {"workload": r["workload"], "sample": r["sample"],
                       "launch": "32 x SMs blocks of 256 threads, grid-stride i loop (StePS/src/forces_cuda.cu:1053)",
                       "source": "StePS/src/forces_cuda.cu compiled unmodified for sm_103a (nvcc -O3)"},
            "roofline": {"bound": "fp32", "achieved": v * r["flops_per_pair"] / 1e12, "unit": "TFLOP/s",
                         "flops_per_pair": r["flops_per_pair"]},
            "fp32_build": a, "fp64_build": r["fp64_build"], "accuracy_fp32_vs_fp64": r["accuracy_fp32_vs_fp64"],
            "e2e": None, "e2e_note": "kernel time only; the reference wrapper's per-call allocations and copies "
                                     "(forces_cuda.cu:976-1105) are not timed"}
    print(json.dumps(line), flush=True)


def nominal_fp32_peak(sm_mhz):
    """FP32 FMA issue peak from the device's SM count and the sampled SM clock
    (128 FP32 lanes per SM, an FMA counted as 2 flops), TFLOP/s."""
    try:
        import torch

        nsm = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        return None, None
    if not sm_mhz:
        return None, nsm
    return nsm * 128 * 2 * sm_mhz * 1e6 / 1e12, nsm


def setup_engine_workload(eng, ps, table):
    eng.set_particles(ps.m, ps.eps)
    if table and table["kind"] == "t3":
        eng.build_table_t3(*table["args"])
    elif table:
        eng.build_table_s1r2(*table["args"])
    eng.upload_positions(ps.x)


def measure(eng, S, ps, p, flops, table, steps, warmup, fp64_sample, f32_peak, f64_peak, shape_fixed=False,
            flush=True):
    """One workload on the resident engine: autotune (unless the shape is
    fixed), warm-up, `steps` timed force evaluations (CUDA events on the
    library stream, L2 flushed between them), the FP64 kernel on an i sample
    and the mixed kernel's error against it. Positions must be resident."""
    n = ps.n
    t_tune = time.perf_counter()
    shape = None if shape_fixed else eng.autotune(p)
    t_tune = time.perf_counter() - t_tune
    for _ in range(warmup):
        eng.forces_resident(p, S.MIXED)
    eng.synchronize()
    launches0 = eng.launch_count()
    step_ms, kernel_ms, prep_ms = [], [], []
    for _ in range(steps):
        if flush:
            eng.flush_l2(512 << 20)  # evict L2 (129 MB) between steps; outside the step's events
        eng.mark(0)
        eng.forces_resident(p, S.MIXED)
        eng.mark(1)
        step_ms.append(eng.elapsed_ms(0, 1))
        prep_ms.append(eng.phase_ms(0))
        kernel_ms.append(eng.phase_ms(1))
    eng.synchronize()
    launches = eng.launch_count() - launches0
    pairs_step = float(n) * float(n)
    kern_ms = float(np.mean(kernel_ms))
    kern_rate = pairs_step / (kern_ms * 1e-3)
    Fmixed = eng.download_forces(n)
    fs = min(fp64_sample, n)
    lo = n // 2 - fs // 2
    hi = lo + fs - 1
    eng.forces_resident(p, S.FP64, lo, hi)
    eng.synchronize()
    f64_ms = eng.phase_ms(1)
    F64 = eng.download_forces(hi - lo + 1)
    f64_rate = fs * n / (f64_ms * 1e-3)
    rel = np.linalg.norm(Fmixed[lo:hi + 1] - F64, axis=1) / np.linalg.norm(F64, axis=1)
    achieved = kern_rate * flops / 1e12
    return {
        "step_ms": step_ms, "kernel_ms": kern_ms, "prep_ms": float(np.mean(prep_ms)), "kern_rate": kern_rate,
        "value": pairs_step * steps / (float(sum(step_ms)) * 1e-3), "shape": shape, "launches": int(launches),
        "autotune_s": None if shape_fixed else t_tune,
        "achieved": achieved, "frac": achieved / (f32_peak / 1e12), "Fmixed": Fmixed,
        "fp64": {"pairs_per_s": f64_rate, "kernel_ms": f64_ms, "sample_i": fs,
                 "frac_of_fp64_peak": f64_rate * flops / f64_peak, "fp64_peak_tflops": f64_peak / 1e12},
        "speedup_vs_fp64": kern_rate / f64_rate,
        "accuracy": {"p50": float(np.percentile(rel, 50)), "p99": float(np.percentile(rel, 99)),
                     "max": float(rel.max()), "sample": f"{fs} i particles vs the FP64 kernel"},
    }


def shape_desc(shape, args):
    """The kernel shape; the variant names the R^3 pair loop, or for T^3 with
    a table the lane mapping (the other workloads have one pair loop)."""
    w = getattr(args, "workload", "cfg1")
    table_t3 = w == "cfg3"

    def loop(v):
        if w in ("cfg0", "cfg1", "cfg4"):
            return LOOPS[v]
        if table_t3:
            return "quad lanes" if v == 1 else "one i per lane"
        return "fp32"

    if shape:
        return {"threads": shape[0], "ipt": shape[1], "pair_loop": loop(shape[2])}
    return (args.shape or "128x2") + " " + loop(max(args.variant, 0))


def traffic_of(workload_name, n, shape):
    if not shape:
        return None
    return NCU_TRAFFIC.get((workload_name, n, shape[0], shape[1], shape[2]))


def run_ours(args, ws, rank, local, dist):
    import steps_gb300 as S

    ps, p, flops, desc, table = workload(args, rank)
    n = ps.n
    eng = S.Engine(local)
    setup_engine_workload(eng, ps, table)
    f32_peak, f64_peak = eng.measure_peaks()
    if args.variant >= 0:
        eng.set_variant(args.variant)
    if args.shape:
        th, ipt = (int(v) for v in args.shape.split("x"))
        eng.set_tuning(th, ipt, 0)
    fixed = args.no_autotune or args.variant >= 0 or bool(args.shape)
    shape_used = None
    if args.shape and args.variant >= 0:
        shape_used = (int(args.shape.split("x")[0]), int(args.shape.split("x")[1]), args.variant)

    clocks = ClockSampler(local)
    clocks.start()
    barrier(dist)
    r = measure(eng, S, ps, p, flops, table, args.steps, args.warmup, args.fp64_sample, f32_peak, f64_peak,
                shape_fixed=fixed)
    barrier(dist)
    clk = clocks.stop()
    total_ms = allmax(dist, float(sum(r["step_ms"])))
    pairs_step = float(n) * float(n)
    value = ws * pairs_step * args.steps / (total_ms * 1e-3)
    Fmixed = r["Fmixed"]

    # e2e through the host-buffer C-ABI call (H2D positions, D2H forces inside),
    # the host arrays in page-locked memory; and the same with ordinary
    # (pageable) arrays, as the reference's driver hands over malloc memory.
    x_pin = eng.host_array(ps.x.shape)
    x_pin[...] = ps.x
    F_host = eng.host_array((n, 3))
    e2e_s, e2e_pg = [], []
    for _ in range(args.e2e_steps):
        barrier(dist)
        t0 = time.perf_counter()
        eng.forces(x_pin, p, S.MIXED, out=F_host)
        e2e_s.append(time.perf_counter() - t0)
    x_pg = np.array(ps.x, copy=True)
    F_pg = np.empty((n, 3))
    for _ in range(args.e2e_steps):
        t0 = time.perf_counter()
        eng.forces(x_pg, p, S.MIXED, out=F_pg)
        e2e_pg.append(time.perf_counter() - t0)
    e2e_t = allmax(dist, float(np.mean(e2e_s)))
    e2e_value = ws * pairs_step / e2e_t

    nominal, nsm = nominal_fp32_peak(clk.get("sm_mhz"))
    achieved = r["achieved"]
    timed_shape = r["shape"] or shape_used
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.mean(r["step_ms"])), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 pairs / f64 accumulate (positions f64)",
        "data": "synthetic (seeded; no public dataset)",
        "config": {"workload": desc + ", one full force evaluation per step", "n": n, "pairs_per_step": pairs_step,
                   "parallelism": "one independent realisation per GPU" if ws > 1 else "1 GPU",
                   "l2": "512 MB flush between steps", "precision": "mixed",
                   "kernel_shape": shape_desc(r["shape"], args), "prep_ms": r["prep_ms"],
                   "autotune_s": r["autotune_s"]},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(x_pin.nbytes),
                "d2h_bytes_per_step": int(F_host.nbytes), "ms_per_step": e2e_t * 1e3,
                "host_memory": "page-locked (steps_gpu_host_alloc)"},
        "e2e_pageable": {"value": pairs_step / float(np.mean(e2e_pg)), "unit": UNIT,
                         "ms_per_step": float(np.mean(e2e_pg)) * 1e3,
                         "host_memory": "ordinary malloc'd numpy arrays, as the reference's driver passes x and F"},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": f32_peak / 1e12, "unit": "TFLOP/s",
                     "frac": r["frac"], "traffic": traffic_of(args.workload, n, timed_shape),
                     "traffic_note": "DRAM bytes of one pair-kernel launch from an ncu capture of the timed shape "
                                     "(null: no capture of this shape); compute-bound",
                     "peak_kind": "FP32 FMA issue peak measured in this process (dependent-FMA-chain kernel); "
                                  "MEASURED_PEAKS.json holds HBM and bf16-tensor figures only",
                     "nominal_peak_at_sampled_clock": nominal, "sms": nsm,
                     "frac_of_nominal": achieved / nominal if nominal else None,
                     "flops_per_pair": flops, "kernel_ms": r["kernel_ms"]},
        "fp64": r["fp64"],
        "speedup_vs_fp64": r["speedup_vs_fp64"],
        "accuracy_mixed_vs_fp64": r["accuracy"],
        "e2e_vs_resident_max_abs_diff": float(np.abs(F_host - Fmixed).max()),
        "gpu_launches": r["launches"],
        "clocks": clk,
    }
    eng.free_host_arrays()
    return line, ps, p, host_table(table, eng), eng, (f32_peak, f64_peak)


def kdk_measure(eng, S, W, ps, steps, warmup, f32_peak, nkdk=4, dt=1e-3):
    """The N = 32,768 workload as specified: one force evaluation, then
    `nkdk` KDK steps at fixed dt from rest (steps_gpu_forces_resident +
    steps_gpu_kdk), in mixed precision and in FP64. A step is the whole
    sequence, CUDA events around it; the uploads of the start state are
    outside. Mixed R^3 KDK steps rebuild the tiles in the previous Morton
    order between re-sorts."""
    import math

    n = ps.n
    p = S.params(S.R3)
    rho_part = float(ps.m.min()) / (4.0 * math.pi * W.PARTICLE_RADII ** 3 / 3.0)
    zeros = np.zeros_like(ps.x)
    eng.set_particles(ps.m, ps.eps)
    eng.upload_positions(ps.x)
    t_tune = time.perf_counter()
    shape = eng.autotune(p)
    t_tune = time.perf_counter() - t_tune
    res = {}
    for name, prec in (("mixed", S.MIXED), ("fp64", S.FP64)):
        ms = []
        for it in range(warmup + steps):
            eng.upload_positions(ps.x)
            eng.upload_velocities(zeros)
            eng.mark(0)
            eng.forces_resident(p, prec)
            eng.kdk(p, prec, nkdk, dt, rho_part=rho_part)
            eng.mark(1)
            if it >= warmup:
                ms.append(eng.elapsed_ms(0, 1))
        res[name] = {"ms_per_step": float(np.mean(ms)), "x": eng.state()[0], "F": eng.state()[2]}
    pairs = (nkdk + 1) * float(n) * float(n)
    x, F = res["mixed"]["x"], res["mixed"]["F"]
    fs = min(2048, n)
    lo = n // 2 - fs // 2
    eng.upload_positions(x)
    eng.forces_resident(p, S.FP64, lo, lo + fs - 1)
    F64 = eng.download_forces(fs)
    rel = np.linalg.norm(F[lo:lo + fs] - F64, axis=1) / np.linalg.norm(F64, axis=1)
    value = pairs / (res["mixed"]["ms_per_step"] * 1e-3)
    f64_value = pairs / (res["fp64"]["ms_per_step"] * 1e-3)
    return {"workload": f"R3 compactified N={n} R_max=480 Mpc: one force evaluation + {nkdk} KDK steps at dt={dt} "
                        f"from rest (the workload as specified), mixed and FP64",
            "value": value, "unit": UNIT, "ms_per_step": res["mixed"]["ms_per_step"], "steps": steps,
            "pairs_per_step": pairs, "kernel_shape": shape_desc(shape, argparse.Namespace(shape="", variant=-1, workload="cfg0")),
            "autotune_s": t_tune,
            "roofline": {"bound": "fp32", "frac_of_step": value * 20 / f32_peak, "peak": f32_peak / 1e12,
                         "flops_per_pair": 20,
                         "note": "whole step (ordering, tiling, kicks and drifts included) over the FP32 peak"},
            "fp64": {"pairs_per_s": f64_value, "ms_per_step": res["fp64"]["ms_per_step"]},
            "speedup_vs_fp64": value / f64_value,
            "accuracy_mixed_vs_fp64": {"p50": float(np.percentile(rel, 50)), "p99": float(np.percentile(rel, 99)),
                                       "max": float(rel.max()),
                                       "sample": f"{fs} i particles: final mixed forces vs the FP64 kernel at the "
                                                 f"final positions"}}


def batch_measure(eng, S, sets, steps, warmup, f32_peak, plain_steps=1):
    """Workload 4: independent compactified R^3 realisations; one force
    evaluation + 10 fixed-dt KDK steps as one persistent kernel under a CUDA
    graph, against a CUDA graph of per-phase kernels and against
    per-realisation plain launches."""
    nsteps, h = 10, 1e-3
    pairs = (nsteps + 1) * float(sum(float(s.n) ** 2 for s in sets))
    p = S.params(S.R3)
    xs, ms, es = [s.x for s in sets], [s.m for s in sets], [s.eps for s in sets]
    eng.set_variant(1)

    def timed(graph):
        eng.batch_set(xs, ms, es)
        eng.mark(2)
        eng.batch_run(p, S.MIXED, nsteps, h, graph=graph)
        eng.mark(3)
        return eng.elapsed_ms(2, 3)

    for _ in range(max(1, warmup)):  # tunes the persistent kernel and captures its graph
        timed(1)
    launches0 = eng.launch_count()
    g_ms = [timed(1) for _ in range(steps)]
    launches = eng.launch_count() - launches0
    x0, v0, F0 = eng.batch_get(0)  # the persistent run's final state
    timed(2)  # tunes the per-phase graph
    pp_ms = [timed(2) for _ in range(max(1, plain_steps))]
    plain_ms = [timed(0) for _ in range(max(1, plain_steps))]
    # accuracy spot check: realisation 0's last forces against the FP64 kernel at the same positions
    eng.set_particles(sets[0].m, sets[0].eps)
    F64 = eng.forces(x0, p, S.FP64)
    rel = np.linalg.norm(F0 - F64, axis=1) / np.linalg.norm(F64, axis=1)
    gt = float(np.median(g_ms))
    pt = float(np.median(plain_ms))
    ppt = float(np.median(pp_ms))
    value = pairs / (gt * 1e-3)
    return {"value": value, "ms_per_step": gt, "pairs_per_step": pairs, "steps": steps, "launches": int(launches),
            "total_particles": int(sum(s.n for s in sets)),
            "plain_launches": {"pairs_per_s": pairs / (pt * 1e-3), "ms_per_step": pt,
                               "what": "per-realisation force launches + KDK kernels"},
            "per_phase_graph": {"pairs_per_s": pairs / (ppt * 1e-3), "ms_per_step": ppt,
                                "what": "one CUDA graph of per-phase kernels, re-ordering every step"},
            "speedup_graph_vs_plain": pt / gt, "speedup_vs_per_phase_graph": ppt / gt, "frac": value * 20 / f32_peak,
            "accuracy": {"p50": float(np.percentile(rel, 50)), "p99": float(np.percentile(rel, 99)),
                         "max": float(rel.max()),
                         "sample": f"realisation 0 (N={sets[0].n}) after the run, vs the FP64 kernel"}}


def run_batch(args, ws, rank, local, dist):
    import steps_gb300 as S
    from steps_gb300 import workloads as W

    sets = W.r3_ensemble(64, scale=args.batch_scale)
    eng = S.Engine(local)
    f32_peak, _ = eng.measure_peaks()
    clocks = ClockSampler(local)
    clocks.start()
    r = batch_measure(eng, S, sets, args.steps, args.warmup, f32_peak, plain_steps=max(1, args.steps // 2))
    clk = clocks.stop()
    gt = allmax(dist, r["ms_per_step"])
    value = ws * r["pairs_per_step"] / (gt * 1e-3)
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": gt, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 pairs / f64 accumulate (positions f64)", "data": "synthetic (seeded; no public dataset)",
        "config": {"workload": f"batched ensemble: {len(sets)} R3 realisations, N_k log-uniform [8192, 262144] "
                               f"(total {r['total_particles']}), 1 force + 10 KDK steps per step, one persistent "
                               "kernel under a CUDA graph", "pairs_per_step": r["pairs_per_step"],
                   "l2": "inputs re-uploaded before every step (outside the timed events)"},
        "plain_launches": r["plain_launches"],
        "per_phase_graph": r["per_phase_graph"],
        "speedup_graph_vs_plain": r["speedup_graph_vs_plain"],
        "speedup_vs_per_phase_graph": r["speedup_vs_per_phase_graph"],
        "roofline": {"bound": "fp32", "achieved": value / ws * 20 / 1e12, "peak": f32_peak / 1e12,
                     "unit": "TFLOP/s", "frac": r["frac"], "traffic": None,
                     "peak_kind": "FP32 FMA issue peak measured in this process", "flops_per_pair": 20},
        "accuracy_mixed_vs_fp64": r["accuracy"],
        "gpu_launches": r["launches"],
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "note": "device-resident ensemble; see config"},
        "clocks": clk,
    }


# The other workloads measured by the default run, with short samples.
CONFIGS = [
    ("cfg0", {"workload": "cfg0"}),
    ("cfg2_images", {"workload": "cfg2"}),
    ("cfg2_table_o0", {"workload": "cfg2", "s1_table": True, "order": 0, "n": 1 << 20}),
    ("cfg2_table_o2", {"workload": "cfg2", "s1_table": True, "order": 2, "n": 1 << 20}),
    ("cfg2_table_o4", {"workload": "cfg2", "s1_table": True, "order": 4, "n": 1 << 20}),
    ("cfg3_o2", {"workload": "cfg3", "order": 2}),
    ("cfg3_o4", {"workload": "cfg3", "order": 4}),
    ("cfg3_o2_ng127", {"workload": "cfg3", "order": 2, "t3_level": 3}),
]
REF_GPU = [
    ("r3", {"workload": "cfg1"}),
    ("t3", {"workload": "cfg3", "order": 4}),
    ("s1_images", {"workload": "cfg2"}),
    ("s1_table_o0", {"workload": "cfg2", "s1_table": True, "order": 0, "n": 1 << 20}),
    ("s1_table_o2", {"workload": "cfg2", "s1_table": True, "order": 2, "n": 1 << 20}),
    ("s1_table_o4", {"workload": "cfg2", "s1_table": True, "order": 4, "n": 1 << 20}),
]


def config_args(args, over):
    ns = argparse.Namespace(**vars(args))
    ns.n, ns.order, ns.s1_table, ns.t3_level = 0, 2, False, 0
    for k, v in over.items():
        setattr(ns, k, v)
    return ns


def run_configs(args, eng, peaks, local):
    """Every other workload, briefly: 1 warm-up + 3 timed evaluations (2 for the
    slow ones), the FP64 kernel on 2048 i, a ~2 s CPU baseline sample."""
    import steps_gb300 as S
    from steps_gb300 import workloads as W

    f32_peak, f64_peak = peaks
    threads = os.cpu_count() or 1
    out = {}
    clocks = ClockSampler(local)
    clocks.start()
    t_all = time.perf_counter()
    for name, over in CONFIGS:
        t0 = time.perf_counter()
        ca = config_args(args, over)
        ps, p, flops, desc, table = workload(ca)
        eng.set_variant(0)
        setup_engine_workload(eng, ps, table)
        slow = (ps.n * ps.n * flops) > 5e13
        r = measure(eng, S, ps, p, flops, table, 2 if slow else 3, 1, 2048, f32_peak, f64_peak)
        tab = host_table(table, eng)
        rate, dt, pairs, ni = cpu_baseline(ps, p, 0, threads, tab, seconds=2.0)
        out[name] = {"workload": desc, "value": r["value"], "unit": UNIT, "ms_per_step": float(np.mean(r["step_ms"])),
                     "steps": len(r["step_ms"]), "kernel_ms": r["kernel_ms"], "prep_ms": r["prep_ms"],
                     "kernel_pairs_per_s": r["kern_rate"], "kernel_shape": shape_desc(r["shape"], ca),
                     "autotune_s": r["autotune_s"],
                     "roofline": {"bound": "fp32", "frac": r["frac"], "achieved": r["achieved"],
                                  "peak": f32_peak / 1e12, "unit": "TFLOP/s", "flops_per_pair": flops},
                     "fp64": r["fp64"], "speedup_vs_fp64": r["speedup_vs_fp64"],
                     "accuracy_mixed_vs_fp64": r["accuracy"],
                     "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                                      "sample": f"{ni} i particles x all {ps.n} j ({dt:.1f} s)"},
                     "wall_s": time.perf_counter() - t0}
    t0 = time.perf_counter()
    eng.set_variant(0)
    out["cfg0_kdk"] = kdk_measure(eng, S, W, W.workload("cfg0"), 3, 1, f32_peak)
    out["cfg0_kdk"]["wall_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    sets = W.r3_ensemble(64)
    r = batch_measure(eng, S, sets, 2, 1, f32_peak)
    out["cfg4"] = {"workload": f"batched ensemble: 64 R3 realisations, N_k log-uniform [8192, 262144] "
                               f"(total {r['total_particles']}), 1 force + 10 KDK steps, one persistent kernel under a CUDA graph",
                   "value": r["value"], "unit": UNIT, "ms_per_step": r["ms_per_step"], "steps": r["steps"],
                   "roofline": {"bound": "fp32", "frac": r["frac"], "peak": f32_peak / 1e12, "flops_per_pair": 20},
                   "plain_launches": r["plain_launches"], "speedup_graph_vs_plain": r["speedup_graph_vs_plain"],
                   "per_phase_graph": r["per_phase_graph"],
                   "speedup_vs_per_phase_graph": r["speedup_vs_per_phase_graph"],
                   "accuracy_mixed_vs_fp64": r["accuracy"], "wall_s": time.perf_counter() - t0}
    eng.set_variant(0)
    clk = clocks.stop()
    out["_clocks"] = clk
    out["_wall_s"] = time.perf_counter() - t_all
    return out


def run_ref_gpu_block(args):
    out = {}
    t_all = time.perf_counter()
    for name, over in REF_GPU:
        ca = config_args(args, over)
        ps, p, flops, desc, table = workload(ca)
        r = ref_gpu_measure(ca, ps, p, flops, desc, table, 0.5, 2, 1)
        if r is None:
            return {"unavailable": "oracle/_ref/forces_cuda_*.cubin not built (needs the reference tree at build time)"}
        out[name] = r
    out["_wall_s"] = time.perf_counter() - t_all
    return out


def add_ratios(line):
    """Our kernel's pair rate over the reference CUDA builds' on the same
    workloads (kernel time against kernel time)."""
    cf, rg = line.get("configs") or {}, line.get("ref_gpu") or {}
    pairs = {"r3": None, "t3": "cfg3_o4", "s1_images": "cfg2_images", "s1_table_o0": "cfg2_table_o0",
             "s1_table_o2": "cfg2_table_o2", "s1_table_o4": "cfg2_table_o4"}
    for name, ours in pairs.items():
        r = rg.get(name)
        if not isinstance(r, dict) or "fp32_build" not in r:
            continue
        if ours is None:  # the headline workload
            mixed = line["config"]["pairs_per_step"] / (line["roofline"]["kernel_ms"] * 1e-3)
            f64 = line["fp64"]["pairs_per_s"]
        else:
            mixed = cf.get(ours, {}).get("kernel_pairs_per_s")
            f64 = cf.get(ours, {}).get("fp64", {}).get("pairs_per_s")
        if mixed:
            r["mixed_over_ref_fp32"] = mixed / r["fp32_build"]["pairs_per_s"]
        if f64:
            r["fp64_over_ref_fp64"] = f64 / r["fp64_build"]["pairs_per_s"]


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        if args.ref_device == "gpu":
            run_reference_gpu(args, ws, rank)
        else:
            run_reference(args, ws, rank)
        return
    dist = dist_init(ws)
    if args.workload == "cfg4":
        line = run_batch(args, ws, rank, local, dist)
        if rank == 0:
            print(json.dumps(line), flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return
    line, ps, p, tab, eng, peaks = run_ours(args, ws, rank, local, dist)
    if rank == 0:
        threads = os.cpu_count() or 1
        rate, dt, pairs, ni = cpu_baseline(ps, p, args.cpu_sample, threads, tab, seconds=args.cpu_seconds)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                                "build": "oracle port, -O3 -ffast-math (the reference's release flags)",
                                "sample": f"{ni} i particles x all {ps.n} j ({dt:.1f} s of CPU work)"}
        if ws == 1 and args.workload == "cfg1" and not args.no_configs and not args.n:
            line["configs"] = run_configs(args, eng, peaks, local)
            line["ref_gpu"] = run_ref_gpu_block(args)
            add_ratios(line)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
