"""Benchmark of the GB300 MSM engine (BLS12-377 G1) -- one JSON line on rank 0.

Workload (the largest single-GPU plain configuration): one MSM of N = 2^24 seeded bases
k_i * G (resident in HBM in precomputed twisted-Edwards form) with uniform 253-bit scalars per
step.  Inputs are synthetic and seeded; scalar and base buffers (512 MB + 2.4 GB) exceed the
129 MB L2, so no flush is needed between steps.

  value  MSMs/s with the step's scalars already in device memory (msm_mult_device)
  e2e    MSMs/s through msm_mult with host scalars in pinned buffers: H2D of 32 B per point and
         D2H of the 144-byte result inside the timed region (`e2e_pageable`: the same from
         pageable buffers, the memory the reference's harness passes)
  extra  points/s, per-step p50/p99, the uneven batch (64 MSMs of 2^10..2^20 over a shared 2^20
         base set: one pass with a shared sort replayed from a CUDA graph vs one pass per MSM),
         the served mix (Poisson arrivals, sizes 2^12..2^22 over a 2^22 base set), the oracle
         port timed on the host cores, the same 2^24 MSM over the plain resident form (144 B
         per base, no tables: `plain_144B_per_base`) and the fixed-base large MSM (4 x 2^26
         over one resident base set, batch 0 checked against the oracle: `fixed_base_4x`), and the
         NTT track (one 2^24-point Goldilocks NTT, device and host to host, checked against the
         oracle: `ntt`).

`--impl reference` times the CPU port of the reference's oracle algorithm (arkworks-style
Pippenger, oracle/cpu_msm.c) on all host cores on the same workload; the reference itself
(OCaml RTL + XRT host, Rust/arkworks harness) cannot run on this machine.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

C_MUL = 588     # one Montgomery product: 12 x 12 limb products, lo and hi, plus the reduction
C_MADD = 4116   # 7 Montgomery products x 588 IMAD (12 x 32-bit limbs)
C_ADD = 5292    # 9 products


def accumulate_imad(stats):
    """IMAD (588 per product) that k_accumulate executes in one pass: every run (task) starts
    from its first base with one product, and each further entry is a 7-product mixed add.  The
    survey's convention credits one mixed add per sorted entry (entries x 4116), which counts
    6 products per run that the kernel does not do."""
    entries, tasks = int(stats["entries"]), int(stats["tasks"])
    return (entries - tasks) * C_MADD + tasks * C_MUL


def hbm_view(achieved_bytes_per_s):
    """Algorithmic HBM rate of k_accumulate (144 B base + 4 B entry per point and window) against
    the measured copy bandwidth in MEASURED_PEAKS.json, or the 6.8 TB/s fallback."""
    peak, src = 6800.0, "fallback 6.8 TB/s"
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak, src = float(json.load(f)["hbm_gbs"]), "of measured (MEASURED_PEAKS.json hbm_gbs)"
    except Exception:
        pass
    if not achieved_bytes_per_s:
        return None
    a = achieved_bytes_per_s / 1e9
    return {"achieved": a, "peak": peak, "unit": "GB/s", "frac": a / peak, "peak_source": src}


def imad_model(n: int, c: int) -> float:
    w = math.ceil(253 / c)
    return n * w * C_MADD + w * 2 ** (c - 1) * 2 * C_ADD + 253 * C_ADD + w * C_ADD


def algorithmic_imad(n: int) -> float:
    """A(N) = min over c in 10..16 of the IMAD count of a signed-window Pippenger."""
    return min(imad_model(n, c) for c in range(10, 17))


# ---------------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def percentile(v, p):
    s = sorted(v)
    k = min(len(s) - 1, max(0, int(math.ceil(p / 100.0 * len(s))) - 1))
    return s[k]


# ---------------------------------------------------------------------------------------------
def cpu_msm_time(points, scalars, threads):
    from oracle import cpu as ocpu
    t0 = time.perf_counter()
    out = ocpu.msm(points, scalars, threads=threads)
    return time.perf_counter() - t0, out


def workload_config(log2n):
    """The config both arms report for the plain workload (one MSM of 2^log2n points)."""
    n = 1 << log2n
    return {"workload": f"plain single MSM, BLS12-377 G1, N=2^{log2n}", "n": n,
            "l2": f"inputs larger than L2: {n * 32 / 2**20:.0f} MB of scalars and at least "
                  f"{n * 144 / 2**20:.0f} MB of resident base records per MSM; no L2 flush"}


def run_reference(args, rank, world):
    """Reference arm: the CPU port of the oracle algorithm on all host cores."""
    if rank != 0:
        return
    from oracle import cpu as ocpu  # this arm loads the oracle library and nothing of the engine
    n = 1 << args.log2n
    cores = os.cpu_count() or 1
    pts = ocpu.gen_bases(args.seed, n, threads=cores)
    sc = ocpu.gen_scalars(args.seed + 1, n, threads=cores)  # the engine's draws for this seed
    # warm-up steps page in the code and the inputs on a 2^16-point slice; every timed step is a
    # full MSM of the configured size (about 15 s at 2^24 on 16 Grace cores)
    nw = min(n, 1 << 16)
    for _ in range(args.warmup):
        cpu_msm_time(pts[:nw], sc[:nw], cores)
    times = [cpu_msm_time(pts, sc, cores)[0] for _ in range(args.steps)]
    t = sum(times)
    v = args.steps / t
    line = {
        "impl": "reference", "metric": "msm_per_s", "value": v, "unit": "MSM/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded k_i*G bases, uniform 253-bit scalars)",
        "config": workload_config(args.log2n),
        "cpu_baseline": {"value": v, "unit": "MSM/s", "cores": cores, "kind": "port",
                         "sample": f"one full MSM of 2^{args.log2n} points per timed step; "
                                   f"warm-up steps on the first {nw} points"},
        "e2e": {"value": v, "unit": "MSM/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "points_per_s": v * n,
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local):
    import hardcaml_zprize_gb300 as eng
    from hardcaml_zprize_gb300 import build
    build.build()
    import torch

    n = 1 << args.log2n
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    os.environ["MSM_DEVICE"] = str(local)
    info = eng.device_info()
    peaks = eng.measure_int_peaks()
    peak_imad = peaks["mad_lo"]  # the IMAD pipe's instruction peak (64 per clock per SM)

    # ---- data: seeded bases on the GPU, scalars on the host ----
    t0 = time.perf_counter()
    pts = eng.generate_bases(args.seed, n)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    ctx = eng.multi_scalar_mult_init(pts)
    t_init = time.perf_counter() - t0
    nsteps = args.steps + args.warmup
    host_sc = [eng.generate_scalars(args.seed + 1 + rank * 1000 + s, n) for s in range(min(nsteps, 2))]
    dev_sc = [torch.from_numpy(h.view(np.uint8).reshape(-1)).to(dev) for h in host_sc]
    # pinned host copies for the end-to-end leg, made here so that pinning settles before any timing
    pinned_t = [torch.empty(h.nbytes, dtype=torch.uint8, pin_memory=True) for h in host_sc]
    pinned = [t.numpy().view(np.uint64).reshape(-1, 4) for t in pinned_t]
    for p_, h in zip(pinned, host_sc):
        p_[:] = h
    torch.cuda.synchronize()

    sizes, offs = [n], [0]

    def step_device(i):
        return ctx.mult_device(sizes, offs, dev_sc[i % len(dev_sc)].data_ptr())

    # ---- value: resident inputs ----
    for i in range(args.warmup):
        step_device(i)
    lat = []
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            s0 = time.perf_counter()
            step_device(i)
            lat.append(time.perf_counter() - s0)
        torch.cuda.synchronize()
        t_dev = time.perf_counter() - t0
    barrier(world)
    t_dev = max_over_ranks(t_dev, world)
    clocks = clk.summary()

    # ---- per-stage timing (CUDA events on the pipeline stream), separate pass ----
    ctx.set_timing(True)
    stage_acc = {}
    reps = max(2, min(args.steps, 5))
    for i in range(reps):
        step_device(i)
        for k, v in ctx.last_timings().items():
            stage_acc[k] = stage_acc.get(k, 0.0) + v / reps
    stats = ctx.last_pass_stats()
    ctx.set_timing(False)
    cfg = ctx.config(n)
    ctx_info = ctx.info()

    # ---- e2e: host scalars through msm_mult, from pinned host buffers (the scalars the harness
    # passes are plain pageable memory; the same loop over those is `e2e_pageable`) ----
    def e2e_loop(bufs):
        for i in range(args.warmup + 2):
            eng.multi_scalar_mult(ctx, pts, bufs[i % len(bufs)])
        barrier(world)
        t0 = time.perf_counter()
        out = None
        for i in range(args.steps):
            out = eng.multi_scalar_mult(ctx, pts, bufs[i % len(bufs)])
        t = time.perf_counter() - t0
        barrier(world)
        return max_over_ranks(t, world), out

    t_e2e, last = e2e_loop(pinned)
    t_e2e_pageable, _ = e2e_loop(host_sc)

    value = world * args.steps / t_dev
    e2e = world * args.steps / t_e2e
    ms_per_step = 1e3 * t_dev / args.steps
    msm_s = t_dev / args.steps
    t_acc = stage_acc.get("accumulate", 0) * 1e-3
    entries = int(stats["entries"])  # mixed adds of one pass: its nonzero digits
    acc_imad = accumulate_imad(stats)
    achieved = acc_imad / t_acc if t_acc > 0 else None
    traffic = None
    tf = os.path.join(ROOT, "profiles", "k_accumulate_traffic.json")
    if os.path.exists(tf):
        try:
            tr = json.load(open(tf))
            traffic = tr["bytes_per_point_window"] * entries
        except Exception:
            traffic = None
    line = {
        "metric": "msm_per_s", "value": value, "unit": "MSM/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded k_i*G bases, uniform 253-bit scalars)",
        # both arms carry the same config; the layout this pass ran is beside it
        "config": workload_config(args.log2n),
        "layout": {"l2": f"inputs larger than L2 ({n * 32 / 2**20:.0f} MB scalars, "
                         f"{ctx_info['resident_bytes'] / 2**30:.1f} GB of resident base records: "
                         + (f"fixed-base tables of width {ctx_info['table_bits']} "
                            f"({ctx_info['table_windows']} records per base)"
                            + (f" and of width {ctx_info['table2_bits']} ({ctx_info['table2_windows']} "
                               f"records per base)" if ctx_info['table2_windows'] else "")
                            if ctx_info['table_bits'] else "144 B per base") + "); no L2 flush needed",
                   "resident_bytes": ctx_info["resident_bytes"],
                   "window_bits": cfg["window_bits"], "signed_digits": cfg["signed_digits"] == 1,
                   "seg_len": cfg["seg_len"], "red_len_log2": cfg["red_len_log2"],
                   "fixed_base_tables": cfg["fixed_base"] == 1},
        "e2e": {"value": e2e, "unit": "MSM/s", "h2d_bytes_per_step": n * 32,
                "d2h_bytes_per_step": 144, "host_buffers": "pinned"},
        "e2e_pageable": {"value": world * args.steps / t_e2e_pageable, "unit": "MSM/s",
                         "h2d_bytes_per_step": n * 32, "d2h_bytes_per_step": 144},
        "gpu_launches": int(stats["kernels"]) * args.steps,  # counted by the driver per pass
        "points_per_s": value * n,
        "latency_ms": {"p50": 1e3 * percentile(lat, 50), "p99": 1e3 * percentile(lat, 99)},
        "roofline": {
            "bound": "imad", "kernel": "k_accumulate",
            "achieved": achieved / 1e12 if achieved else None, "peak": peak_imad / 1e12,
            "unit": "TIMAD/s", "frac": (achieved / peak_imad) if achieved else None,
            "traffic": traffic,
            "algorithmic_imad_per_launch": acc_imad, "entries_per_launch": entries,
            "runs_per_launch": int(stats["tasks"]),
            "imad_convention_one_madd_per_entry": entries * C_MADD,
            "peak_source": "measured in this run: independent mad.lo chains on all SMs "
                           "(msm_measure_int_peaks); algorithmic count 588 IMAD per 12-limb "
                           "product, 7 products per mixed add after each run's first entry "
                           "(1 product)",
            "peak_mad_lo_hi_pairs": peaks["mad_lo_hi"] / 1e12, "peak_mad_hi": peaks["mad_hi"] / 1e12,
            "frac_vs_lo_hi_pairs": (achieved / peaks["mad_lo_hi"]) if achieved else None,
            # A(N) counts a windowed signed Pippenger (c in 10..16); the pass runs on fixed-base
            # tables and does less work than that, so this is an effective rate, not a roofline
            "effective_vs_windowed_A_N": {
                "achieved_tera": algorithmic_imad(n) / msm_s / 1e12,
                "frac_of_peak": algorithmic_imad(n) / msm_s / peak_imad,
                "A_N_imad": algorithmic_imad(n)},
            # the same kernel against the copy bandwidth: how far it is from being memory-bound
            "hbm": hbm_view(entries * 148 / t_acc if t_acc > 0 else None),
        },
        "stages_ms": stage_acc,
        # achieved HBM rates of the two input streams: k_accumulate reads a 144 B base (table
        # entry) and a 4 B sorted entry per point and window; k_count reads the 32 B scalars
        "streams_gbs": {
            "bases_in_accumulate": entries * 148 / t_acc / 1e9 if t_acc > 0 else None,
            "scalars_in_count": n * 32 / (stage_acc.get("count", 0) * 1e-3) / 1e9
            if stage_acc.get("count", 0) > 0 else None,
        },
        "pass_stats": stats,
        "clocks": clocks,
        "device": info,
        "setup_s": {"generate_bases": t_gen, "msm_init": t_init},
    }

    # ---- uneven batch: batched (one pass, shared sort, graph) vs plain (one pass per MSM) ----
    if not args.skip_batched and rank == 0:
        line["batched"] = bench_batched(args, eng, ctx, torch, dev)
    # ---- served mix ----
    if not args.skip_served and rank == 0:
        line["served"] = bench_served(args, eng, ctx, n)
    # ---- CPU baseline on the host cores, plus a bit-exact check of the GPU result ----
    out_cpu = None
    last_sc = host_sc[(args.steps - 1) % len(host_sc)]
    if not args.skip_cpu and rank == 0:
        cores = os.cpu_count() or 1
        t_cpu, out_cpu = cpu_msm_time(pts, last_sc, cores)
        line["cpu_baseline"] = {"value": 1.0 / t_cpu, "unit": "MSM/s", "cores": cores, "kind": "port",
                                "sample": f"one full MSM of 2^{args.log2n} points (oracle/cpu_msm.c, "
                                          f"arkworks-0.3-style Pippenger, OpenMP over windows)"}
        line["parity_vs_cpu"] = bool(np.array_equal(last[0], out_cpu))
        line["speedup_vs_cpu"] = {"value": value * t_cpu, "e2e": e2e * t_cpu}
    ctx.close()
    # ---- the same MSM on the plain resident form: 144 B per base, no tables ----
    if not args.skip_plain_form and rank == 0:
        line["plain_144B_per_base"] = bench_plain_form(args, eng, torch, dev, pts, dev_sc, last_sc,
                                                       out_cpu, peak_imad, local)
    del pts
    # ---- the NTT track: one 2^24-point Goldilocks NTT per step ----
    if not args.skip_ntt and rank == 0:
        line["ntt"] = bench_ntt(args, args.ntt_log2n, local, check=not args.skip_cpu)
    # ---- fixed-base large MSM: 4 x 2^26 over one resident base set ----
    if not args.skip_large and rank == 0:
        line["fixed_base_4x"] = fixed_base_large(args, eng, peaks, local, 26, check=not args.skip_cpu)
    if rank == 0:
        print(json.dumps(line), flush=True)


def bench_plain_form(args, eng, torch, dev, pts, dev_sc, last_sc, out_cpu, peak_imad, local):
    """One MSM per step over a context without fixed-base tables (MSM_FIXED_BASE=0): the
    resident form is one 144-byte precomputed record per base and the pass is a windowed signed
    Pippenger, as in the reference's one-record-per-point layout."""
    n = pts.shape[0]
    prev = os.environ.get("MSM_FIXED_BASE")
    os.environ["MSM_FIXED_BASE"] = "0"
    try:
        ctx = eng.multi_scalar_mult_init(pts)
    finally:
        if prev is None:
            os.environ.pop("MSM_FIXED_BASE", None)
        else:
            os.environ["MSM_FIXED_BASE"] = prev
    try:
        info = ctx.info()
        cfg = ctx.config(n)
        for i in range(args.warmup):
            ctx.mult_device([n], [0], dev_sc[i % len(dev_sc)].data_ptr())
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            t0 = time.perf_counter()
            for i in range(args.steps):
                ctx.mult_device([n], [0], dev_sc[i % len(dev_sc)].data_ptr())
            torch.cuda.synchronize()
            t = time.perf_counter() - t0
        ctx.set_timing(True)
        stages = {}
        reps = max(2, min(args.steps, 5))
        for i in range(reps):
            ctx.mult_device([n], [0], dev_sc[i % len(dev_sc)].data_ptr())
            for k, v in ctx.last_timings().items():
                stages[k] = stages.get(k, 0.0) + v / reps
        stats = ctx.last_pass_stats()
        ctx.set_timing(False)
        got = ctx.mult(last_sc)[0]
        t_acc = stages.get("accumulate", 0) * 1e-3
        acc_imad = accumulate_imad(stats)
        return {
            "workload": f"plain single MSM, N=2^{args.log2n}, windowed signed digits over 144 B records",
            "resident_bytes": info["resident_bytes"], "window_bits": cfg["window_bits"],
            "value": args.steps / t, "unit": "MSM/s", "ms_per_step": 1e3 * t / args.steps,
            "stages_ms": stages, "pass_stats": stats,
            "roofline": {"bound": "imad", "kernel": "k_accumulate",
                         "achieved": acc_imad / t_acc / 1e12 if t_acc else None,
                         "peak": peak_imad / 1e12, "unit": "TIMAD/s",
                         "frac": acc_imad / t_acc / peak_imad if t_acc else None,
                         "algorithmic_imad_per_launch": acc_imad},
            "windowed_A_N": {"achieved_tera": algorithmic_imad(n) / (t / args.steps) / 1e12,
                             "frac_of_peak": algorithmic_imad(n) / (t / args.steps) / peak_imad},
            "parity_vs_cpu": None if out_cpu is None else bool(np.array_equal(got, out_cpu)),
            "clocks": clk.summary(),
        }
    finally:
        ctx.close()


def add_mod_r(a: np.ndarray, b: np.ndarray, r: np.ndarray) -> np.ndarray:
    """(a + b) mod r for rows of 4 little-endian u64 limbs with a, b < r (vectorised)."""
    out = np.empty_like(a)
    carry = np.zeros(a.shape[0], dtype=np.uint64)
    for k in range(4):
        s = a[:, k] + b[:, k]
        c1 = s < a[:, k]
        s2 = s + carry
        c2 = s2 < s
        out[:, k] = s2
        carry = (c1 | c2).astype(np.uint64)
    ge = np.zeros(a.shape[0], dtype=bool)
    decided = np.zeros(a.shape[0], dtype=bool)
    for k in range(3, -1, -1):
        gt, lt = out[:, k] > r[k], out[:, k] < r[k]
        ge |= ~decided & gt
        decided |= gt | lt
    ge |= ~decided  # equal to r
    borrow = np.zeros(a.shape[0], dtype=np.uint64)
    for k in range(4):
        v = out[:, k]
        d = v - r[k] - borrow
        nb = ((v < r[k]) | ((v == r[k]) & (borrow == 1))).astype(np.uint64)
        out[:, k] = np.where(ge, d, v)
        borrow = np.where(ge, nb, 0).astype(np.uint64)
    return out


def fixed_base_large(args, eng, peaks, local, log2n, check=True):
    """Fixed-base large MSM: 2^log2n bases loaded once, then 4 independent seeded scalar vectors of
    2^log2n uniform scalars back to back (the shape of the reference's 4 x 2^26 benchmark,
    zprize/msm_pippenger/README.md:287-331).  Batch 0 is checked against the oracle on the host
    cores (about a minute at 2^26); the others by size-independent properties: the fixed-base
    result equals the windowed result (another bucket layout and window combine), and
    MSM(s0) + MSM(s1) equals MSM((s0 + s1) mod r)."""
    from oracle import bls12_377 as ref
    n = 1 << log2n
    t0 = time.perf_counter()
    pts = eng.generate_bases(args.seed, n)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    ctx = eng.multi_scalar_mult_init(pts)
    t_init = time.perf_counter() - t0
    batches = 4
    sc = np.concatenate([eng.generate_scalars(args.seed + 1 + b, n) for b in range(batches)])
    try:
        cfg = ctx.config(n)
        info = ctx.info()
        ctx.mult(sc[:n])  # warm-up
        with ClockSampler(local) as clk:
            t0 = time.perf_counter()
            out = ctx.mult(sc)  # 4 MSMs, one pass each; the next scalars go up during a pass
            t_all = time.perf_counter() - t0
        ctx.set_timing(True)
        ctx.mult(sc[:n])
        stages = ctx.last_timings()
        stats = ctx.last_pass_stats()
        ctx.set_timing(False)
        entries = int(stats["entries"])
        windowed = ctx.mult(sc[:n], fixed_base=2)[0]
        s2 = add_mod_r(sc[:n], sc[n:2 * n], np.array(ref.limbs64(ref.R_SCALAR, 4), dtype=np.uint64))
        out2 = ctx.mult(s2)[0]
    finally:
        ctx.close()
    lin = ref.add(ref.decode_projective(out[0].tobytes()), ref.decode_projective(out[1].tobytes())) == \
        ref.decode_projective(out2.tobytes())
    parity = {"fixed_base_equals_windowed": bool(np.array_equal(out[0], windowed)),
              "linearity": bool(lin)}
    if check:
        t0 = time.perf_counter()
        _, want = cpu_msm_time(pts, sc[:n], os.cpu_count() or 1)
        parity["batch0_vs_cpu"] = bool(np.array_equal(out[0], want))
        parity["cpu_s"] = time.perf_counter() - t0
    t_acc = stages.get("accumulate", 0) * 1e-3
    return {
        "workload": f"fixed-base large MSM, BLS12-377 G1, 2^{log2n} resident bases, "
                    f"{batches} scalar vectors back to back, host scalars (msm_mult)",
        "n": n, "batches": batches, "msm_per_s": batches / t_all,
        "per_batch_latency_ms": 1e3 * t_all / batches, "total_s": t_all,
        "window_bits": cfg["window_bits"], "resident_bytes": info["resident_bytes"],
        "h2d_bytes_per_batch": n * 32, "d2h_bytes_per_batch": 144,
        "stages_ms": stages, "pass_stats": stats,
        "hbm_gbs_base_and_scalar_streams": (entries * 148 + n * 32) / t_acc / 1e9 if t_acc else None,
        "imad": {"kernel": "k_accumulate",
                 "achieved_tera": accumulate_imad(stats) / t_acc / 1e12 if t_acc else None,
                 "peak_mad_lo_tera": peaks["mad_lo"] / 1e12,
                 "frac": (accumulate_imad(stats) / t_acc / peaks["mad_lo"]) if t_acc else None,
                 "entries_per_msm": entries, "runs_per_msm": int(stats["tasks"])},
        "parity": parity, "clocks": clk.summary(),
        "setup_s": {"generate_bases": t_gen, "msm_init_with_tables": t_init},
        "reference_fpga": {"total_s": 20.336, "msm_per_s": 4 / 20.336,
                           "source": "reference README: 4 x 2^26 in 20.336 s on AWS F1 (not run here)"},
    }


def bench_ntt(args, log_n, local, check=True):
    """The NTT track at the reference's contest size: one Goldilocks NTT of 2^log_n points per
    step (4-step, two shared-memory passes), on device buffers (`device`) and host to host through
    ntt_evaluate (`e2e`, input read over NVLink-C2C by a copy kernel, output copied back into a
    populated buffer).  The roofline is HBM: each pass reads and writes the vector once
    (2 x 8 B per point).  Inputs are the reference host test's kind (zprize/ntt/host/
    test_random.cpp): uniform values below p, seeded."""
    import torch
    from hardcaml_zprize_gb300 import ntt
    n = 1 << log_n
    rng = np.random.default_rng(args.seed + 13)
    hi = rng.integers(0, 2**32, n, dtype=np.uint64)
    x = ((hi << np.uint64(32)) | rng.integers(0, 2**32, n, dtype=np.uint64)) % np.uint64(ntt.GL_P)
    ctx = ntt.NttContext(log_n)
    try:
        d_in = torch.from_numpy(x.view(np.int64)).cuda()
        d_out = torch.empty_like(d_in)
        stream = torch.cuda.Stream()  # a stream of its own: handle 0 would mean the context's stream
        torch.cuda.synchronize()
        for _ in range(args.warmup):
            ctx.evaluate_device(d_out.data_ptr(), d_in.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        # CUDA events on the launching stream; enough transforms for about half a second, so
        # that the clock sampler (every 200 ms) sees the timed region
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(10):
            ctx.evaluate_device(d_out.data_ptr(), d_in.data_ptr(), stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        steps = min(max(args.steps, int(0.5e3 / max(e0.elapsed_time(e1) / 10, 1e-3)), 10), 20000)
        with ClockSampler(local) as clk:
            e0.record(stream)
            for _ in range(steps):
                ctx.evaluate_device(d_out.data_ptr(), d_in.data_ptr(), stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
            t_dev = e0.elapsed_time(e1) * 1e-3 / steps
        out = np.zeros(n, dtype=np.uint64)
        for _ in range(args.warmup):
            ctx.evaluate(x, out=out)
        stages = {}
        t0 = time.perf_counter()
        for _ in range(steps):
            ctx.evaluate(x, out=out)
            for k, v in ctx.last_timings().items():
                stages[k] = stages.get(k, 0.0) + v / steps
        t_e2e = (time.perf_counter() - t0) / steps
        same = bool(np.array_equal(out, d_out.cpu().numpy().view(np.uint64)))
        # throughput: vectors back to back, uploads and downloads overlapping the transforms
        batch = 8
        xs = np.repeat(x[None, :], batch, axis=0)
        outs = np.zeros_like(xs)
        ctx.evaluate_batch(xs, out=outs)
        # median of five calls: one call moves 2 GB through pageable host memory, and a stall of
        # the host (page reclaim) in one of them should not set the figure
        calls = []
        for _ in range(5):
            t0 = time.perf_counter()
            ctx.evaluate_batch(xs, out=outs)
            calls.append((time.perf_counter() - t0) / batch)
        t_batch = statistics.median(calls)
        same = same and bool(np.array_equal(outs[-1], out))
    finally:
        ctx.close()
    peak, src = 6800.0, "fallback 6.8 TB/s"
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak, src = float(json.load(f)["hbm_gbs"]), "of measured (MEASURED_PEAKS.json hbm_gbs)"
    except Exception:
        pass
    pass_ms = [stages.get("pass_a", 0), stages.get("pass_b", 0)]
    alg = 2 * n * 8  # one read and one write of the vector per pass
    res = {
        "workload": f"Goldilocks NTT, 2^{log_n} points, natural order in and out",
        "n": n, "device": {"value": 1.0 / t_dev, "unit": "NTT/s", "ms_per_ntt": 1e3 * t_dev, "steps": steps},
        "e2e": {"value": 1.0 / t_e2e, "unit": "NTT/s", "ms_per_ntt": 1e3 * t_e2e,
                "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8},
        "throughput_e2e": {"value": 1.0 / t_batch, "unit": "NTT/s", "ms_per_ntt": 1e3 * t_batch,
                           "batch": batch, "calls_ms_per_ntt": [1e3 * c for c in calls],
                           "note": "host to host, 8 vectors per call (ntt_evaluate_batch), median of 5 calls"},
        "stages_ms": stages,
        "roofline": {"bound": "hbm", "kernel": "k_ntt_pass", "unit": "GB/s", "peak": peak,
                     "peak_source": src, "algorithmic_bytes_per_launch": alg,
                     "achieved": [alg / (t * 1e-3) / 1e9 if t else None for t in pass_ms],
                     "frac": [alg / (t * 1e-3) / 1e9 / peak if t else None for t in pass_ms]},
        "device_equals_host_path": same,
        "clocks": clk.summary(),
        "reference_fpga": {"ntt_s": [0.0267, 0.0450], "e2e_s": [0.168, 0.177],
                           "source": "reference docs/zprize_ntt_top.mld: 64-core builds, optimized and "
                                     "normal layout; evaluate with host pre/post-processing (not run here)"},
    }
    if check:
        from oracle import cpu as ocpu
        cores = os.cpu_count() or 1
        t0 = time.perf_counter()
        want = ocpu.ntt(x, threads=cores)
        t_cpu = time.perf_counter() - t0
        res["parity_vs_cpu"] = bool(np.array_equal(out, want))
        res["cpu_baseline"] = {"value": 1.0 / t_cpu, "unit": "NTT/s", "cores": cores, "kind": "port",
                               "sample": f"one NTT of 2^{log_n} points (oracle/cpu_ntt.c: the reference's "
                                         f"radix-2 host model, stages parallel over OpenMP)"}
    return res


def run_ntt(args, rank, world, local):
    """`--workload ntt`: the NTT block alone, as its own line."""
    from hardcaml_zprize_gb300 import build
    build.build()
    os.environ["MSM_DEVICE"] = str(local)
    if rank != 0:
        return
    res = bench_ntt(args, args.ntt_log2n, local, check=not args.skip_cpu)
    line = {
        "metric": "ntt_per_s", "value": res["device"]["value"], "unit": "NTT/s", "n_gpus": world,
        "steps": res["device"]["steps"], "warmup": args.warmup, "ms_per_step": res["device"]["ms_per_ntt"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded uniform values below p)",
        "config": {"workload": res["workload"], "n": res["n"],
                   "l2": "input, pass-A output and output vectors (3 x 8 B per point, 384 MB at "
                         "2^24) exceed the L2; no flush"},
        "e2e": {k: res["e2e"][k] for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step")},
        "roofline": res["roofline"], "clocks": res["clocks"], "ntt": res,
    }
    if "cpu_baseline" in res:
        line["cpu_baseline"] = res["cpu_baseline"]
    print(json.dumps(line), flush=True)


def run_fixed_base_large(args, rank, world, local):
    """`--workload fixed_base_4x`: the fixed-base block alone, as its own line."""
    import hardcaml_zprize_gb300 as eng
    from hardcaml_zprize_gb300 import build
    build.build()
    os.environ["MSM_DEVICE"] = str(local)
    if rank != 0:
        return
    peaks = eng.measure_int_peaks()
    res = fixed_base_large(args, eng, peaks, local, args.log2n, check=not args.skip_cpu)
    line = {
        "metric": "msm_per_s", "value": res["msm_per_s"], "unit": "MSM/s", "n_gpus": world,
        "steps": res["batches"], "warmup": 1, "ms_per_step": res["per_batch_latency_ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded k_i*G bases, uniform 253-bit scalars)",
        "config": {"workload": res["workload"], "n": res["n"], "window_bits": res["window_bits"]},
        "e2e": {"value": res["msm_per_s"], "unit": "MSM/s", "h2d_bytes_per_step": res["n"] * 32,
                "d2h_bytes_per_step": 144},
        "clocks": res["clocks"], "fixed_base_4x": res,
    }
    print(json.dumps(line), flush=True)


def run_sharded(args, rank, world, local):
    """`--workload sharded`: one MSM of 2^log2n points split into contiguous base slices, one per
    rank (each rank keeps only its slice resident), one all-gather of the 144-byte partial points
    (NCCL under torchrun, nothing at one rank) and an engine MSM with scalars 1 that adds them.
    Total work is fixed as ranks are added (strong scaling)."""
    import hardcaml_zprize_gb300 as eng
    from hardcaml_zprize_gb300 import build, shard
    build.build()
    import torch
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    os.environ["MSM_DEVICE"] = str(local)
    n = 1 << args.log2n
    lo, hi = shard.partition(n, world)[rank]
    pts = eng.generate_bases(args.seed, hi - lo, first=lo)
    ctx = eng.multi_scalar_mult_init(pts)
    sc = eng.generate_scalars(args.seed + 1, n)
    d_sc = torch.from_numpy(sc[lo:hi].view(np.uint8).reshape(-1)).to(dev)
    torch.cuda.synchronize()

    def partial(a, b):
        return ctx.mult_device([b - a], [0], d_sc.data_ptr())[0]

    def step():
        if world == 1:
            return shard.combine_on_gpu([partial(lo, hi)])
        return shard.sharded_msm(n, rank, world, partial, shard.combine_on_gpu)

    for _ in range(args.warmup):
        out = step()
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            out = step()
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
    barrier(world)
    t = max_over_ranks(t, world)
    parity = None
    if rank == 0 and not args.skip_cpu:
        from oracle import cpu as ocpu
        parity = bool(np.array_equal(out, ocpu.msm(eng.generate_bases(args.seed, n), sc)))
    ctx.close()
    if rank == 0:
        print(json.dumps({
            "metric": "msm_per_s", "value": args.steps / t, "unit": "MSM/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded k_i*G bases, uniform 253-bit scalars)",
            "config": {"workload": f"one MSM of N=2^{args.log2n} sharded over {world} rank(s) by "
                                   f"base slices, one all-gather of partial points", "n": n,
                       "bases_per_rank": hi - lo},
            "e2e": {"value": args.steps / t, "unit": "MSM/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 144 * world},
            "parity_vs_cpu": parity, "clocks": clk.summary()}), flush=True)


def uneven_mix(seed: int, gen_scalars, m: int = 64, nbase: int = 1 << 20):
    """The uneven batch: m MSMs of sizes floor(2^U), U ~ U[10, 20], each over a slice of a shared
    base set of nbase bases, scalars of the mix (70% uniform 253-bit, 10% 16-bit, 10% 0 or r - 1,
    10% one repeated value per MSM).  Returns (sizes, offsets, concatenated scalars)."""
    rng = np.random.default_rng(seed + 7)
    sizes = [int(2 ** u) for u in rng.uniform(10, 20, m)]
    offs = [int(rng.integers(0, nbase - s + 1)) for s in sizes]
    sc = np.concatenate([gen_scalars(seed + 11, s, kind=1, msm_index=j) for j, s in enumerate(sizes)])
    return sizes, offs, sc


def served_mix(seed: int, gen_scalars, m: int, nbase: int = 1 << 22):
    """The served requests: m requests of sizes floor(2^U), U ~ U[12, 22], over slices of a
    base set of nbase bases, uniform 253-bit scalars.  Returns (rng, sizes, offsets, scalars)."""
    rng = np.random.default_rng(seed + 9)
    sizes = [int(2 ** u) for u in rng.uniform(12, 22, m)]
    offs = [int(rng.integers(0, nbase - s + 1)) for s in sizes]
    reqs = [gen_scalars(seed + 100 + j, s) for j, s in enumerate(sizes)]
    return rng, sizes, offs, reqs


def bench_batched(args, eng, ctx, torch, dev):
    nbase = 1 << 20
    m = 64
    sizes, offs, sc = uneven_mix(args.seed, eng.generate_scalars, m, nbase)
    dsc = torch.from_numpy(sc.view(np.uint8).reshape(-1)).to(dev)
    torch.cuda.synchronize()
    res = {}
    outs = {}
    for name, opts in (("plain", dict(mode=1)), ("batched", dict(mode=2, use_graph=1))):
        for _ in range(max(args.warmup, 2)):
            outs[name] = ctx.mult_device(sizes, offs, dsc.data_ptr(), **opts)
        reps = max(3, min(args.steps, 10))
        t0 = time.perf_counter()
        for _ in range(reps):
            outs[name] = ctx.mult_device(sizes, offs, dsc.data_ptr(), **opts)
        t = (time.perf_counter() - t0) / reps
        res[name] = {"msm_per_s": m / t, "points_per_s": sum(sizes) / t, "ms_per_batch": 1e3 * t}
        # e2e with host scalars
        t0 = time.perf_counter()
        for _ in range(reps):
            ctx.mult_uneven(sizes, offs, sc, **opts)
        te = (time.perf_counter() - t0) / reps
        res[name]["e2e_msm_per_s"] = m / te
    # the autotuner on this mix (untimed), then the tuned one-pass form
    if args.tune_budget_ms > 0:
        tr = ctx.tune_uneven(sizes, offs, sc, budget_ms=args.tune_budget_ms)
        topts = {k: v for k, v in tr["opts"].items() if k != "mode"}
        for _ in range(max(args.warmup, 2)):
            outs["batched_tuned"] = ctx.mult_device(sizes, offs, dsc.data_ptr(), mode=2, use_graph=1, **topts)
        reps = max(3, min(args.steps, 10))
        t0 = time.perf_counter()
        for _ in range(reps):
            outs["batched_tuned"] = ctx.mult_device(sizes, offs, dsc.data_ptr(), mode=2, use_graph=1, **topts)
        t = (time.perf_counter() - t0) / reps
        res["batched_tuned"] = {"msm_per_s": m / t, "points_per_s": sum(sizes) / t, "ms_per_batch": 1e3 * t,
                                "tuner": {"untuned_pass_ms": tr["untuned_ms"], "tuned_pass_ms": tr["tuned_ms"],
                                          "passes_measured": tr["passes_measured"], "pass_options": topts,
                                          "forms_by_log2_size": {str(k): v for k, v in tr["forms"].items()}},
                                "identical_results": bool(np.array_equal(outs["batched_tuned"], outs["plain"]))}
        res["ratio_batched_tuned_over_plain"] = res["batched_tuned"]["msm_per_s"] / res["plain"]["msm_per_s"]
    # the same 64 MSMs as served requests arriving back to back (continuous batching)
    srv = eng.MsmServer(ctx, hbm_budget_bytes=args.served_budget_gb << 30, max_inflight=2)
    first = np.concatenate([[0], np.cumsum(sizes)])
    reps = max(3, min(args.steps, 10))
    for _ in range(args.warmup):  # untimed: the server's slots allocate their workspaces
        for rid in [srv.submit(sc[first[j]:first[j + 1]], offs[j]) for j in range(m)]:
            srv.poll(rid, wait_ms=600000)
    p_before = srv.stats()["passes"]
    t0 = time.perf_counter()
    exact = True
    for _ in range(reps):
        ids = [srv.submit(sc[first[j]:first[j + 1]], offs[j]) for j in range(m)]
        for j, rid in enumerate(ids):
            o, _lat = srv.poll(rid, wait_ms=600000)
            exact &= bool(np.array_equal(o, outs["plain"][j]))
    t = (time.perf_counter() - t0) / reps
    st = srv.stats()
    srv.close()
    res["served"] = {"msm_per_s": m / t, "passes_per_mix": (st["passes"] - p_before) / reps,
                     "same_as_alone": exact}
    res["ratio_batched_over_plain"] = res["batched"]["msm_per_s"] / res["plain"]["msm_per_s"]
    res["ratio_served_over_plain"] = res["served"]["msm_per_s"] / res["plain"]["e2e_msm_per_s"]
    res["e2e_ratio"] = res["batched"]["e2e_msm_per_s"] / res["plain"]["e2e_msm_per_s"]
    res["identical_results"] = bool(np.array_equal(outs["plain"], outs["batched"]))
    res["config"] = {"msms": m, "sizes": "log-uniform 2^10..2^20", "base_set": nbase,
                     "scalars": "70% uniform, 10% 16-bit, 10% 0 or r-1, 10% repeated value"}
    return res


def bench_served(args, eng, ctx, n):
    nbase = min(n, 1 << 22)
    m = args.served_requests
    rng, sizes, offs, reqs = served_mix(args.seed, eng.generate_scalars, m, nbase)
    # plain: one request at a time, after an untimed pass of the largest request (the workspace
    # then holds every size), best of two rounds; the served loads below are multiples of it
    big = max(range(m), key=lambda j: sizes[j])
    ctx.mult_uneven([sizes[big]], [offs[big]], reqs[big])
    t_plain = None
    for _ in range(2):
        t0 = time.perf_counter()
        plain_out = [ctx.mult_uneven([s], [o], r)[0] for s, o, r in zip(sizes, offs, reqs)]
        t = time.perf_counter() - t0
        t_plain = t if t_plain is None else min(t_plain, t)
    plain_rate = m / t_plain
    out = {"plain_msm_per_s": plain_rate, "requests": m, "sizes": "log-uniform 2^12..2^22",
           "base_set": nbase, "rates": []}
    for mult, inflight in [(a, b) for a in args.served_load for b in args.served_inflight]:
        lam = plain_rate * mult
        gaps = rng.exponential(1.0 / lam, m)
        srv = eng.MsmServer(ctx, hbm_budget_bytes=args.served_budget_gb << 30, max_inflight=inflight)
        # untimed warm-up: the largest requests, so every slot holds its workspace
        big = sorted(range(m), key=lambda j: -sizes[j])[:inflight]
        for rid in [srv.submit(reqs[j], offs[j]) for j in big]:
            srv.poll(rid, wait_ms=600000)
        p_before = srv.stats()["passes"]
        ids = []
        t0 = time.perf_counter()
        t_next = t0
        for j in range(m):
            t_next += gaps[j]
            d = t_next - time.perf_counter()
            if d > 0:
                time.sleep(d)
            ids.append(srv.submit(reqs[j], offs[j]))
        lats, exact = [], True
        for j, rid in enumerate(ids):
            o, l = srv.poll(rid, wait_ms=600000)
            lats.append(l)
            exact &= bool(np.array_equal(o, plain_out[j]))
        t = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        out["rates"].append({"offered_per_s": lam, "load_vs_plain": mult, "max_inflight": inflight,
                             "msm_per_s": m / t, "p50_ms": percentile(lats, 50),
                             "p99_ms": percentile(lats, 99), "passes": st["passes"] - p_before,
                             "inflight_peak": st["inflight_peak"], "same_as_alone": exact})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--log2n", type=int, default=24)
    ap.add_argument("--seed", type=int, default=20240601)
    ap.add_argument("--skip-batched", action="store_true")
    ap.add_argument("--skip-served", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-plain-form", action="store_true",
                    help="skip the 144 B-per-base (no tables) form of the headline MSM")
    ap.add_argument("--skip-large", action="store_true", help="skip the 4 x 2^26 fixed-base block")
    ap.add_argument("--skip-ntt", action="store_true", help="skip the NTT block")
    ap.add_argument("--ntt-log2n", type=int, default=24)
    ap.add_argument("--tune-budget-ms", type=int, default=15000,
                    help="time the batch autotuner may spend on the uneven mix (0: skip it)")
    ap.add_argument("--served-requests", type=int, default=48)
    ap.add_argument("--served-load", type=float, nargs="*", default=[0.5, 1.0, 1.5])
    ap.add_argument("--served-budget-gb", type=int, default=16)
    ap.add_argument("--served-inflight", type=int, nargs="*", default=[2, 4],
                    help="server slots (passes in flight) to sweep at each offered load")
    ap.add_argument("--workload", default="plain", choices=["plain", "fixed_base_4x", "sharded", "ntt"],
                    help="plain: the default single-MSM line; fixed_base_4x: 4 MSMs over one "
                         "resident base set (use with --log2n 26); sharded: one MSM split over "
                         "the ranks by base slices")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)  # timed numbers always follow at least 3 warm-up steps
    rank, world, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "fixed_base_4x":
        run_fixed_base_large(args, rank, world, local)
    elif args.workload == "sharded":
        run_sharded(args, rank, world, local)
    elif args.workload == "ntt":
        run_ntt(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
