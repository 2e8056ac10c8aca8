#!/usr/bin/env python3
"""Throughput of the GB300 grammar sweep: Y = M X over a RePair grammar.

Default workload: the 200,000 x 10,000 mosaic genotype matrix (256 founders,
switch rate 0.005, mutation 5e-4, seed 2), RePair-compressed by this
project's compressor, times X of 10,000 x 32 fp32 ~ U[-1,1] ((+,x) semiring).
A step is one multiply of all 32 right-hand sides.  Inputs are synthetic and
seeded; the grammar (about 1 GB of rules and emissions) is larger than the
129 MB L2, so no extra L2 flush is done between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gmr|reference]

--impl reference times the reference's CPU implementation of the path (the
OpenMP level sweep of gpu_engine_test.cu:49-104, as restated in oracle/) on the
host cores, on a bounded sample of the same workload.  Under torchrun each
rank runs an independent replica (the path does not shard across GPUs); the
value is the total over ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "g-mm-repair_gb300"))
sys.path.insert(0, str(REPO))

METRIC = "vectors/s & %HBM roofline, batched+learned vs plain sweep on GB300 (rel err≤1e-5)"
WORKLOADS = {
    # name: rows, cols, founders, switch, mutation, seed
    "mosaic-200000x10000": (200_000, 10_000, 256, 0.005, 5e-4, 2),
    "mosaic-20000x5000": (20_000, 5_000, 64, 0.01, 1e-3, 0),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def load_or_make_grammar(name: str, threads: int = 0):
    import gmr

    rows, cols, F, sw, mu, seed = WORKLOADS[name]
    cache = Path(os.environ.get("GMR_CACHE_DIR", REPO / "_cache"))
    cache.mkdir(parents=True, exist_ok=True)
    base = cache / f"{name}-s{seed}"
    if Path(str(base) + ".vc.R").exists():
        return gmr.Grammar.load(base), rows, cols, {"cached": True}
    t0 = time.perf_counter()
    m = gmr.gen_mosaic(rows, cols, F, sw, mu, seed, threads)
    nnz = m.nnz
    t1 = time.perf_counter()
    g = gmr.repair(m, threads)
    t2 = time.perf_counter()
    del m
    tmp = Path(str(base) + ".tmp")
    g.save(tmp)
    for ext in (".vc.R", ".vc.C", ".val"):
        os.replace(str(tmp) + ext, str(base) + ext)
    log(f"grammar {name}: nnz={nnz} gen {t1 - t0:.1f}s repair {t2 - t1:.1f}s")
    return g, rows, cols, {"cached": False, "nnz": int(nnz), "gen_s": round(t1 - t0, 2),
                           "repair_s": round(t2 - t1, 2)}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if not self.p:
            return None
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def cpu_reference_rate(g, rows, cols, seconds: float, threads: int, gpu_y0=None, x0=None):
    """The reference's OpenMP CPU sweep (oracle restatement), on the host cores."""
    from oracle import oracle as O

    t0 = time.perf_counter()
    sched = O.RefSchedule(g.alpha, g.rules(), g.C())
    build_s = time.perf_counter() - t0
    V = g.values().astype(np.float32)
    rng = np.random.default_rng(1)
    n, spent, err = 0, 0.0, None
    while n < 1 or (spent < seconds and n < 20):
        x = x0 if (n == 0 and x0 is not None) else rng.uniform(-1, 1, cols).astype(np.float32)
        t = time.perf_counter()
        sched.cpu_reference(0, V, x, rows, cols, threads=threads)
        spent += time.perf_counter() - t
        n += 1
    if gpu_y0 is not None and x0 is not None:
        y64 = sched.sweep_f64(0, V.astype(np.float64), x0, rows, cols)
        err = float(np.abs(gpu_y0.astype(np.float64) - y64).max() / max(np.abs(y64).max(), 1e-30))
    return n / spent, n, spent, build_s, err


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    g, rows, cols, _ = load_or_make_grammar(args.workload)
    threads = os.cpu_count() or 1
    per_step = []
    for _ in range(args.warmup + args.steps):
        rate, n, spent, build_s, _ = cpu_reference_rate(g, rows, cols, args.ref_seconds, threads)
        per_step.append(rate)
    vals = per_step[args.warmup:]
    v = statistics.median(vals)
    cfg = workload_config(args, rows, cols)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "vectors/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
        "cpu_baseline": {"value": v, "unit": "vectors/s", "cores": threads, "kind": "port",
                         "sample": f"each step: the reference's OpenMP layered CPU sweep (restated in oracle/) on "
                                   f"1-20 single vectors of the same grammar for ~{args.ref_seconds:.0f} s; "
                                   f"no batched CPU path exists, so vectors/s = 1/t"},
        "e2e": {"value": v, "unit": "vectors/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(args, rows, cols):
    r, c, F, sw, mu, seed = WORKLOADS[args.workload]
    return {"workload": f"{args.workload} mosaic genotype RePair grammar x X[{cols}x{args.B}] fp32 U[-1,1]",
            "rows": rows, "cols": cols, "founders": F, "switch_rate": sw, "mutation": mu, "seed": seed,
            "B": args.B, "semiring": "plustimes",
            "l2": "inputs larger than L2 (grammar streams > 129 MB each step); no flush"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gmr", "reference"], default="gmr")
    ap.add_argument("--workload", choices=list(WORKLOADS), default="mosaic-200000x10000")
    ap.add_argument("--B", type=int, default=32)
    ap.add_argument("--variant", type=int, default=0,
                    help="0 auto (autotuned per-launch table, CUDA graph), 1 plain, 2 fused, 3 graph")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (AUTO = engine defaults)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-seconds", type=float, default=6.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--dump-launches", action="store_true", help="per-launch times and level sizes to stderr")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch

    import gmr

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    gmr.lib()

    if ws > 1 and rank != 0:
        torch.distributed.barrier()
    g, rows, cols, ginfo = load_or_make_grammar(args.workload)
    if ws > 1 and rank == 0:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    plan = gmr.Plan.build(g, rows, cols)
    plan_s = time.perf_counter() - t0
    st = plan.stats
    eng = gmr.Engine(plan, device=local)
    B = args.B
    rng = np.random.default_rng(1 + rank)
    Xh = rng.uniform(-1, 1, (cols, B)).astype(np.float32)
    X = torch.from_numpy(Xh).to(dev)
    Y = torch.empty((rows, B), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    cfg = dict(variant=args.variant)

    def step():
        eng.multiply_device(0, X.data_ptr(), Y.data_ptr(), B, stream=sp, **cfg)

    def timed(n, **c):
        for _ in range(3):
            eng.multiply_device(0, X.data_ptr(), Y.data_ptr(), B, stream=sp, **c)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(n):
            eng.multiply_device(0, X.data_ptr(), Y.data_ptr(), B, stream=sp, **c)
        b.record(stream)
        torch.cuda.synchronize(dev)
        return a.elapsed_time(b) / n

    tuning = {}
    if args.variant == 0:
        default_ms = timed(20, variant=3)
        if not args.no_tune:
            t0 = time.perf_counter()
            eng.autotune(0, X.data_ptr(), Y.data_ptr(), B, stream=sp, reps=3)
            tuning = {"autotune_s": round(time.perf_counter() - t0, 2),
                      "table": [int(v) for v in eng.level_variants(0, B)]}
        tuning["default_vps"] = B * 1000.0 / default_ms

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    launches_per_step = eng.last_launches

    # ---- timed region: K steps, barrier + synchronize on both sides
    sampler = ClockSampler(local)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    sampler.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    if ws > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    if ws > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = ws * B * args.steps / (ms / 1000.0)

    # ---- per-launch times (same kernels, launched one by one) for the roofline
    reps = 5
    lt = np.mean([eng.time_launches(0, X.data_ptr(), Y.data_ptr(), B, stream=sp, variant=args.variant or 0)
                  for _ in range(reps)], axis=0)
    level_ms = float(lt[1:].sum())       # k_level launches: levels + final fold
    if args.dump_launches:
        ops, ems = plan.level_ops(), plan.level_emits()
        log("launch\tms\tops(level k)\temits(level k-1)")
        for i, t_ms in enumerate(lt):
            o = int(ops[i]) if 1 <= i < len(ops) else 0
            em = int(ems[i - 1]) if 1 <= i <= len(ems) else 0
            log(f"{i}\t{t_ms:.4f}\t{o}\t{em}")
    alg_total = plan.alg_bytes(0, B)
    alg_pro = 8.0 * (st["ref_alpha"] - 1) + 4.0 * st["n_vals"] + 4.0 * cols * B + 4.0 * rows * B
    alg_level = alg_total - alg_pro      # 12 N_L + 8 E + 8 E_T
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_level / (level_ms / 1000.0) / 1e9
    step_gbs = alg_total / (ms_per_step / 1000.0) / 1e9
    traffic_file = REPO / "profiles" / "traffic.json"
    traffic = None
    if traffic_file.exists():
        try:
            tj = json.loads(traffic_file.read_text())
            if tj.get("workload") == args.workload and tj.get("B") == B:
                traffic = tj.get("k_level_bytes_per_multiply")
        except Exception:
            traffic = None

    # ---- plain per-level sweep, one vector at a time (the reference's scheme)
    x1 = X[:, :1].contiguous()
    y1 = torch.empty((rows, 1), dtype=torch.float32, device=dev)
    for _ in range(3):
        eng.multiply_device(0, x1.data_ptr(), y1.data_ptr(), 1, stream=sp, variant=1)
    torch.cuda.synchronize(dev)
    kp = max(10, min(200, args.steps))
    e0.record(stream)
    for _ in range(kp):
        eng.multiply_device(0, x1.data_ptr(), y1.data_ptr(), 1, stream=sp, variant=1)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    plain_vps = kp / (e0.elapsed_time(e1) / 1000.0)

    # ---- end to end through the public API with host buffers (pinned)
    Xp = torch.from_numpy(Xh).pin_memory()
    Yp = torch.empty((rows, B), dtype=torch.float32).pin_memory()
    for _ in range(3):
        gmr.lib().gmr_engine_multiply_host(eng._h, 0, Xp.data_ptr(), Yp.data_ptr(), B, None)
    ke = max(10, min(100, args.steps))
    t = time.perf_counter()
    for _ in range(ke):
        rc = gmr.lib().gmr_engine_multiply_host(eng._h, 0, Xp.data_ptr(), Yp.data_ptr(), B, None)
        if rc:
            raise RuntimeError(gmr.lib().gmr_last_error().decode())
    e2e_s = (time.perf_counter() - t) / ke
    e2e_value = ws * B / e2e_s

    out = {
        "metric": METRIC, "value": value, "unit": "vectors/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded mosaic generator + RePair)",
        "config": workload_config(args, rows, cols) | {
            "variant": {0: "auto (autotuned per-launch table, CUDA graph)", 1: "plain", 2: "fused",
                        3: "graph"}[args.variant], "parallelism": f"replicas x{ws}"},
        "tuning": tuning,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": "k_level (all level launches of one multiply)",
                     "alg_bytes_per_multiply": alg_level, "kernel_ms_per_multiply": level_ms,
                     "step_alg_gbs": step_gbs},
        "e2e": {"value": e2e_value, "unit": "vectors/s", "h2d_bytes_per_step": int(cols * B * 4),
                "d2h_bytes_per_step": int(rows * B * 4)},
        "gpu_launches": int(launches_per_step * args.steps),
        "clocks": clocks,
        "plain_sweep_b1": {"value": plain_vps, "unit": "vectors/s", "speedup": value / ws / plain_vps},
        "grammar": {"ops": st["n_ops"], "depth": st["depth"], "layered_rules": st["ref_layered"],
                    "passthrough": st["ref_passthrough"], "emit": st["ref_emit"],
                    "term_emit": st["ref_term_emit"], "terminals": st["ref_alpha"], "plan_s": round(plan_s, 2)}
        | ginfo,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        y0 = Y[:, 0].float().cpu().numpy()
        threads = os.cpu_count() or 1
        rate, n, spent, build_s, err = cpu_reference_rate(g, rows, cols, args.cpu_seconds, threads,
                                                          gpu_y0=y0, x0=Xh[:, 0].copy())
        out["cpu_baseline"] = {"value": rate, "unit": "vectors/s", "cores": threads, "kind": "port",
                               "sample": f"{n} single vectors of the same grammar in {spent:.1f} s with the "
                                         f"reference's OpenMP level sweep (restated in oracle/)"}
        out["rel_err_fp64"] = err
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
