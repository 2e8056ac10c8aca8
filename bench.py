#!/usr/bin/env python3
"""Throughput of the GB300 grammar sweep: Y = M X over a RePair grammar.

Default workload: the 200,000 x 10,000 mosaic genotype matrix (256 founders,
switch rate 0.005, mutation 5e-4, seed 2), RePair-compressed by this
project's compressor, times X of 10,000 x 32 fp32 ~ U[-1,1] ((+,x) semiring).
A step is one multiply of all 32 right-hand sides.  Inputs are synthetic and
seeded; the grammar (about 1 GB of rules and emissions) is larger than the
129 MB L2, so no extra L2 flush is done between steps.  The headline uses the
learned per-launch kernel choice (the committed cost model) and reports the
exhaustive autotuner's choice and the untuned engine beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gmr|reference]
                    [--workload NAME] [--semiring S] [--B B]

Other workloads (not the headline): mosaic-20000x5000 (the CPU-runnable size),
graph-16777216 (copy-model graph, 16.8M nodes, degree 24; --semiring boolean
with B = 32 bit-packed frontiers, or tropical) and pack8 (eight uneven mosaic
grammars, each with its own B, in one graph launch).

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
MOSAICS = {
    # name: rows, cols, founders, switch, mutation, seed
    "mosaic-200000x10000": (200_000, 10_000, 256, 0.005, 5e-4, 2),
    "mosaic-20000x5000": (20_000, 5_000, 64, 0.01, 1e-3, 0),
}
GRAPH = (16_777_216, 24, 0.7, 3)  # nodes, mean out-degree, copy probability, seed
# bytes each lane moves per value access: the engine's default, or GMR_LANE_BYTES
LANE_BYTES = os.environ.get("GMR_LANE_BYTES", "default: 32 for (+,x) tiles of >= 32 words, else 16")
WORKLOADS = list(MOSAICS) + ["graph-16777216", "pack8"]
SR_IDS = {"plustimes": 0, "boolean": 1, "tropical": 2}
INT_MAX = 2**31 - 1


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def slowest_rank_ms(ms: float, ws: int, device=None) -> float:
    """Length of the timed region on the slowest rank (every rank gets it):
    a max all-reduce over the process group (NCCL on the GPUs, gloo on CPU)."""
    if ws <= 1:
        return ms
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_vps(ws: int, B: int, steps: int, ms: float) -> float:
    """Vectors per second of the whole job: every rank multiplies its own B
    right-hand sides per step (replicas, weak scaling)."""
    return ws * B * steps / (ms / 1000.0)


def cache_dir() -> Path:
    d = Path(os.environ.get("GMR_CACHE_DIR", REPO / "_cache"))
    d.mkdir(parents=True, exist_ok=True)
    return d


def cached_grammar(key: str, make):
    """Grammar from the cache directory, or make() -> (grammar, info) and store it."""
    import gmr

    base = cache_dir() / key
    if Path(str(base) + ".vc.R").exists():
        return gmr.Grammar.load(base), {"cached": True}
    g, info = make()
    tmp = Path(str(base) + ".tmp")
    g.save(tmp)
    for ext in (".vc.R", ".vc.C", ".val"):
        os.replace(str(tmp) + ext, str(base) + ext)
    return g, info | {"cached": False}


REPAIR_ON_GPU = True  # the reference arm builds its grammar with the host compressor


def repair_device():
    """GPU of this rank for the RePair compressor (identical grammar to the
    host compressor), or None for the host compressor."""
    if not REPAIR_ON_GPU:
        return None
    try:
        import torch
        if torch.cuda.is_available():
            return int(os.environ.get("LOCAL_RANK", "0"))
    except ImportError:
        pass
    return None


def mosaic_grammar(rows, cols, F, sw, mu, seed):
    import gmr

    def make():
        t0 = time.perf_counter()
        m = gmr.gen_mosaic(rows, cols, F, sw, mu, seed)
        t1 = time.perf_counter()
        g = gmr.repair(m, device=repair_device())
        t2 = time.perf_counter()
        log(f"grammar mosaic {rows}x{cols}: nnz={m.nnz} gen {t1 - t0:.1f}s repair {t2 - t1:.1f}s")
        return g, {"nnz": int(m.nnz), "gen_s": round(t1 - t0, 2), "repair_s": round(t2 - t1, 2),
                   "repair_on": "gpu" if repair_device() is not None else "host"}

    return cached_grammar(f"mosaic-{rows}x{cols}-f{F}-s{seed}", make)


def graph_grammar(weighted: bool):
    import gmr

    nodes, deg, cp, seed = GRAPH

    def make():
        t0 = time.perf_counter()
        m = gmr.gen_copy_graph(nodes, deg, cp, weighted, seed)
        t1 = time.perf_counter()
        g = gmr.repair(m, device=repair_device())
        t2 = time.perf_counter()
        log(f"grammar graph {nodes}: nnz={m.nnz} gen {t1 - t0:.1f}s repair {t2 - t1:.1f}s")
        return g, {"nnz": int(m.nnz), "gen_s": round(t1 - t0, 2), "repair_s": round(t2 - t1, 2),
                   "repair_on": "gpu" if repair_device() is not None else "host"}

    return cached_grammar(f"graph-{nodes}-d{deg}-w{int(weighted)}-s{seed}", make)


def workload_grammar(args):
    if args.workload in MOSAICS:
        rows, cols, F, sw, mu, seed = MOSAICS[args.workload]
        g, info = mosaic_grammar(rows, cols, F, sw, mu, seed)
        return g, rows, cols, info
    g, info = graph_grammar(args.semiring == "tropical")
    return g, GRAPH[0], GRAPH[0], info


def make_inputs(sr: int, cols: int, B: int, seed: int):
    """Host inputs in the engine's element type: fp32 U[-1,1]; bit-packed 1 %-dense
    frontiers; int32 with 99 % INT_MAX (+inf) and 1 % U{0..1000}."""
    rng = np.random.default_rng(seed)
    if sr == 0:
        return rng.uniform(-1, 1, (cols, B)).astype(np.float32)
    if sr == 1:
        W = (B + 31) // 32
        bits = rng.random((cols, W * 32)) < 0.01
        bits[:, B:] = False
        words = (bits.reshape(cols, W, 32).astype(np.uint64) << np.arange(32, dtype=np.uint64)).sum(axis=2)
        return words.astype(np.uint32)
    X = np.full((cols, B), INT_MAX, dtype=np.int32)
    hot = rng.random((cols, B)) < 0.01
    X[hot] = rng.integers(0, 1001, int(hot.sum()))
    return X


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


class NvmlEnergy:
    """Total-energy counter of one GPU through NVML (libnvidia-ml, ctypes); the
    reference measures mJ per vector the same way (gpu_engine.cu NVML replay)."""

    def __init__(self, index: int):
        import ctypes
        self.h = None
        try:
            self.lib = ctypes.CDLL("libnvidia-ml.so.1")
            if self.lib.nvmlInit_v2() != 0:
                return
            h = ctypes.c_void_p()
            if self.lib.nvmlDeviceGetHandleByIndex_v2(index, ctypes.byref(h)) != 0:
                return
            self.h = h
        except OSError:
            self.h = None

    def mj(self):
        import ctypes
        if self.h is None:
            return None
        e = ctypes.c_ulonglong()
        if self.lib.nvmlDeviceGetTotalEnergyConsumption(self.h, ctypes.byref(e)) != 0:
            return None
        return float(e.value)


def measured_peak_hbm():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def oracle_x(sr: int, Xh: np.ndarray, col: int) -> np.ndarray:
    """Column `col` of the inputs as the reference's float x."""
    if sr == 0:
        return Xh[:, col].astype(np.float32)
    if sr == 1:
        return ((Xh[:, col // 32] >> np.uint32(col % 32)) & 1).astype(np.float32)
    x = Xh[:, col].astype(np.float64)
    x[x >= 1e9] = 1e9
    return x.astype(np.float32)


def cpu_reference_rate(g, sr, rows, cols, seconds: float, threads: int, sched=None):
    """The reference's OpenMP CPU sweep (oracle restatement), timed on the host
    cores over single vectors for about `seconds`."""
    from oracle import oracle as O

    t0 = time.perf_counter()
    if sched is None:
        sched = O.RefSchedule(g.alpha, g.rules(), g.C())
    build_s = time.perf_counter() - t0
    V = g.values().astype(np.float32)
    rng = np.random.default_rng(1)
    n, spent = 0, 0.0
    while n < 1 or (spent < seconds and n < 20):
        if sr == 0:
            x = rng.uniform(-1, 1, cols).astype(np.float32)
        else:
            x = oracle_x(sr, make_inputs(sr, cols, 1 if sr == 2 else 32, 1 + n), 0)
        t = time.perf_counter()
        sched.cpu_reference(sr, V, x, rows, cols, threads=threads)
        spent += time.perf_counter() - t
        n += 1
    return n / spent, n, spent, build_s


def column_words(sr, Yh: np.ndarray, b: int) -> np.ndarray:
    """Right-hand side b of an engine output [rows][words] as int64 / float64."""
    if sr == 0:
        return Yh.view(np.float32)[:, b].astype(np.float64)
    if sr == 1:
        return ((Yh.view(np.uint32)[:, b // 32] >> np.uint32(b % 32)) & 1).astype(np.int64)
    return Yh.view(np.int32)[:, b].astype(np.int64)


def check_all_columns(sched, V, sr, Xh, Yh, rows, cols, B, threads):
    """Every right-hand side of a timed multiply against the oracle, on the
    host cores (one column per thread; the oracle's C calls release the GIL):
    (+,x) as relative max-norm against the FP64 sweep (cpu_selftest.cpp:67-102),
    (OR,AND) and (min,+) bit for bit against the reference's int sweep
    (gpu_engine_test.cu:49-104).  Runs outside the timed region."""
    from concurrent.futures import ThreadPoolExecutor

    V32 = np.asarray(V, dtype=np.float32)
    V64 = V32.astype(np.float64)

    def one(b):
        x = oracle_x(sr, Xh, b)
        got = column_words(sr, Yh, b)
        if sr == 0:
            ref = sched.sweep_f64(0, V64, x, rows, cols)
            return float(np.abs(got - ref).max(initial=0.0) / max(np.abs(ref).max(initial=0.0), 1e-30)), 0
        ref = sched.cpu_reference(sr, V32, x, rows, cols, threads=1).astype(np.int64)
        return 0.0, int(np.sum(got != ref))

    t = time.perf_counter()
    with ThreadPoolExecutor(max(1, min(threads, B))) as ex:
        res = list(ex.map(one, range(B)))
    out = {"columns": B, "seconds": round(time.perf_counter() - t, 1), "threads": max(1, min(threads, B))}
    if sr == 0:
        errs = [r[0] for r in res]
        out |= {"rel_err_fp64_max": max(errs), "worst_column": int(np.argmax(errs)), "tolerance": 1e-5,
                "ok": bool(max(errs) <= 1e-5)}
    else:
        mism = [r[1] for r in res]
        out |= {"mismatches": int(sum(mism)), "worst_column": int(np.argmax(mism)), "ok": sum(mism) == 0,
                "against": "the reference's int sweep (oracle restatement), bit for bit"}
    return out


def source_hash(table: str = "") -> str:
    """Hash of the sources that make the sweep kernels: a traffic figure is
    only reported for the build it was measured on."""
    import hashlib

    h = hashlib.sha256()
    files = ["g-mm-repair_gb300/csrc/engine.cu", "g-mm-repair_gb300/csrc/device_util.cuh",
             "g-mm-repair_gb300/csrc/async_copy.cuh", "g-mm-repair_gb300/csrc/gmr_internal.h", "include/gmr.h"]
    if table == "learned":  # the table the cost models pick
        files.append("g-mm-repair_gb300/gmr/models/cost_model.gmrmlp")
        if (REPO / "g-mm-repair_gb300/gmr/models/mode_model.gmrmlp").exists():
            files.append("g-mm-repair_gb300/gmr/models/mode_model.gmrmlp")
    for f in files:
        h.update((REPO / f).read_bytes())
    return h.hexdigest()[:16]


def traffic_entry(key: str):
    """DRAM bytes per multiply from profiles/traffic.json, or (None, why)."""
    tf = REPO / "profiles" / "traffic.json"
    if not tf.exists():
        return None, "no traffic capture committed"
    try:
        ent = json.loads(tf.read_text()).get(key)
    except Exception as e:  # noqa: BLE001
        return None, f"unreadable traffic file: {e}"
    if not isinstance(ent, dict):
        return None, f"no capture for {key}"
    table = key.rsplit("/", 1)[-1]
    if ent.get("source_hash") != source_hash(table):
        return None, (f"capture {ent.get('source_hash')} is of other kernel sources than this build "
                      f"({source_hash(table)})")
    return ent, None


def reference_gpu_rate(g, sr, rows, cols, Xh, B, device, seconds=1.5):
    """The reference's own GPU engine on this GPU: its kernels
    (gpu-engine/gpu_engine.cu, compiled to PTX in oracle/_ref) with its host
    sequence (restated in oracle/ref/ref_gpu.cpp), single-vector and batched
    at this B, on the same grammar; returns rates and its first column."""
    from oracle import oracle as O

    why = O.RefGpu.available()
    if why:
        return {"unavailable": why}, None
    ref = O.RefGpu(device)
    sched = O.RefSchedule(g.alpha, g.rules(), g.C())
    V = g.values().astype(np.float32)
    if sr == 1:  # the reference's Boolean engine takes one 0/1 float per vector
        Xf = ((Xh[:, :, None] >> np.arange(32, dtype=np.uint32)) & 1).reshape(cols, -1)[:, :B].astype(np.float32)
    elif sr == 2:
        Xf = np.minimum(Xh.astype(np.float64), 1e9).astype(np.float32)
    else:
        Xf = Xh.astype(np.float32)
    out = {"how": "the reference's kernels (gpu_engine.cu eval_level_layered / emit_level and the batched ones) "
                  "in its host sequence, device memory, ms from CUDA events around the iterations"}
    y0 = None
    for b, X in ((1, Xf[:, :1]), (B, Xf)):
        Y, ms = ref.run(sched, sr, V, X, rows, cols, iters=1)
        iters = max(2, min(200, int(seconds * 1000.0 / max(ms, 1e-3))))
        Y, ms = ref.run(sched, sr, V, X, rows, cols, iters=iters)
        out[f"B{b}"] = {"vps": b * 1000.0 / ms, "ms_per_multiply": ms, "iters": iters}
        if b == B:
            y0 = Y[:, 0]
    return out, y0


def dtype_of(sr):
    return {0: "f32", 1: "u32 (32 bit-packed OR-AND vectors)", 2: "i32"}[sr]


def workload_config(args, rows, cols):
    cfg = {"workload": args.workload, "semiring": args.semiring, "B": args.B, "rows": rows, "cols": cols,
           "l2": "inputs larger than L2 (grammar streams > 129 MB each step); no flush"}
    if args.workload in MOSAICS:
        r, c, F, sw, mu, seed = MOSAICS[args.workload]
        cfg |= {"kind": "mosaic genotype RePair grammar", "founders": F, "switch_rate": sw, "mutation": mu,
                "seed": seed, "x": "fp32 U[-1,1]" if args.semiring == "plustimes" else args.semiring}
    elif args.workload == "graph-16777216":
        cfg |= {"kind": "copy-model graph RePair grammar", "degree": GRAPH[1], "copy_prob": GRAPH[2],
                "seed": GRAPH[3]}
    return cfg


VARIANT_NAMES = {0: "auto (learned per-launch table, CUDA graph)", 1: "plain", 2: "fused", 3: "graph",
                 4: "persistent"}


def run_config(args, rows, cols, ws):
    """The line's config: the same keys on both arms."""
    return workload_config(args, rows, cols) | {"variant": VARIANT_NAMES[args.variant],
                                                "lane_bytes": LANE_BYTES,
                                                "parallelism": f"replicas x{ws}"}


def run_reference(args):
    """The reference's CPU implementation of the path on the host cores: one
    step = one vector through the OpenMP layered sweep (gpu_engine_test.cu:49-104,
    restated in oracle/); the schedule is built once, outside the timed steps."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    if args.workload == "pack8":
        print(json.dumps({"impl": "reference", "unavailable": "pack8 has no single-grammar CPU path"}))
        return 0
    from oracle import oracle as O

    g, rows, cols, _ = workload_grammar(args)
    threads = os.cpu_count() or 1
    sr = SR_IDS[args.semiring]
    sched = O.RefSchedule(g.alpha, g.rules(), g.C())
    V = g.values().astype(np.float32)
    Xh = make_inputs(sr, cols, max(args.steps + args.warmup, 1) if sr != 1 else 32, 1)
    times = []
    for i in range(args.warmup + args.steps):
        x = oracle_x(sr, Xh, i % Xh.shape[1] if sr != 1 else i % 32)
        t = time.perf_counter()
        sched.cpu_reference(sr, V, x, rows, cols, threads=threads)
        times.append(time.perf_counter() - t)
    timed = times[args.warmup:]
    v = len(timed) / sum(timed)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "vectors/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * sum(timed) / len(timed),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype_of(sr),
        "data": "synthetic", "config": run_config(args, rows, cols, ws),
        "cpu_baseline": {"value": v, "unit": "vectors/s", "cores": threads, "kind": "port",
                         "sample": f"{len(timed)} single vectors of the same grammar, one per step, through the "
                                   f"reference's OpenMP layered CPU sweep (restated in oracle/), {threads} threads; "
                                   f"no batched CPU path exists, so vectors/s = steps / time"},
        "e2e": {"value": v, "unit": "vectors/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not args.no_reference_gpu:
        # beside the CPU arm: the reference's own GPU engine on this machine's GPU
        # (not the line's value), single-vector and batched at this B
        B = args.B
        Xb = make_inputs(sr, cols, B, 1)
        try:
            line["reference_gpu"], _ = reference_gpu_rate(g, sr, rows, cols, Xb, B, int(os.environ.get(
                "LOCAL_RANK", "0")))
        except (RuntimeError, OSError) as e:
            line["reference_gpu"] = {"unavailable": str(e).splitlines()[0] if str(e) else "no GPU"}
    print(json.dumps(line), flush=True)
    return 0


def timed_loop(torch, stream, fn, n):
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(n):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / n


def cusparse_baseline(torch, args, rows, cols, B, n=20):
    """cuSPARSE CSR SpMM (through torch.sparse) on the UNCOMPRESSED matrix of the
    same workload, fp32, same B: the reference's library baseline
    (gpu-engine/cusparse_test.cu:432-502).  Reported beside the engine; not the
    path under test."""
    import gmr

    if args.workload not in MOSAICS or args.semiring != "plustimes":
        return None
    r, c, F, sw, mu, seed = MOSAICS[args.workload]
    t0 = time.perf_counter()
    m = gmr.gen_mosaic(r, c, F, sw, mu, seed)
    codes = m.codes()
    del m
    ends = np.flatnonzero(codes == 0)
    crow = np.zeros(rows + 1, dtype=np.int64)
    crow[1:len(ends) + 1] = ends - np.arange(len(ends))
    crow[len(ends) + 1:] = crow[len(ends)]
    colv = (codes[codes != 0] - 1).astype(np.int32)  # value index 0: every stored value is 1
    del codes
    nnz = int(colv.size)
    try:
        A = torch.sparse_csr_tensor(torch.from_numpy(crow).cuda(), torch.from_numpy(colv).to(torch.int64).cuda(),
                                    torch.ones(nnz, device="cuda"), size=(rows, cols))
    except RuntimeError as e:  # out of memory or unsupported
        return {"unavailable": str(e).splitlines()[0]}
    build_s = time.perf_counter() - t0
    X = torch.rand((cols, B), device="cuda") * 2 - 1
    stream = torch.cuda.current_stream()
    for _ in range(3):
        Yc = A @ X
    ms = timed_loop(torch, stream, lambda: A @ X, n)
    x1 = X[:, :1].contiguous()
    for _ in range(3):
        A @ x1
    ms1 = timed_loop(torch, stream, lambda: A @ x1, n)
    Y_torch = (A @ X).cpu()
    out = {"spmm_vps": B * 1000.0 / ms, "spmm_ms": ms, "spmv_vps": 1000.0 / ms1, "nnz": nnz,
           "csr_bytes": int(nnz * 8 + (rows + 1) * 8), "build_s": round(build_s, 1),
           "how": "torch.sparse_csr_tensor @ dense (cuSPARSE), fp32, int64 indices"}
    del A, Yc
    torch.cuda.empty_cache()
    try:
        gen = cusparse_generic(torch, crow, colv, rows, cols, X, B, n, Y_torch)
    except Exception as e:  # noqa: BLE001  (a baseline: report, do not fail the bench)
        gen = {"unavailable": f"{type(e).__name__}: {e}"}
    out["generic"] = gen
    best = max([v for v in (gen.get("spmm_vps") or {}).values() if isinstance(v, float)] + [out["spmm_vps"]])
    out["best_spmm_vps"] = best
    torch.cuda.empty_cache()
    return out


# cuSPARSE generic-API constants (cusparse.h, library_types.h)
_CUDA_R_32F, _CUSPARSE_INDEX_32I, _CUSPARSE_INDEX_BASE_ZERO, _CUSPARSE_OP_N, _CUSPARSE_ORDER_ROW = 0, 2, 0, 0, 2
_SPMM_ALGS = {"ALG_DEFAULT": 0, "CSR_ALG1": 4, "CSR_ALG2": 6, "CSR_ALG3": 12}
_SPMV_ALGS = {"ALG_DEFAULT": 0, "CSR_ALG1": 2, "CSR_ALG2": 3}


def cusparse_generic(torch, crow, colv, rows, cols, X, B, n, Y_check):
    """cuSPARSE's generic SpMM / SpMV called directly, int32 CSR indices, with
    every algorithm the reference's baseline sweeps (ALG_DEFAULT, CSR_ALG2,
    CSR_ALG3 for B > 1, and CSR_ALG1; gpu-engine/cusparse_test.cu:432-502).
    Each algorithm's Y is compared with torch's CSR product of the same X."""
    import ctypes as C

    lib = None
    for name in ("libcusparse.so.12", "/usr/local/cuda/lib64/libcusparse.so.12", "libcusparse.so"):
        try:
            lib = C.CDLL(name)
            break
        except OSError:
            continue
    if lib is None:
        return {"unavailable": "libcusparse not found"}
    P, I64, VP = C.c_void_p, C.c_int64, C.POINTER(C.c_void_p)

    def ok(st, what):
        if st != 0:
            raise RuntimeError(f"{what}: cusparse status {st}")

    dev_crow = torch.from_numpy(crow.astype(np.int32)).cuda()
    dev_col = torch.from_numpy(colv).cuda()
    nnz = int(colv.size)
    vals = torch.ones(nnz, device="cuda")
    Y = torch.empty((rows, B), device="cuda")
    h, A, Xd, Yd = P(), P(), P(), P()
    stream = torch.cuda.current_stream()
    ok(lib.cusparseCreate(C.byref(h)), "create")
    ok(lib.cusparseSetStream(h, P(stream.cuda_stream)), "stream")
    ok(lib.cusparseCreateCsr(C.byref(A), I64(rows), I64(cols), I64(nnz), P(dev_crow.data_ptr()),
                             P(dev_col.data_ptr()), P(vals.data_ptr()), _CUSPARSE_INDEX_32I, _CUSPARSE_INDEX_32I,
                             _CUSPARSE_INDEX_BASE_ZERO, _CUDA_R_32F), "csr")
    ok(lib.cusparseCreateDnMat(C.byref(Xd), I64(cols), I64(B), I64(B), P(X.data_ptr()), _CUDA_R_32F,
                               _CUSPARSE_ORDER_ROW), "X")
    ok(lib.cusparseCreateDnMat(C.byref(Yd), I64(rows), I64(B), I64(B), P(Y.data_ptr()), _CUDA_R_32F,
                               _CUSPARSE_ORDER_ROW), "Y")
    one, zero = C.c_float(1.0), C.c_float(0.0)
    res, errs = {}, {}
    ref = Y_check.numpy().astype(np.float64)
    den = max(np.abs(ref).max(), 1e-30)
    for name, alg in _SPMM_ALGS.items():
        size = C.c_size_t()
        st = lib.cusparseSpMM_bufferSize(h, _CUSPARSE_OP_N, _CUSPARSE_OP_N, C.byref(one), A, Xd, C.byref(zero), Yd,
                                         _CUDA_R_32F, alg, C.byref(size))
        if st != 0:
            res[name] = f"unsupported (status {st})"
            continue
        buf = torch.empty(max(int(size.value), 16), dtype=torch.uint8, device="cuda")
        if alg == _SPMM_ALGS["CSR_ALG3"]:
            st = lib.cusparseSpMM_preprocess(h, _CUSPARSE_OP_N, _CUSPARSE_OP_N, C.byref(one), A, Xd, C.byref(zero),
                                             Yd, _CUDA_R_32F, alg, P(buf.data_ptr()))
            if st != 0:
                res[name] = f"unsupported (preprocess status {st})"
                continue

        def run():
            ok(lib.cusparseSpMM(h, _CUSPARSE_OP_N, _CUSPARSE_OP_N, C.byref(one), A, Xd, C.byref(zero), Yd,
                                _CUDA_R_32F, alg, P(buf.data_ptr())), name)

        try:
            for _ in range(3):
                run()
            ms = timed_loop(torch, stream, run, n)
        except RuntimeError as e:
            res[name] = f"unsupported ({e})"
            continue
        res[name] = B * 1000.0 / ms
        errs[name] = float(np.abs(Y.cpu().numpy().astype(np.float64) - ref).max() / den)
        del buf
    # SpMV, B = 1, first column of X
    x1 = X[:, 0].contiguous()
    y1 = torch.empty(rows, device="cuda")
    xv, yv = P(), P()
    ok(lib.cusparseCreateDnVec(C.byref(xv), I64(cols), P(x1.data_ptr()), _CUDA_R_32F), "x")
    ok(lib.cusparseCreateDnVec(C.byref(yv), I64(rows), P(y1.data_ptr()), _CUDA_R_32F), "y")
    resv = {}
    for name, alg in _SPMV_ALGS.items():
        size = C.c_size_t()
        st = lib.cusparseSpMV_bufferSize(h, _CUSPARSE_OP_N, C.byref(one), A, xv, C.byref(zero), yv, _CUDA_R_32F,
                                         alg, C.byref(size))
        if st != 0:
            resv[name] = f"unsupported (status {st})"
            continue
        buf = torch.empty(max(int(size.value), 16), dtype=torch.uint8, device="cuda")

        def runv():
            ok(lib.cusparseSpMV(h, _CUSPARSE_OP_N, C.byref(one), A, xv, C.byref(zero), yv, _CUDA_R_32F, alg,
                                P(buf.data_ptr())), name)

        for _ in range(3):
            runv()
        resv[name] = 1000.0 / timed_loop(torch, stream, runv, n)
        del buf
    for d in (xv, yv):
        lib.cusparseDestroyDnVec(d)
    for d in (Xd, Yd):
        lib.cusparseDestroyDnMat(d)
    lib.cusparseDestroySpMat(A)
    lib.cusparseDestroy(h)
    return {"spmm_vps": res, "spmm_rel_err_vs_torch": errs, "spmv_vps": resv,
            "how": "cusparseSpMM / cusparseSpMV (generic API, ctypes), int32 CSR, row-major X and Y, fp32"}


def run_pack8(args):
    """Eight mosaic grammars of uneven size (rows ~U{5k..200k}, cols ~U{1k..10k},
    seeds 10-17), each with its own B in {1, 4, 16, 64}, packed into one graph
    launch of per-engine branches (the default pack mode).  The same pack as
    one launch per level over all grammars, as one persistent kernel, and the
    engines one after another are timed beside it."""
    import torch

    import gmr

    rng = np.random.default_rng(17)
    engines, Xs, Ys, Bs, total_alg, info, grammars, Xhs = [], [], [], [], 0.0, [], [], []
    for i in range(8):
        rows, cols = int(rng.integers(5_000, 200_001)), int(rng.integers(1_000, 10_001))
        g, gi = mosaic_grammar(rows, cols, 64, 0.01, 1e-3, 10 + i)
        plan = gmr.Plan.build(g, rows, cols)
        B = [1, 4, 16, 64][i % 4]
        eng = gmr.Engine(plan)
        Xh = make_inputs(0, cols, B, 100 + i)
        X = torch.from_numpy(Xh).cuda()
        grammars.append((g, rows, cols))
        Xhs.append(Xh)
        Y = torch.empty((rows, B), device="cuda")
        st = torch.cuda.current_stream().cuda_stream
        eng.autotune(0, X.data_ptr(), Y.data_ptr(), B, stream=st)
        engines.append(eng)
        Xs.append(X)
        Ys.append(Y)
        Bs.append(B)
        total_alg += plan.alg_bytes(0, B)
        info.append({"rows": rows, "cols": cols, "B": B, "ops": plan.stats["n_ops"]})
    pack = gmr.Pack(engines)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    def packed():
        pack.multiply_device([0] * 8, [x.data_ptr() for x in Xs], [y.data_ptr() for y in Ys], Bs, stream=sp)

    def sequential():
        for e, x, y, b in zip(engines, Xs, Ys, Bs):
            e.multiply_device(0, x.data_ptr(), y.data_ptr(), b, stream=sp)

    for _ in range(args.warmup):
        packed()
        sequential()
    ms_seq = timed_loop(torch, stream, sequential, args.steps)
    pack.set_mode(gmr.Pack.LEVELS)  # one launch per level over all grammars
    for _ in range(args.warmup):
        packed()
    ms_levels = timed_loop(torch, stream, packed, args.steps)
    pack.set_mode(gmr.Pack.PERSISTENT)  # one cooperative kernel for the whole pack
    for _ in range(args.warmup):
        packed()
    ms_persistent = timed_loop(torch, stream, packed, args.steps)
    torch.cuda.synchronize()
    persistent_ran = pack.status()[0]
    pack.set_mode(gmr.Pack.GRAPH)  # the headline: the default, one graph of per-engine branches
    for _ in range(args.warmup):
        packed()
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.3)
    ms = timed_loop(torch, stream, packed, args.steps)
    clocks = sampler.stop()
    vecs = sum(Bs)
    check = None
    if not args.no_check:
        from oracle import oracle as O
        check = []
        for (g, rows, cols), Xh, Yd, B in zip(grammars, Xhs, Ys, Bs):
            sched = O.RefSchedule(g.alpha, g.rules(), g.C())
            check.append(check_all_columns(sched, g.values(), 0, Xh, Yd.cpu().numpy(), rows, cols, B,
                                           os.cpu_count() or 1))
        check = {"grammars": check, "ok": all(c["ok"] for c in check),
                 "rel_err_fp64_max": max(c["rel_err_fp64_max"] for c in check)}
    out = {"metric": METRIC, "value": vecs * 1000.0 / ms, "unit": "vectors/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": "pack8", "grammars": info, "seeds": list(range(10, 18)),
                      "l2": "inputs larger than L2; no flush"},
           "sequential_vps": vecs * 1000.0 / ms_seq, "pack_gain": ms_seq / ms,
           "mode": "one graph launch of per-engine branches (default pack mode)",
           "levels_pack_vps": vecs * 1000.0 / ms_levels, "levels_pack_gain": ms_seq / ms_levels,
           "persistent_pack_vps": vecs * 1000.0 / ms_persistent, "persistent_pack_gain": ms_seq / ms_persistent,
           "persistent_ran": persistent_ran,
           "step_alg_gbs": total_alg / (ms / 1000.0) / 1e9, "gpu_launches": int(pack.last_launches * args.steps),
           "clocks": clocks, "check": check}
    print(json.dumps(out), flush=True)
    return 0


def run_repair_compare(args):
    """RePair of the workload's matrix on the GPU and on all host cores: both
    timed, grammars compared symbol for symbol."""
    import gmr

    if args.workload in MOSAICS:
        r, c, F, sw, mu, seed = MOSAICS[args.workload]
        m = gmr.gen_mosaic(r, c, F, sw, mu, seed)
    else:
        nodes, deg, cp, seed = GRAPH
        m = gmr.gen_copy_graph(nodes, deg, cp, args.semiring == "tropical", seed)
    gmr.repair(gmr.gen_mosaic(500, 100, 8, 0.02, 1e-3, 1), device=0)  # loads the kernels
    t = time.perf_counter()
    gd = gmr.repair(m, device=0)
    td = time.perf_counter() - t
    t = time.perf_counter()
    gh = gmr.repair(m)
    th = time.perf_counter() - t
    same = gd.alpha == gh.alpha and np.array_equal(gd.rules(), gh.rules()) and np.array_equal(gd.C(), gh.C())
    print(json.dumps({"metric": "RePair seconds", "unit": "s", "value": td, "higher_is_better": False,
                      "config": {"workload": args.workload, "symbols": int(m.info.len), "nnz": int(m.nnz)},
                      "host_s": th, "host_threads": os.cpu_count(), "speedup": th / td, "identical": bool(same),
                      "rules": int(len(gd.rules())), "C": int(len(gd.C()))}))
    return 0


def run_other_op(args):
    """Left product (Y = X^T M) or fixpoint iteration timed on the workload's grammar."""
    import torch

    import gmr

    g, rows, cols, ginfo = workload_grammar(args)
    plan = gmr.Plan.build(g, rows, cols)
    eng = gmr.Engine(plan)
    sr, B = SR_IDS[args.semiring], args.B
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    out = {"metric": f"{args.op} vectors/s", "unit": "vectors/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "higher_is_better": True, "dtype": dtype_of(sr), "data": "synthetic",
           "config": workload_config(args, rows, cols) | {"op": args.op}}
    if args.op == "left":
        t0 = time.perf_counter()
        eng.enable_left(plan)
        out["prepare_s"] = round(time.perf_counter() - t0, 2)
        X = torch.from_numpy(make_inputs(sr, rows, B, 5).view(np.int32)).cuda()
        Y = torch.empty((cols, X.shape[1]), dtype=torch.int32, device="cuda")
        for _ in range(args.warmup):
            eng.multiply_left_device(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp)
        ms = timed_loop(torch, stream, lambda: eng.multiply_left_device(sr, X.data_ptr(), Y.data_ptr(), B,
                                                                         stream=sp), args.steps)
        out |= {"value": B * 1000.0 / ms, "ms_per_step": ms}
    else:
        if rows != cols:
            print(json.dumps({"unavailable": "fixpoint needs a square matrix (graph workload)"}))
            return 0
        X0 = make_inputs(sr, cols, B, 5)
        if sr == 2:
            X0 = np.where(X0 == INT_MAX, np.int32(1_000_000_000), X0).astype(np.int32)
        X = torch.from_numpy(X0.view(np.int32)).cuda()
        Y = torch.empty_like(X)
        eng.multiply_device(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp)  # graph capture
        Xs = X.clone()
        torch.cuda.synchronize()
        t = time.perf_counter()
        iters = eng.fixpoint_device(sr, X.data_ptr(), Y.data_ptr(), B, max_iters=10_000, stream=sp)
        torch.cuda.synchronize()
        s = time.perf_counter() - t
        out |= {"value": B / s, "ms_per_step": s * 1000.0, "iterations": iters,
                "ms_per_iteration": s * 1000.0 / max(iters, 1), "start_nonzero_words": int((Xs != 0).sum())}
    print(json.dumps(out), flush=True)
    return 0


def load_mode_model(learn):
    """The emission-mode model, when one is committed (else the learned table
    pulls every level's emissions)."""
    return learn.Mlp.load(learn.MODE_MODEL_PATH) if learn.MODE_MODEL_PATH.exists() else None


def run_launch_list(args):
    """One eager multiply of the workload, launch by launch, with the
    headline's per-launch table (--table learned | autotuned | default), after
    --warmup others: the command that the ncu captures of k_level run.  Prints
    the per-launch device times and the launch count of one multiply."""
    import torch

    import gmr
    from gmr import learn

    torch.cuda.set_device(0)
    g, rows, cols, _ = workload_grammar(args)
    plan = gmr.Plan.build(g, rows, cols, device=0)
    eng = gmr.Engine(plan)
    sr, B = SR_IDS[args.semiring], args.B
    Xh = make_inputs(sr, cols, B, 1)
    X = torch.from_numpy(Xh.view(np.int32)).cuda()
    Y = torch.empty((rows, Xh.shape[1]), dtype=torch.int32, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    if args.table == "learned":
        learn.choose_learned(eng, plan, learn.Mlp.load(learn.MODEL_PATH), sr, B, mode_model=load_mode_model(learn))
    elif args.table == "autotuned":
        eng.autotune(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp, reps=3)
    elif args.table == "push":  # default variants, every level pushes its emissions into Y
        d = plan.stats["depth"]
        eng.set_level_variants(sr, B, [0] + [gmr.LEVEL_PUSH] * d + [0])
    elif args.table == "stage":  # default variants, every level stages its left-child windows
        d = plan.stats["depth"]
        eng.set_level_variants(sr, B, [0] + [gmr.LEVEL_STAGE] * d + [0])
    table = eng.level_variants(sr, B)
    for _ in range(args.warmup):
        eng.time_launches(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp)
    ms = eng.time_launches(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp)
    print(json.dumps({"op": "launches", "workload": args.workload, "semiring": args.semiring, "B": B,
                      "table_kind": args.table, "table": None if table is None else [int(v) for v in table],
                      "launches_per_multiply": int(eng.last_launches), "level_launches": int(eng.last_launches) - 1,
                      "warmup_multiplies": args.warmup, "launch_ms": [round(float(t), 5) for t in ms],
                      "source_hash": source_hash(args.table)}), flush=True)
    return 0


def run_gather_sweep(args):
    """The gather calibration along every load path: random 128-byte units
    (and larger units for bulk copies) from a buffer that fits in L2 (64 MB)
    and one that does not (4 GB), at several depths of loads in flight."""
    import gmr

    cases = ([("load16", d, 128) for d in (1, 2, 4, 8, 16)] + [("load32", d, 128) for d in (2, 4, 8)] +
             [("seq16", d, 128) for d in (4, 16)] + [("bulk", d, 128) for d in (2, 8, 16, 32, 64)] +
             [("bulk", 4, u) for u in (512, 2048, 8192)])
    rows = []
    for buf in (64 << 20, 4 << 30):
        for mode, depth, unit in cases:
            gbs = gmr.measure_gather(buf, mode=mode, depth=depth, unit_bytes=unit)
            rows.append({"buffer_mb": buf >> 20, "mode": mode, "depth": depth, "unit_bytes": unit,
                         "gbs": round(gbs, 1)})
            print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
    print(json.dumps({"op": "gather", "unit": "GB/s", "results": rows}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gmr", "reference"], default="gmr")
    ap.add_argument("--workload", choices=WORKLOADS, default="mosaic-200000x10000")
    ap.add_argument("--semiring", choices=list(SR_IDS), default=None)
    ap.add_argument("--B", type=int, default=32)
    ap.add_argument("--variant", type=int, default=0,
                    help="0 auto (learned / autotuned per-launch table, CUDA graph), 1 plain, 2 fused, 3 graph, "
                         "4 persistent")
    ap.add_argument("--push", type=int, default=0, choices=[0, 1, 2, 3],
                    help="how each level's emissions reach Y: 0 as the per-launch table says, 1 gathered by the "
                         "next launch (pull), 2 pushed by every level that can, 3 every level that can "
                         "interleaves (source chunks, each folded by the next launch)")
    ap.add_argument("--no-check", action="store_true", help="skip checking every column against the oracle")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner and the learned choice")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--dump-launches", action="store_true", help="per-launch times and level sizes to stderr")
    ap.add_argument("--no-cusparse", action="store_true", help="skip the cuSPARSE CSR baseline")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="--impl reference: skip timing the reference's own GPU engine beside its CPU sweep")
    ap.add_argument("--table", choices=["learned", "autotuned", "default", "push", "stage"], default="learned",
                    help="--op launches: the per-launch table of the multiply")
    ap.add_argument("--op", choices=["right", "left", "fixpoint", "repair", "gather", "launches"], default="right",
                    help="right: Y = M X (the headline); left: Y = X^T M; fixpoint: X <- X (+) M X to convergence; "
                         "repair: RePair of the workload's matrix on the GPU vs the host; "
                         "gather: the random-gather calibration along every load path; "
                         "launches: one eager multiply launch by launch (the ncu capture's command)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.semiring is None:
        args.semiring = "boolean" if args.workload == "graph-16777216" else "plustimes"
    if args.impl == "reference":
        global REPAIR_ON_GPU
        REPAIR_ON_GPU = False
        return run_reference(args)
    if args.workload == "pack8":
        return run_pack8(args)
    if args.op == "repair":
        return run_repair_compare(args)
    if args.op == "gather":
        return run_gather_sweep(args)
    if args.op == "launches":
        return run_launch_list(args)
    if args.op != "right":
        return run_other_op(args)

    import torch

    import gmr
    from gmr import learn

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    gmr.lib()

    if ws > 1 and rank != 0:
        torch.distributed.barrier()
    g, rows, cols, ginfo = workload_grammar(args)
    if ws > 1 and rank == 0:
        torch.distributed.barrier()
    # schedule: built on the GPU (timed on a second build, after the first
    # loaded the kernels), checked array for array against the host build
    t0 = time.perf_counter()
    plan = gmr.Plan.build(g, rows, cols, device=local)
    plan_dev_first_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    plan = gmr.Plan.build(g, rows, cols, device=local)
    plan_dev_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    plan_host = gmr.Plan.build(g, rows, cols)
    plan_s = time.perf_counter() - t0
    plan_same = plan_host.stats == plan.stats and all(
        np.array_equal(plan.array(a), plan_host.array(a)) for a in
        ("op_l", "op_r", "op_c", "lvl_off", "em_off", "em_src", "em_row", "term_val", "term_col", "seg_off",
         "seg_row", "seg_start"))
    del plan_host
    st = plan.stats
    eng = gmr.Engine(plan, device=local)
    sr = SR_IDS[args.semiring]
    B = args.B
    Xh = make_inputs(sr, cols, B, 1 + rank)
    words = Xh.shape[1]
    X = torch.from_numpy(Xh.view(np.int32)).to(dev)
    Y = torch.empty((rows, words), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    cfg = dict(variant=args.variant, push=args.push)

    def step():
        eng.multiply_device(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp, **cfg)

    def step_cfg(**c):
        eng.multiply_device(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp, **c)

    nvml = NvmlEnergy(local)

    def energy_of(fn, seconds=1.5):
        """mJ per vector of fn() repeated for about `seconds` (NVML energy counter)."""
        if nvml.h is None:
            return None
        fn()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize(dev)
        n = max(1, int(seconds / max(time.perf_counter() - t0, 1e-5)))
        e0 = nvml.mj()
        for _ in range(n):
            fn()
        torch.cuda.synchronize(dev)
        e1 = nvml.mj()
        return None if e0 is None or e1 is None else (e1 - e0) / (n * B)

    def timed(n, **c):
        for _ in range(3):
            eng.multiply_device(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp, **c)
        return timed_loop(torch, stream, lambda: eng.multiply_device(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp,
                                                                     **c), n)

    tuning = {}
    if args.variant == 0:
        tuning["default_vps"] = B * 1000.0 / timed(20, variant=3)
        tuning["default_pull_vps"] = B * 1000.0 / timed(20, variant=3, push=1)
        tuning["default_push_vps"] = B * 1000.0 / timed(20, variant=3, push=2)
        # the same untuned multiply with 16- and 32-byte lane accesses, back to back
        tuning["default_lane16_vps"] = B * 1000.0 / timed(20, variant=3, lane_bytes=16)
        tuning["default_lane32_vps"] = B * 1000.0 / timed(20, variant=3, lane_bytes=32)
        if not args.no_tune:
            t0 = time.perf_counter()
            eng.autotune(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp, reps=3)
            tuning["autotune_s"] = round(time.perf_counter() - t0, 2)
            tuning["autotuned_table"] = [int(v) for v in eng.level_variants(sr, B)]
            auto_ms = timed(30)
            tuning["autotuned_vps"] = B * 1000.0 / auto_ms
            tuning["autotuned_mj_per_vector"] = energy_of(lambda: step_cfg(variant=0))
            # energy-aware table: chunked twins within 10 % of the fastest variant
            eng.autotune(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp, reps=3, energy_tolerance=0.10)
            tuning["energy_table"] = [int(v) for v in eng.level_variants(sr, B)]
            tuning["energy_table_vps"] = B * 1000.0 / timed(30)
            tuning["energy_table_mj_per_vector"] = energy_of(lambda: step_cfg(variant=0))
            eng.autotune(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp, reps=3)

            def slot_us():  # eager per-launch-slot device times of the installed table (median of 3)
                runs = [eng.time_launches(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp) for _ in range(3)]
                n = min(len(r) for r in runs)
                return [round(float(np.median([r[i] for r in runs])) * 1000.0, 1) for i in range(n)]

            tuning["autotuned_slot_us"] = slot_us()
            if learn.MODEL_PATH.exists():
                model = learn.Mlp.load(learn.MODEL_PATH)
                t0 = time.perf_counter()
                learn.choose_learned(eng, plan, model, sr, B, mode_model=load_mode_model(learn))
                tuning["learned_choice_s"] = round(time.perf_counter() - t0, 3)
                tuning["learned_table"] = [int(v) for v in eng.level_variants(sr, B)]
                tuning["learned_slot_us"] = slot_us()
                learned_ms = timed(30)
                tuning["learned_vps"] = B * 1000.0 / learned_ms
                tuning["learned_regret_vs_autotuner"] = learned_ms / auto_ms - 1.0
                if learned_ms <= 1.10 * auto_ms:
                    tuning["headline"] = "learned"
                else:  # the learned pick falls back to the autotuner's measured choice
                    eng.set_level_variants(sr, B, tuning["autotuned_table"])
                    tuning["headline"] = "autotuned (the learned pick was more than 10 % slower)"
            else:
                tuning["headline"] = "autotuned (no trained cost model present)"

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
    Y_timed = Y.cpu().numpy()  # the timed multiplies' result, checked against the oracle below
    ms = slowest_rank_ms(e0.elapsed_time(e1), ws, dev)
    ms_per_step = ms / args.steps
    value = whole_job_vps(ws, B, args.steps, ms)

    # ---- energy per vector: NVML energy counter around >= 2 s of steps
    energy = None
    nv = nvml
    if nv.h is not None:
        n_e = max(1, int(2000.0 / max(ms_per_step, 1e-3)))
        torch.cuda.synchronize(dev)
        e_start, t_start = nv.mj(), time.perf_counter()
        for _ in range(n_e):
            step()
        torch.cuda.synchronize(dev)
        e_end, t_end = nv.mj(), time.perf_counter()
        if e_start is not None and e_end is not None and e_end > e_start:
            joules = (e_end - e_start) / 1000.0
            energy = {"mj_per_vector": 1000.0 * joules / (n_e * B), "avg_power_w": joules / (t_end - t_start),
                      "steps": n_e, "how": "NVML total energy counter around the steps (whole GPU)"}

    # ---- per-launch times (the same kernels launched one by one) for the roofline
    reps = 5
    lt = np.mean([eng.time_launches(sr, X.data_ptr(), Y.data_ptr(), B, stream=sp, **cfg)
                  for _ in range(reps)], axis=0)
    eager_level_ms = float(lt[1:].sum()) if len(lt) > 1 else float(lt.sum())  # k_level launches (persistent: one)
    # the dominant kernel's time inside the timed graph replay: the step's time
    # times the level launches' share of the same launches timed one by one
    level_share = eager_level_ms / float(lt.sum()) if len(lt) > 1 else 1.0
    level_ms = ms_per_step * level_share
    assert level_ms <= ms_per_step
    if args.dump_launches:
        ops, ems = plan.level_ops(), plan.level_emits()
        log("launch\tms\tops(level k)\temits(level k-1)")
        for i, t_ms in enumerate(lt):
            o = int(ops[i]) if 1 <= i < len(ops) else 0
            em = int(ems[i - 1]) if 1 <= i <= len(ems) else 0
            log(f"{i}\t{t_ms:.4f}\t{o}\t{em}")
    alg_total = plan.alg_bytes(sr, B)
    alg_pro = 8.0 * (st["ref_alpha"] - 1) + 4.0 * st["n_vals"] + 4.0 * cols * words + 4.0 * rows * words
    alg_level = alg_total - alg_pro      # 12 N_L + 8 E + 8 E_T
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_level / (level_ms / 1000.0) / 1e9
    # value traffic the sweep must move at this B (every emission gathers one
    # value, every rule reads two and writes one), against the measured ceilings
    # of random 128-byte gathers from L2 and from HBM on this GPU
    vbytes = 4.0 * words * (st["n_emit"] + st["n_term_emit"] + 3 * st["n_ops"])
    lane_mode = "load32" if eng.lane_bytes(sr, B) == 32 else "load16"  # the load path the sweep uses here
    ceil_l2 = gmr.measure_gather(64 << 20, mode=lane_mode, depth=4, device=local)
    ceil_hbm = gmr.measure_gather(4 << 30, mode=lane_mode, depth=4, device=local)
    l2_seq = gmr.measure_gather_bandwidth(64 << 20, device=local, sequential=True)
    value_gbs = vbytes / (level_ms / 1000.0) / 1e9
    step_gbs = alg_total / (ms_per_step / 1000.0) / 1e9
    head = tuning.get("headline", "")
    tkey = (f"{args.workload}/{args.semiring}/B{B}/"
            f"{'learned' if head == 'learned' else 'autotuned' if head.startswith('autotuned') else 'default'}")
    traffic_ent, traffic_why = traffic_entry(tkey)
    traffic = traffic_ent["dram_bytes_per_multiply"] if traffic_ent else None

    # ---- plain per-level sweep, one vector at a time (the reference's scheme)
    x1 = torch.from_numpy(make_inputs(sr, cols, 1, 7).view(np.int32)).to(dev)
    y1 = torch.empty((rows, 1), dtype=torch.int32, device=dev)
    for _ in range(3):
        eng.multiply_device(sr, x1.data_ptr(), y1.data_ptr(), 1, stream=sp, variant=1)
    torch.cuda.synchronize(dev)
    kp = max(10, min(100, args.steps))
    plain_ms = timed_loop(torch, stream,
                          lambda: eng.multiply_device(sr, x1.data_ptr(), y1.data_ptr(), 1, stream=sp, variant=1), kp)
    plain_vps = 1000.0 / plain_ms

    # ---- end to end through the public API with host buffers (pinned): every
    # step copies its X in and its Y out; steps are pipelined (two staging
    # pairs), and the one-call-per-step synchronous figure is kept beside it
    ke = max(10, min(100, args.steps))
    Xps = [torch.from_numpy(make_inputs(sr, cols, B, 100 + i).view(np.int32)).pin_memory() for i in range(4)]
    Yps = [torch.empty((rows, words), dtype=torch.int32).pin_memory() for _ in range(4)]
    xs = [Xps[i % 4].data_ptr() for i in range(ke)]
    ys = [Yps[i % 4].data_ptr() for i in range(ke)]
    eng.multiply_host_many(sr, xs[:4], ys[:4], B)
    t = time.perf_counter()
    eng.multiply_host_many(sr, xs, ys, B)
    e2e_s = (time.perf_counter() - t) / ke
    e2e_value = ws * B / e2e_s
    for _ in range(3):
        gmr.lib().gmr_engine_multiply_host(eng._h, sr, Xps[0].data_ptr(), Yps[0].data_ptr(), B, None)
    t = time.perf_counter()
    for _ in range(ke):
        rc = gmr.lib().gmr_engine_multiply_host(eng._h, sr, Xps[0].data_ptr(), Yps[0].data_ptr(), B, None)
        if rc:
            raise RuntimeError(gmr.lib().gmr_last_error().decode())
    e2e_sync_value = ws * B / ((time.perf_counter() - t) / ke)

    out = {
        "metric": METRIC, "value": value, "unit": "vectors/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": dtype_of(sr), "data": "synthetic (seeded generator + RePair)",
        "config": run_config(args, rows, cols, ws),
        "tuning": tuning,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "traffic_source": traffic_ent if traffic_ent else {"unavailable": traffic_why},
                     "kernel": "k_level (all level launches of one multiply)",
                     "alg_bytes_per_multiply": alg_level, "kernel_ms_per_multiply": level_ms,
                     "kernel_ms_source": "timed graph replay (ms_per_step) x the level launches' share of the "
                                         "same launches timed one by one",
                     "level_share": level_share, "eager_level_ms": eager_level_ms,
                     "step_alg_gbs": step_gbs,
                     "gather_ceiling": {"value_bytes_per_multiply": vbytes, "achieved_gbs": value_gbs,
                                        "l2_random_128B_gbs": ceil_l2, "hbm_random_128B_gbs": ceil_hbm,
                                        "l2_sequential_gbs": l2_seq,
                                        "frac_of_l2_ceiling": value_gbs / ceil_l2}},
        "e2e": {"value": e2e_value, "unit": "vectors/s", "h2d_bytes_per_step": int(cols * words * 4),
                "d2h_bytes_per_step": int(rows * words * 4), "api": "gmr_engine_multiply_host_many (pipelined)",
                "synchronous_per_call_value": e2e_sync_value},
        "gpu_launches": int(launches_per_step * args.steps),
        "energy": energy,
        "clocks": clocks,
        "plain_sweep_b1": {"value": plain_vps, "unit": "vectors/s", "speedup": value / ws / plain_vps},
        "grammar": {"ops": st["n_ops"], "depth": st["depth"], "layered_rules": st["ref_layered"],
                    "passthrough": st["ref_passthrough"], "max_width": st["ref_max_width"],
                    "emit": st["ref_emit"], "term_emit": st["ref_term_emit"], "terminals": st["ref_alpha"],
                    "plan_s": round(plan_s, 2), "plan_device_s": round(plan_dev_s, 3),
                    "plan_device_first_s": round(plan_dev_first_s, 3), "plan_device_identical": plan_same} | ginfo,
    }
    if rank == 0 and ws == 1 and not args.no_cusparse:
        del eng  # free the engine's device memory before building the CSR baseline
        torch.cuda.synchronize(dev)
        out["cusparse_csr"] = cusparse_baseline(torch, args, rows, cols, B)
        if out["cusparse_csr"] and "spmm_vps" in out["cusparse_csr"]:
            out["cusparse_csr"]["engine_speedup"] = value / out["cusparse_csr"]["best_spmm_vps"]
    sched = None
    threads = os.cpu_count() or 1
    if rank == 0 and not args.no_check:
        from oracle import oracle as O
        sched = O.RefSchedule(g.alpha, g.rules(), g.C())
        out["check"] = check_all_columns(sched, g.values(), sr, Xh, Y_timed, rows, cols, B, threads)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        rate, n, spent, build_s = cpu_reference_rate(g, sr, rows, cols, args.cpu_seconds, threads, sched=sched)
        out["cpu_baseline"] = {"value": rate, "unit": "vectors/s", "cores": threads, "kind": "port",
                               "sample": f"{n} single vectors of the same grammar in {spent:.1f} s with the "
                                         f"reference's OpenMP level sweep (restated in oracle/)"}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
