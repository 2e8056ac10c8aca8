"""Learned scheduler: a small MLP cost model for the per-launch kernel variant.

For every launch of a multiply (the launch of level k: rules of level k and
emissions of level k-1) the engine can run any of GMR_N_LEVEL_VARIANTS kernel
variants (emission folding strategy x rules-per-CTA grid).  The exhaustive
autotuner (gmr_engine_autotune) measures all of them with the timing
recorder; this module turns those measurements into training data, trains a
3 x 64 fp32 MLP on the GPU with the library's own forward/backward/Adam
kernels, and uses it (gmr_engine_choose_learned, an inference kernel) to pick
the variants without measuring.  When no model is available the measured
autotuner choice is used; the autotuner also judges the model's regret.  The
model only picks schedules: every variant computes the same Y.

    python -m gmr.learn --out DIR [--grammars N]   # record, train, evaluate (GPU)
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import time
from pathlib import Path

import numpy as np

from . import _lib as L
from . import LEVEL_INTERLEAVE, Engine, Grammar, Plan, _check, gen_copy_graph, gen_mosaic, lib, repair, semiring_id

N_BASE = 17
N_VAR = 20
IN_DIM = N_BASE + N_VAR
MODEL_PATH = Path(__file__).resolve().parent / "models" / "cost_model.gmrmlp"
# Emission-mode model: per launch slot, log(time) given the slot's features and
# whether level k-1 and level k are interleaved (pull otherwise).
MODE_MODEL_PATH = Path(__file__).resolve().parent / "models" / "mode_model.gmrmlp"
MODE_IN = N_BASE + 2
PULL, INTERLEAVE = 0, 2           # the engine's mode indices (1 = push, not learned: it loses)
CHUNK_SLOTS = 1 << 19             # source slots per chunk (the engine's default)
MODE_DOMAIN = "(+,x), B >= 32"    # where the mode model was trained and is applied


def launch_features(plan: Plan, semiring, B: int) -> np.ndarray:
    """[depth + 2][16] base features of every launch slot (slot 0 = prologue, zeros)."""
    d = plan.stats["depth"]
    out = np.zeros((d + 2) * N_BASE, dtype=np.float32)
    n = C.c_int()
    _check(lib().gmr_plan_launch_features(plan._h, semiring_id(semiring), B, out.ctypes.data_as(L.F32P), len(out),
                                          C.byref(n)))
    return out.reshape(n.value, N_BASE)


def model_inputs(base: np.ndarray) -> np.ndarray:
    """[slots][16] -> [slots * N_VAR][26]: base features + variant one-hot."""
    slots = base.shape[0]
    X = np.zeros((slots, N_VAR, IN_DIM), dtype=np.float32)
    X[:, :, :N_BASE] = base[:, None, :]
    X[:, np.arange(N_VAR), N_BASE + np.arange(N_VAR)] = 1.0
    return X.reshape(slots * N_VAR, IN_DIM)


class Mlp:
    """The cost model (libgmr's gmr_mlp): in -> 64 -> 64 -> 64 -> 1, ReLU, fp32."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def create(cls, in_dim=IN_DIM, hidden=64, layers=3, seed=0) -> "Mlp":
        h = C.c_void_p()
        _check(lib().gmr_mlp_create(in_dim, hidden, layers, seed, C.byref(h)))
        return cls(h)

    @classmethod
    def load(cls, path=MODEL_PATH) -> "Mlp":
        h = C.c_void_p()
        _check(lib().gmr_mlp_load(os.fsencode(str(path)), C.byref(h)))
        return cls(h)

    def save(self, path):
        _check(lib().gmr_mlp_save(self._h, os.fsencode(str(path))))

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().gmr_mlp_free(self._h)
            self._h = C.c_void_p()

    @property
    def n_params(self) -> int:
        n = C.c_int64()
        _check(lib().gmr_mlp_info(self._h, None, None, None, C.byref(n)))
        return n.value

    def params(self) -> np.ndarray:
        p = np.zeros(self.n_params, dtype=np.float32)
        _check(lib().gmr_mlp_params(self._h, p.ctypes.data_as(L.F32P), None, len(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(lib().gmr_mlp_params(self._h, None, p.ctypes.data_as(L.F32P), len(p)))

    def set_norm(self, mean, std):
        mean = np.ascontiguousarray(mean, dtype=np.float32)
        std = np.ascontiguousarray(std, dtype=np.float32)
        _check(lib().gmr_mlp_set_norm(self._h, mean.ctypes.data_as(L.F32P), std.ctypes.data_as(L.F32P)))

    def predict(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros(len(X), dtype=np.float32)
        _check(lib().gmr_mlp_predict(self._h, X.ctypes.data_as(L.F32P), len(X), Y.ctypes.data_as(L.F32P)))
        return Y

    def gradients(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = C.c_float()
        _check(lib().gmr_mlp_gradients(self._h, X.ctypes.data_as(L.F32P), T.ctypes.data_as(L.F32P), len(X),
                                       g.ctypes.data_as(L.F32P), len(g), C.byref(loss)))
        return g, float(loss.value)

    def train(self, X, T, epochs=60, batch=512, lr=2e-3, seed=0) -> float:
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        loss = C.c_float()
        _check(lib().gmr_mlp_train(self._h, X.ctypes.data_as(L.F32P), T.ctypes.data_as(L.F32P), len(X), epochs,
                                   batch, lr, seed, C.byref(loss)))
        return float(loss.value)


def choose_learned(eng: Engine, plan: Plan, model: Mlp, semiring, B: int, mode_model: Mlp | None = None) -> np.ndarray:
    """Installs the model's per-launch choice; returns its predictions [slots][variants] (log us).
    With mode_model (applied in its training domain, (+,x) at B >= 32), the
    levels it predicts faster interleaved get GMR_LEVEL_INTERLEAVE."""
    slots = plan.stats["depth"] + 2
    pred = np.zeros(slots * N_VAR, dtype=np.float32)
    _check(lib().gmr_engine_choose_learned(eng._h, plan._h, model._h, semiring_id(semiring), B,
                                           pred.ctypes.data_as(L.F32P), len(pred)))
    if mode_model is not None and semiring_id(semiring) == 0 and B >= 32:
        modes = choose_modes(plan, mode_model, semiring, B)
        table = eng.level_variants(semiring, B)
        for k, m in enumerate(modes):
            if m == INTERLEAVE:
                table[k] |= LEVEL_INTERLEAVE
        eng.set_level_variants(semiring, B, table)
    return pred.reshape(slots, N_VAR)


def interleave_allowed(plan: Plan, chunk_slots: int = CHUNK_SLOTS) -> np.ndarray:
    """[slots] bool: level k can run in source chunks (two chunks or more)."""
    lvl = plan.array("lvl_off")
    d = plan.stats["depth"]
    ok = np.zeros(d + 2, dtype=bool)
    for k in range(1, d + 1):
        ok[k] = lvl[k] - lvl[k - 1] > chunk_slots
    return ok


def mode_inputs(base: np.ndarray, mp: int, m: int) -> np.ndarray:
    """[slots][18]: base features + (level k-1 interleaved, level k interleaved)."""
    x = np.zeros((base.shape[0], MODE_IN), dtype=np.float32)
    x[:, :N_BASE] = base
    x[:, N_BASE] = 1.0 if mp == INTERLEAVE else 0.0
    x[:, N_BASE + 1] = 1.0 if m == INTERLEAVE else 0.0
    return x


def best_chain(cost, allowed) -> tuple[list, float]:
    """The cheapest choice of pull / interleave per level: cost[k][mp][m] (any
    array indexable so; NaN or <= 0 = not available) for slots 1..D+1, level
    D+1 (the final fold) pulled.  Returns (mode per slot, total)."""
    n = len(allowed)
    inf = float("inf")
    acc = {PULL: 0.0, INTERLEAVE: inf}
    back = []
    for k in range(1, n):
        last = k == n - 1
        nxt, frm = {}, {}
        for m in (PULL, INTERLEAVE):
            if m == INTERLEAVE and (last or not allowed[k]):
                nxt[m] = inf
                continue
            best, arg = inf, PULL
            for mp in (PULL, INTERLEAVE):
                c = cost[k][mp][m]
                if acc[mp] == inf or not np.isfinite(c) or c <= 0:
                    continue
                if acc[mp] + c < best:
                    best, arg = acc[mp] + c, mp
            nxt[m], frm[m] = best, arg
        back.append(frm)
        acc = nxt
    modes = [PULL] * n
    m = PULL
    for k in range(n - 1, 0, -1):
        modes[k] = m
        m = back[k - 1].get(m, PULL)
    return modes, acc[PULL]


def choose_modes(plan: Plan, mode_model: Mlp, semiring, B: int) -> list:
    """Emission mode per launch slot (PULL / INTERLEAVE) from the mode model's
    predicted slot times, by the autotuner's chain recursion."""
    base = launch_features(plan, semiring, B)
    n = base.shape[0]
    cost = np.full((n, 3, 3), np.nan)
    for mp in (PULL, INTERLEAVE):
        for m in (PULL, INTERLEAVE):
            cost[:, mp, m] = np.exp(mode_model.predict(mode_inputs(base, mp, m)))
    return best_chain(cost, interleave_allowed(plan))[0]


def mode_rows(base: np.ndarray, costs: np.ndarray):
    """Training rows of the mode model from one autotune's mode costs [slots][3][3] (ms)."""
    X, T = [], []
    for mp in (PULL, INTERLEAVE):
        for m in (PULL, INTERLEAVE):
            c = costs[:, mp, m]
            keep = (np.arange(len(c)) >= 1) & (c > 0)
            if keep.any():
                X.append(mode_inputs(base, mp, m)[keep])
                T.append(np.log(c[keep] * 1000.0).astype(np.float32))
    if not X:
        return np.zeros((0, MODE_IN), np.float32), np.zeros(0, np.float32)
    return np.concatenate(X), np.concatenate(T)


# ---------------------------------------------------------------- corpus
def corpus_specs(n_mosaic: int, n_graph: int, seed0: int = 100, full: bool = True):
    """Seeded grammar specs of the scheduler corpus, one seed per grammar:
    mosaics take seeds seed0 .. seed0 + n_mosaic - 1, graphs the next n_graph
    (seed0 = 100 and 192 + 64 grammars give seeds 100-355).  Mosaics: rows
    10k-500k and cols 1k-20k, both log-uniform, with rows shrunk so that
    rows x cols x 1/2 stays below 1.2e9 non-zeros (the size the GPU RePair
    holds comfortably; 500k x 20k would be 5e9), founders 16-1024, switch
    rate 1e-3 to 5e-2.  Weighted copy-model graphs: 1M-16.8M nodes
    (log-uniform), degree 8-64, copy probability 0.3-0.9.  full=False keeps
    small ranges (rows 10k-60k, cols 1k-10k, nodes 0.2M-1.5M, degree 8-32)
    for quick runs."""
    specs = []
    for i in range(n_mosaic):
        r = np.random.default_rng(seed0 + i)
        if full:
            rows = int(np.exp(r.uniform(np.log(10_000), np.log(500_000))))
            cols = int(np.exp(r.uniform(np.log(1_000), np.log(20_000))))
            rows = int(min(rows, 2.4e9 / cols))
        else:
            rows, cols = int(r.integers(10_000, 60_001)), int(r.integers(1_000, 10_001))
        specs.append(dict(kind="mosaic", seed=seed0 + i, rows=rows, cols=cols, founders=int(2 ** r.uniform(4, 10)),
                          switch=float(10 ** r.uniform(-3, np.log10(5e-2))), mutation=1e-3))
    for i in range(n_graph):
        seed = seed0 + n_mosaic + i
        r = np.random.default_rng(seed)
        nodes = (int(np.exp(r.uniform(np.log(1_000_000), np.log(16_777_216)))) if full
                 else int(r.integers(200_000, 1_500_001)))
        degree = int(r.integers(8, 65)) if full else int(r.integers(8, 33))
        # every other graph weighted (U{1..100} weights, as for (min,+)), the
        # others plain adjacency (as for (OR,AND)): their terminals differ
        # in kind (one per (weight, column) against one per column)
        specs.append(dict(kind="graph", seed=seed, nodes=nodes, degree=degree, copy=float(r.uniform(0.3, 0.9)),
                          weighted=i % 2 == 0))
    return specs


def make_grammar(spec, threads=0, device=None):
    """Grammar of a corpus spec; device = GPU for the RePair compressor (the
    same grammar as the host compressor)."""
    if spec["kind"] == "mosaic":
        m = gen_mosaic(spec["rows"], spec["cols"], spec["founders"], spec["switch"], spec["mutation"], spec["seed"],
                       threads)
        return repair(m, threads, device=device), spec["rows"], spec["cols"]
    m = gen_copy_graph(spec["nodes"], spec["degree"], spec["copy"], spec.get("weighted", True), spec["seed"], threads)
    return repair(m, threads, device=device), spec["nodes"], spec["nodes"]


def random_inputs(torch, semiring: int, cols: int, B: int, seed: int):
    g = torch.Generator(device="cuda").manual_seed(seed)
    if semiring == 0:
        X = torch.rand((cols, B), device="cuda", generator=g) * 2 - 1
        return X, B
    if semiring == 1:
        W = (B + 31) // 32
        X = torch.randint(0, 2**31 - 1, (cols, W), device="cuda", generator=g, dtype=torch.int32)
        return X, W
    X = torch.randint(0, 1000, (cols, B), device="cuda", generator=g, dtype=torch.int32)
    return X, B


def record(eng: Engine, plan: Plan, semiring: int, B: int, seed: int, reps: int = 3):
    """Autotuner timings of every (launch, variant) -> (inputs, log us, times [slots][V] ms, base features)."""
    import torch

    X, words = random_inputs(torch, semiring, eng.cols, B, seed)
    Y = torch.empty((eng.rows, words), device="cuda", dtype=X.dtype)
    stream = torch.cuda.current_stream().cuda_stream
    times = eng.autotune(semiring, X.data_ptr(), Y.data_ptr(), B, stream=stream, reps=reps)
    base = launch_features(plan, semiring, B)
    return training_rows(base, times) + (times, base)


def training_rows(base: np.ndarray, times: np.ndarray):
    """Model inputs and targets (log us) of every (launch, variant) but the prologue slot's."""
    Xin = model_inputs(base)
    T = np.log(np.maximum(times.reshape(-1), 1e-4) * 1000.0).astype(np.float32)  # ms -> log us
    keep = np.repeat(np.arange(base.shape[0]) >= 1, N_VAR)  # drop the prologue slot
    return Xin[keep], T[keep]


def sweep_time(eng: Engine, semiring: int, B: int, table, seed: int, n: int = 10) -> float:
    """Device time (ms) of one AUTO multiply (CUDA graph) with `table` installed."""
    import torch

    X, words = random_inputs(torch, semiring, eng.cols, B, seed)
    Y = torch.empty((eng.rows, words), device="cuda", dtype=X.dtype)
    st = torch.cuda.current_stream()
    eng.set_level_variants(semiring, B, table)
    for _ in range(3):
        eng.multiply_device(semiring, X.data_ptr(), Y.data_ptr(), B, stream=st.cuda_stream)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(n):
        eng.multiply_device(semiring, X.data_ptr(), Y.data_ptr(), B, stream=st.cuda_stream)
    b.record(st)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / n


def plain_time(eng: Engine, semiring: int, B: int, seed: int, n: int = 5) -> float:
    import torch

    X, words = random_inputs(torch, semiring, eng.cols, B, seed)
    Y = torch.empty((eng.rows, words), device="cuda", dtype=X.dtype)
    st = torch.cuda.current_stream()
    for _ in range(2):
        eng.multiply_device(semiring, X.data_ptr(), Y.data_ptr(), B, stream=st.cuda_stream, variant=1)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(n):
        eng.multiply_device(semiring, X.data_ptr(), Y.data_ptr(), B, stream=st.cuda_stream, variant=1)
    b.record(st)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / n


def run_modes(args, specs, hold, out: Path):
    """Records the autotuner's emission-mode costs on the corpus mosaics at
    (+,x) and the given B, trains the mode model, and evaluates on the
    held-out mosaics: the regret of its chain against the measured best chain
    of pull / interleave, and its gain over pulling every level."""
    import torch

    Bs = [int(b) for b in args.Bs.split(",")]
    tr_X, tr_T, held = [], [], []
    t0 = time.time()
    for gi, spec in enumerate(specs):
        if spec["kind"] != "mosaic":
            continue
        f = out / f"rec_modes_{gi}.npz"
        if f.exists():
            z = np.load(f)
            recs = [(z[f"base{i}"], z[f"costs{i}"], z[f"allowed{i}"]) for i in range(len(z["B"]))]
        else:
            g, rows, cols = make_grammar(spec, device=0)
            plan = Plan.build(g, rows, cols, device=0)
            eng = Engine(plan)
            recs = []
            for B in Bs:
                X, words = random_inputs(torch, 0, cols, B, 1000 * gi + B)
                Y = torch.empty((rows, words), device="cuda", dtype=X.dtype)
                eng.autotune(0, X.data_ptr(), Y.data_ptr(), B, stream=torch.cuda.current_stream().cuda_stream)
                costs = eng.mode_costs(0, B)
                if costs is None:  # no level of this grammar can interleave or push
                    costs = np.full((plan.stats["depth"] + 2, 3, 3), -1.0, np.float32)
                recs.append((launch_features(plan, 0, B), costs, interleave_allowed(plan)))
            arrays = {"B": np.array(Bs)}
            for i, (b, c, a) in enumerate(recs):
                arrays.update({f"base{i}": b, f"costs{i}": c, f"allowed{i}": a})
            np.savez_compressed(f, **arrays)
            del eng
        for base, costs, allowed in recs:
            if gi in hold:
                held.append((base, costs, allowed))
            else:
                x, t = mode_rows(base, costs)
                tr_X.append(x)
                tr_T.append(t)
        print(json.dumps(dict(grammar=gi, held_out=gi in hold, elapsed_s=round(time.time() - t0, 1))), flush=True)
    X, T = np.concatenate(tr_X), np.concatenate(tr_T)
    model = Mlp.create(in_dim=MODE_IN, seed=2)
    mean, std = X.mean(axis=0), X.std(axis=0)
    std[std < 1e-6] = 1.0
    model.set_norm(mean, std)
    loss = model.train(X, T, epochs=args.mode_epochs, batch=256, lr=2e-3, seed=5)
    model.save(out / "mode_model.gmrmlp")
    regrets, gains = [], []
    for base, costs, allowed in held:
        meas = np.where(costs > 0, costs, np.nan)
        if not np.isfinite(meas[:, PULL, PULL][1:]).all():
            continue
        _, t_best = best_chain(meas, allowed)
        pred = np.full(costs.shape, np.nan)
        for mp in (PULL, INTERLEAVE):
            for m in (PULL, INTERLEAVE):
                pred[:, mp, m] = np.exp(model.predict(mode_inputs(base, mp, m)))
        modes, _ = best_chain(pred, allowed)
        t_pick = sum(meas[k][modes[k - 1]][modes[k]] for k in range(1, len(modes)))
        if not np.isfinite(t_pick):  # a pair the autotuner did not measure: count it as pulling
            modes = [PULL] * len(modes)
            t_pick = np.nansum(meas[1:, PULL, PULL])
        t_pull = np.nansum(meas[1:, PULL, PULL])
        regrets.append(t_pick / t_best - 1.0)
        gains.append(t_pull / t_pick)
    report = dict(train_rows=int(len(X)), train_mse=loss, heldout_cases=len(regrets),
                  regret_mean=float(np.mean(regrets)) if regrets else None,
                  regret_p90=float(np.percentile(regrets, 90)) if regrets else None,
                  gain_vs_all_pull_mean=float(np.mean(gains)) if gains else None,
                  record_s=round(time.time() - t0, 1), Bs=Bs, domain=MODE_DOMAIN)
    (out / "mode_report.json").write_text(json.dumps(report, indent=1))
    print(json.dumps(report), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--mosaic", type=int, default=36)
    ap.add_argument("--graph", type=int, default=12)
    ap.add_argument("--holdout", type=float, default=0.25)
    ap.add_argument("--Bs", default="1,8,32,128")
    ap.add_argument("--epochs", type=int, default=80)
    ap.add_argument("--seed", type=int, default=1, help="initialisation seed of the variant model")
    ap.add_argument("--small", action="store_true", help="the earlier small size ranges")
    ap.add_argument("--modes", action="store_true",
                    help="record the emission-mode costs of the corpus mosaics at (+,x) and --Bs, and train the mode "
                         "model instead of the variant model")
    ap.add_argument("--mode-epochs", type=int, default=300)
    ap.add_argument("--resume", default=None,
                    help="a directory holding rec_<grammar>.npz files of an earlier run: those grammars are loaded, "
                         "not recorded again")
    args = ap.parse_args()
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    Bs = [int(b) for b in args.Bs.split(",")]
    specs = corpus_specs(args.mosaic, args.graph, full=not args.small)
    rng = np.random.default_rng(7)
    order = rng.permutation(len(specs))
    n_hold = int(round(len(specs) * args.holdout))
    hold = set(order[:n_hold].tolist())
    if args.modes:
        return run_modes(args, specs, hold, out)
    rows_tr, rows_te = [], []
    t0 = time.time()
    for gi, spec in enumerate(specs):
        # each grammar's records are saved as they are made (rec_<gi>.npz), so
        # that a run cut short can be resumed from its output directory
        done = [Path(d) / f"rec_{gi}.npz" for d in (args.resume, out) if d]
        done = [f for f in done if f.exists()]
        if done:
            z = np.load(done[0], allow_pickle=False)
            recs = []
            for i in range(len(z["sr"])):
                base = z[f"base{i}"]
                if base.shape[1] == N_BASE - 1:  # recorded before the in-place-terminals feature
                    if spec["kind"] != "mosaic":
                        raise SystemExit(f"rec_{gi}: a graph recorded without the in-place-terminals feature")
                    base = np.concatenate([base, np.zeros((base.shape[0], 1), np.float32)], axis=1)
                Xin, T = training_rows(base, z[f"times{i}"])
                recs.append(dict(g=gi, sr=int(z["sr"][i]), B=int(z["B"][i]), X=Xin, T=T, times=z[f"times{i}"]))
            info = dict(grammar=gi, loaded=str(done[0]))
        else:
            g, rows, cols = make_grammar(spec, device=0)
            plan = Plan.build(g, rows, cols, device=0)
            eng = Engine(plan)
            recs = []
            for sr in (0, 1, 2):
                for B in Bs:
                    seed = 1000 * gi + 10 * sr + B
                    Xin, T, times, base = record(eng, plan, sr, B, seed)
                    recs.append(dict(g=gi, sr=sr, B=B, X=Xin, T=T, times=times, base=base))
            arrays = {"sr": np.array([r["sr"] for r in recs]), "B": np.array([r["B"] for r in recs])}
            for i, r in enumerate(recs):
                arrays.update({f"base{i}": r["base"], f"times{i}": r["times"]})
            np.savez_compressed(out / f"rec_{gi}.npz", **arrays)
            info = dict(grammar=gi, spec=spec, ops=plan.stats["n_ops"], depth=plan.stats["depth"])
            del eng
        (rows_te if gi in hold else rows_tr).extend(recs)
        print(json.dumps(info | dict(held_out=gi in hold, elapsed_s=round(time.time() - t0, 1))), flush=True)
    Xtr = np.concatenate([r["X"] for r in rows_tr])
    Ttr = np.concatenate([r["T"] for r in rows_tr])
    model = Mlp.create(seed=args.seed)
    mean, std = Xtr.mean(axis=0), Xtr.std(axis=0)
    std[std < 1e-6] = 1.0
    model.set_norm(mean, std)
    t1 = time.time()
    loss = model.train(Xtr, Ttr, epochs=args.epochs, batch=512, lr=2e-3, seed=3)
    train_s = time.time() - t1
    model.save(out / "cost_model.gmrmlp")
    # held-out regret: predicted choice vs measured best, on the measured times
    regrets, default_gain, wins = [], [], 0
    for r in rows_te:
        times = r["times"][1:]                      # [slots-1][V] ms
        pred = model.predict(r["X"]).reshape(times.shape)
        pick = pred.argmin(axis=1)
        t_learn = times[np.arange(len(pick)), pick].sum()
        t_best = times.min(axis=1).sum()
        t_default = times[:, 0].sum()
        regrets.append(t_learn / t_best - 1.0)
        default_gain.append(t_default / t_learn)
        wins += t_learn <= t_default
    te_loss = float(np.mean((model.predict(np.concatenate([r["X"] for r in rows_te])) -
                             np.concatenate([r["T"] for r in rows_te])) ** 2))
    report = dict(grammars=len(specs), train_grammars=len(specs) - n_hold, heldout_grammars=n_hold,
                  train_rows=int(len(Xtr)), train_mse=loss, heldout_mse=te_loss, train_s=round(train_s, 2),
                  regret_mean=float(np.mean(regrets)), regret_median=float(np.median(regrets)),
                  regret_p90=float(np.percentile(regrets, 90)), within_10pct=float(np.mean(np.array(regrets) <= 0.10)),
                  gain_vs_default_mean=float(np.mean(default_gain)), learned_not_slower_than_default=wins / len(rows_te),
                  cases=len(rows_te), record_s=round(t1 - t0, 1))
    (out / "report.json").write_text(json.dumps(report, indent=1))
    print(json.dumps(report), flush=True)


if __name__ == "__main__":
    main()
