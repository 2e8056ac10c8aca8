"""CUDA engine (libgmr.so, through the C-ABI) against the oracle.

Tolerances: (+,x) fp32 results are compared with an FP64 oracle sweep on
float32-rounded values V, as relative max-norm ||y - y64||_inf / ||y64||_inf
<= 1e-5; (OR,AND) and (min,+) results must be bit-exact against the oracle's
restatement of the reference's int sweep (gpu_engine_test.cu:49-104)."""
import os

import numpy as np
import pytest

import gmr
from helpers import INF, SEMIRINGS, brute_left, golden_cases, golden_meta, interp_left, load_case
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-5
VARIANTS = {"plain": gmr.VARIANT_PLAIN, "fused": gmr.VARIANT_FUSED, "graph": gmr.VARIANT_GRAPH}


def relmax(y, ref):
    ref = np.asarray(ref, dtype=np.float64)
    den = max(np.abs(ref).max(initial=0.0), 1e-30)
    return float(np.abs(np.asarray(y, dtype=np.float64) - ref).max(initial=0.0) / den)


def random_X(sr, cols, B, seed):
    rng = np.random.default_rng(seed)
    if sr == 0:
        return rng.uniform(-1, 1, (cols, B)).astype(np.float32)
    if sr == 1:
        return (rng.random((cols, B)) < 0.3).astype(np.float32)
    X = rng.integers(0, 1000, (cols, B)).astype(np.float32)
    X[rng.random((cols, B)) < 0.2] = 1e9
    return X


def engine_inputs(sr, X):
    """float host matrix -> the engine's input words."""
    if sr == 0:
        return X.astype(np.float32)
    if sr == 1:
        return gmr.pack_bits(X)
    return np.where(X >= INF, np.int32(2**31 - 1), X).astype(np.int32)  # INT_MAX = +inf


def engine_outputs(sr, Y, B):
    return gmr.unpack_bits(Y, B) if sr == 1 else Y


def oracle_columns(sched, sr, V, X, rows, cols):
    out = []
    for b in range(X.shape[1]):
        if sr == 0:
            out.append(sched.sweep_f64(0, V.astype(np.float32).astype(np.float64), X[:, b], rows, cols))
        else:
            out.append(sched.cpu_reference(sr, V.astype(np.float32), X[:, b], rows, cols, threads=1))
    return np.stack(out, axis=1)


def check(sr, Y, ref):
    if sr == 0:
        assert relmax(Y, ref) <= TOL, relmax(Y, ref)
    else:
        np.testing.assert_array_equal(np.asarray(Y, dtype=np.int64), np.asarray(ref, dtype=np.int64))


@pytest.fixture(params=golden_cases())
def case(request):
    c = load_case(request.param)
    g = gmr.Grammar.from_arrays(int(c["alpha"]), c["rules"], c["C"], c["V"])
    c["plan"] = gmr.Plan.build(g, int(c["rows"]), int(c["cols"]))
    c["sched"] = O.RefSchedule(int(c["alpha"]), c["rules"], c["C"])
    return c


@pytest.mark.parametrize("sr", range(3))
@pytest.mark.parametrize("variant", list(VARIANTS))
def test_golden_single_vector(case, sr, variant):
    """B = 1 against the reference's own stored outputs."""
    name = SEMIRINGS[sr]
    eng = gmr.Engine(case["plan"])
    x = case[f"x_{name}"].reshape(-1, 1)
    Y = engine_outputs(sr, eng.multiply(engine_inputs(sr, x), sr, B=1, variant=VARIANTS[variant]), 1)[:, 0]
    if sr == 0:
        ref = case["sched"].sweep_f64(0, case["V"].astype(np.float32).astype(np.float64), x[:, 0],
                                      int(case["rows"]), int(case["cols"]))
        check(0, Y, ref)
        assert relmax(Y, case["y64_plustimes"]) <= 1e-5
    else:
        check(sr, Y, case[f"y32_{name}"])  # the reference's int sweep, bit for bit
    assert eng.last_launches > 0


CONFIGS = [
    dict(variant=gmr.VARIANT_PLAIN),                                       # reference scheme
    dict(variant=gmr.VARIANT_GRAPH),                                       # engine default
    dict(variant=gmr.VARIANT_FUSED, emit_mode=gmr.EMIT_SEGMENTED),
    dict(variant=gmr.VARIANT_FUSED, emit_mode=gmr.EMIT_ATOMIC, vec_tile=2),
    dict(variant=gmr.VARIANT_GRAPH, emit_mode=gmr.EMIT_ROWS, vec_tile=4, tile_levels=2),
    dict(variant=gmr.VARIANT_GRAPH, emit_mode=gmr.EMIT_SEGMENTED, vec_tile=8, ops_per_cta=5),
    dict(variant=gmr.VARIANT_PERSISTENT),                                  # one cooperative launch
    dict(variant=gmr.VARIANT_PERSISTENT, emit_mode=gmr.EMIT_ROWS),
    dict(variant=gmr.VARIANT_GRAPH, push=gmr.PUSH_ALWAYS),                 # rules push their emissions
    dict(variant=gmr.VARIANT_FUSED, push=gmr.PUSH_ALWAYS, emit_mode=gmr.EMIT_ROWS, vec_tile=4, tile_levels=2),
    dict(variant=gmr.VARIANT_FUSED, push=gmr.PUSH_ALWAYS, emit_mode=gmr.EMIT_ATOMIC),
    # 32-byte lane accesses (8 words per lane) where the tile allows them
    dict(variant=gmr.VARIANT_GRAPH, lane_bytes=32),
    dict(variant=gmr.VARIANT_PERSISTENT, lane_bytes=32),
    dict(variant=gmr.VARIANT_FUSED, lane_bytes=32, emit_mode=gmr.EMIT_ROWS, vec_tile=8, tile_levels=2),
    dict(variant=gmr.VARIANT_FUSED, lane_bytes=32, emit_mode=gmr.EMIT_ATOMIC, vec_tile=16),
    dict(variant=gmr.VARIANT_GRAPH, lane_bytes=32, push=gmr.PUSH_ALWAYS, emit_mode=gmr.EMIT_SEGMENTED,
         ops_per_cta=5),
]


@pytest.mark.parametrize("sr", range(3))
@pytest.mark.parametrize("B", [2, 3, 8, 32, 33, 64, 128, 256])
def test_golden_batched(case, sr, B):
    rows, cols = int(case["rows"]), int(case["cols"])
    X = random_X(sr, cols, B, 100 + B)
    ref = oracle_columns(case["sched"], sr, case["V"], X, rows, cols)
    eng = gmr.Engine(case["plan"])
    for cfg in CONFIGS:
        Y = engine_outputs(sr, eng.multiply(engine_inputs(sr, X), sr, B=B, **cfg), B)
        check(sr, Y, ref)


@pytest.mark.parametrize("sr", [0, 2])
@pytest.mark.parametrize("B", [8, 32, 128])
def test_wide_lanes_every_level_table(case, sr, B, monkeypatch):
    """32-byte lane accesses as the engine default (GMR_LANE_BYTES=32):
    every per-launch table (folds, grids, source chunks, push, interleave)
    matches the oracle."""
    monkeypatch.setenv("GMR_LANE_BYTES", "32")
    monkeypatch.setenv("GMR_CHUNK_SLOTS", "5")
    rows, cols = int(case["rows"]), int(case["cols"])
    X = random_X(sr, cols, B, 700 + B)
    ref = oracle_columns(case["sched"], sr, case["V"], X, rows, cols)
    eng = gmr.Engine(case["plan"])
    Xw = engine_inputs(sr, X)
    for table in ([v] * (eng.depth + 2) for v in (0, 3, 4, 10, 13, 32, 35, 45, 64, 67, 77, 128, 133, 138, 192)):
        eng.set_level_variants(sr, B, table)
        check(sr, eng.multiply(Xw, sr, B=B), ref)
    eng.set_level_variants(sr, B, None)
    check(sr, eng.multiply(Xw, sr, B=B, variant=gmr.VARIANT_PERSISTENT), ref)


@pytest.fixture(scope="module")
def staging_grammar():
    rows, cols = 12000, 2500
    m = gmr.gen_mosaic(rows, cols, 48, 0.01, 0.001, 41, threads=4)
    g = gmr.repair(m, 4)
    plan = gmr.Plan.build(g, rows, cols)
    return dict(plan=plan, sched=O.RefSchedule(g.alpha, g.rules(), g.C()), V=g.values(), rows=rows, cols=cols)


@pytest.mark.parametrize("sr,B", [(0, 32), (0, 128), (0, 8), (1, 256), (2, 64), (2, 4)])
def test_staged_left_child_windows(staging_grammar, sr, B):
    """GMR_LEVEL_STAGE on every level (left-child windows staged in shared
    memory by bulk copies), with runs whose window fits and runs whose window
    does not (read from global memory): every semiring matches the oracle and
    no staged wait gave up."""
    gd = staging_grammar
    plan = gd["plan"]
    words = B if sr != 1 else (B + 31) // 32
    if words * 4 >= 128:  # values of 128 bytes or more: some runs' windows exceed the stage
        lanes = words // (8 if sr == 0 and words >= 32 else 4)  # lanes per rule at the default lane width
        assert plan.window_stats(2 * (256 // lanes), words)[:, 0].min() < 1.0
    X = random_X(sr, gd["cols"], B, 900 + B)
    ref = oracle_columns(gd["sched"], sr, gd["V"], X, gd["rows"], gd["cols"])
    eng = gmr.Engine(plan)
    Xw = engine_inputs(sr, X)
    for v in (0, 2, 13):
        eng.set_level_variants(sr, B, [v | 128] * (eng.depth + 2))
        check(sr, engine_outputs(sr, eng.multiply(Xw, sr, B=B), B), ref)  # AUTO: the installed table
        assert eng.status() == (0, 0)


@pytest.mark.parametrize("sr", range(3))
@pytest.mark.parametrize("B", [1, 5, 32, 40])
def test_direct_terminal_emissions(case, sr, B, monkeypatch):
    """Terminal emissions folded as leaf(V, X[col]) straight from X (the mode
    the engine picks when the terminal table dwarfs X), forced on: every
    variant, the per-launch tables (chunked ones included) and the
    persistent kernel still match the oracle."""
    monkeypatch.setenv("GMR_DIRECT_TERMS", "1")
    monkeypatch.setenv("GMR_CHUNK_SLOTS", "5")  # several source chunks per level: interleaving applies
    rows, cols = int(case["rows"]), int(case["cols"])
    X = random_X(sr, cols, B, 500 + B)
    ref = oracle_columns(case["sched"], sr, case["V"], X, rows, cols)
    eng = gmr.Engine(case["plan"])
    Xw = engine_inputs(sr, X)
    for cfg in CONFIGS:
        check(sr, engine_outputs(sr, eng.multiply(Xw, sr, B=B, **cfg), B), ref)
    rng = np.random.default_rng(B)
    for table in ([v] * (eng.depth + 2) for v in (0, 3, 4, 10, 13, 32, 35, 45, 64, 67, 77)):
        eng.set_level_variants(sr, B, table)
        check(sr, engine_outputs(sr, eng.multiply(Xw, sr, B=B), B), ref)
    eng.set_level_variants(sr, B, rng.integers(0, eng.N_LEVEL_VARIANTS, eng.depth + 2))
    check(sr, engine_outputs(sr, eng.multiply(Xw, sr, B=B), B), ref)
    eng.set_level_variants(sr, B, rng.integers(0, eng.N_LEVEL_VARIANTS, eng.depth + 2) |
                           (rng.random(eng.depth + 2) < 0.5) * gmr.LEVEL_PUSH)
    check(sr, engine_outputs(sr, eng.multiply(Xw, sr, B=B), B), ref)


@pytest.fixture(scope="module")
def wgraph():
    """Weighted copy graph whose terminal table is over 4x its column count,
    so the engine picks direct terminals by itself."""
    m = gmr.gen_copy_graph(30000, 24, 0.7, True, 21)
    g = gmr.repair(m)
    plan = gmr.Plan.build(g, 30000, 30000)
    assert plan.stats["n_terms"] > 4 * 30000
    return dict(g=g, plan=plan, sched=O.RefSchedule(g.alpha, g.rules(), g.C()), V=g.values())


@pytest.mark.parametrize("sr,B", [(1, 32), (1, 1), (2, 1), (2, 3), (0, 4)])
def test_graph_direct_terminals_auto(wgraph, sr, B):
    X = random_X(sr, 30000, B, 900 + B)
    ref = oracle_columns(wgraph["sched"], sr, wgraph["V"], X, 30000, 30000)
    eng = gmr.Engine(wgraph["plan"])
    for cfg in (dict(variant=gmr.VARIANT_GRAPH), dict(variant=gmr.VARIANT_PLAIN),
                dict(variant=gmr.VARIANT_PERSISTENT)):
        check(sr, engine_outputs(sr, eng.multiply(engine_inputs(sr, X), sr, B=B, **cfg), B), ref)


@pytest.mark.parametrize("sr", range(3))
def test_device_pointers_and_stream(case, sr):
    torch = pytest.importorskip("torch")
    rows, cols, B = int(case["rows"]), int(case["cols"]), 8
    X = random_X(sr, cols, B, 7)
    ref = oracle_columns(case["sched"], sr, case["V"], X, rows, cols)
    Xw = engine_inputs(sr, X)
    dX = torch.from_numpy(Xw.view(np.int32)).cuda()
    dY = torch.empty((rows, Xw.shape[1]), dtype=torch.int32, device="cuda")
    eng = gmr.Engine(case["plan"])
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        for _ in range(3):  # graph replay on a side stream
            eng.multiply_device(sr, dX.data_ptr(), dY.data_ptr(), B, stream=s.cuda_stream)
    s.synchronize()
    Yw = dY.cpu().numpy().view({0: np.float32, 1: np.uint32, 2: np.int32}[sr])
    check(sr, engine_outputs(sr, Yw, B), ref)


@pytest.mark.parametrize("sr", range(3))
def test_legacy_entry_points(case, sr, monkeypatch, capfd):
    """The drop-in pair with the reference's layered schedule and stdout lines."""
    name = SEMIRINGS[sr]
    monkeypatch.setenv("SEMIRING", name)
    s = case["sched"]
    rows, cols = int(case["rows"]), int(case["cols"])
    vi, ci = s.terminal_tables(cols)
    Vf = case["V"].astype(np.float32)
    x = case[f"x_{name}"]
    y = gmr.run_gpu_right_multiply_layered(rows, cols, s.alpha, s.rules_lrc(), vi, ci, Vf, x, s.gpu_schedule(),
                                           iters=3)
    out = capfd.readouterr().out
    assert "GPU kernel: " in out and " ms/vector." in out and "MEM analytic bytes: " in out
    ref = case[f"y32_{name}"]
    check(sr, y, ref if sr else case["sched"].sweep_f64(0, Vf.astype(np.float64), x, rows, cols))
    B = 5
    X = random_X(sr, cols, B, 3)
    Y = gmr.run_gpu_right_multiply_batched(rows, cols, s.alpha, s.rules_lrc(), vi, ci, Vf, X.reshape(-1),
                                           s.gpu_schedule(), B, iters=2)
    assert "GPU batched (B=5): " in capfd.readouterr().out
    check(sr, Y, oracle_columns(s, sr, case["V"], X, rows, cols))


@pytest.mark.parametrize("sr", range(3))
def test_autotuned_and_mixed_tables(case, sr):
    """Every per-launch variant table gives the same results (it only picks schedules)."""
    torch = pytest.importorskip("torch")
    rows, cols, B = int(case["rows"]), int(case["cols"]), 32
    X = random_X(sr, cols, B, 77)
    ref = oracle_columns(case["sched"], sr, case["V"], X, rows, cols)
    eng = gmr.Engine(case["plan"])
    Xw = engine_inputs(sr, X)
    dX = torch.from_numpy(Xw.view(np.int32)).cuda()
    dY = torch.empty((rows, Xw.shape[1]), dtype=torch.int32, device="cuda")
    times = eng.autotune(sr, dX.data_ptr(), dY.data_ptr(), B)
    assert times.shape == (eng.depth + 2, eng.N_LEVEL_VARIANTS) and np.all(times[1:] > 0)
    best = eng.level_variants(sr, B)
    modes = gmr.LEVEL_PUSH | gmr.LEVEL_INTERLEAVE | gmr.LEVEL_STAGE
    assert best is not None and np.array_equal(best[1:] & (255 - modes), times[1:].argmin(axis=1))
    assert not np.any(best[[0, eng.depth + 1]] & modes)  # only levels 1..depth push or interleave
    rng = np.random.default_rng(sr)
    mixed = rng.integers(0, eng.N_LEVEL_VARIANTS, eng.depth + 2) | (rng.random(eng.depth + 2) < 0.5) * gmr.LEVEL_PUSH
    for table in (best, rng.integers(0, eng.N_LEVEL_VARIANTS, eng.depth + 2), mixed):
        eng.set_level_variants(sr, B, table)
        Y = engine_outputs(sr, eng.multiply(Xw, sr, B=B), B)  # AUTO uses the table
        check(sr, Y, ref)
    eng.set_level_variants(sr, B, None)
    assert eng.level_variants(sr, B) is None


@pytest.mark.parametrize("sr", range(3))
def test_energy_aware_autotune(case, sr):
    """With a tolerance, each launch takes the chunked twin of its fastest
    variant when that is within the tolerance; results are unchanged."""
    torch = pytest.importorskip("torch")
    rows, cols, B = int(case["rows"]), int(case["cols"]), 32
    X = random_X(sr, cols, B, 78)
    ref = oracle_columns(case["sched"], sr, case["V"], X, rows, cols)
    eng = gmr.Engine(case["plan"])
    Xw = engine_inputs(sr, X)
    dX = torch.from_numpy(Xw.view(np.int32)).cuda()
    dY = torch.empty((rows, Xw.shape[1]), dtype=torch.int32, device="cuda")
    tol = 0.5
    times = eng.autotune(sr, dX.data_ptr(), dY.data_ptr(), B, energy_tolerance=tol)
    table = eng.level_variants(sr, B)
    for slot in range(1, eng.depth + 2):
        b = int(times[slot].argmin())
        want = b + 10 if b < 10 and times[slot, b + 10] <= times[slot, b] * (1 + tol) else b
        assert table[slot] & (255 - gmr.LEVEL_PUSH - gmr.LEVEL_INTERLEAVE - gmr.LEVEL_STAGE) == want
    check(sr, engine_outputs(sr, eng.multiply(Xw, sr, B=B), B), ref)
    with pytest.raises(gmr.GmrError):
        eng.autotune(sr, dX.data_ptr(), dY.data_ptr(), B, energy_tolerance=1.5)


def test_persistent_barrier_timeout_reports_status(c1):
    """A grid-barrier wait limited to one poll gives up: the host gets
    GMR_ERR_TIMEOUT, and the next multiply on the same context is correct."""
    eng = c1["eng"]
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, (5000, 8)).astype(np.float32)
    timeouts = 0
    for _ in range(3):
        try:
            eng.multiply(x, 0, B=8, variant=gmr.VARIANT_PERSISTENT, spin_limit=1)
        except gmr.GmrError as e:
            assert e.code == 7 and "gave up" in str(e)
            timeouts += 1
    assert timeouts >= 1
    failed, phase = eng.status()
    assert failed in (0, 1)
    y = eng.multiply(x, 0, B=8, variant=gmr.VARIANT_PERSISTENT)
    assert eng.status()[0] == 0
    ref = c1["sched"].sweep_f64(0, c1["V"], x[:, 3], 20000, 5000)
    assert relmax(y[:, 3], ref) <= TOL


def test_packed_multi_grammar_launch():
    """Eight uneven grammars, each with its own semiring and B, in one graph launch."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(10)
    engines, scheds, args = [], [], []
    for i in range(8):
        rows, cols = int(rng.integers(300, 3000)), int(rng.integers(64, 700))
        m = gmr.gen_mosaic(rows, cols, 16, 0.02, 0.002, 10 + i, threads=4)
        g = gmr.repair(m, 4)
        engines.append(gmr.Engine(gmr.Plan.build(g, rows, cols)))
        scheds.append((O.RefSchedule(g.alpha, g.rules(), g.C()), g.values(), rows, cols))
        sr, B = i % 3, [1, 4, 16, 64][i % 4]
        X = random_X(sr, cols, B, 50 + i)
        Xw = engine_inputs(sr, X)
        dX = torch.from_numpy(Xw.view(np.int32)).cuda()
        dY = torch.zeros((rows, Xw.shape[1]), dtype=torch.int32, device="cuda")
        args.append((sr, B, X, dX, dY))
    pack = gmr.Pack(engines)
    for _ in range(2):  # capture, then replay
        pack.multiply_device([a[0] for a in args], [a[3].data_ptr() for a in args], [a[4].data_ptr() for a in args],
                             [a[1] for a in args], stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert pack.last_launches >= 8 * 3
    assert pack.status()[0] is False  # mixed semirings: the graph of per-engine branches
    for (sched, V, rows, cols), (sr, B, X, dX, dY) in zip(scheds, args):
        Yw = dY.cpu().numpy().view({0: np.float32, 1: np.uint32, 2: np.int32}[sr])
        check(sr, engine_outputs(sr, Yw, B), oracle_columns(sched, sr, V, X, rows, cols))


PACK_WIDTHS = {0: [1, 3, 4, 16, 33, 64, 2, 8], 1: [1, 40, 64, 128, 200, 32, 7, 96], 2: [1, 3, 4, 16, 33, 64, 2, 8]}


@pytest.fixture(scope="module")
def pack_grammars():
    rng = np.random.default_rng(12)
    out = []
    for i in range(8):
        rows, cols = int(rng.integers(200, 4000)), int(rng.integers(64, 900))
        m = gmr.gen_mosaic(rows, cols, 16, 0.02, 0.002, 30 + i, threads=4)
        g = gmr.repair(m, 4)
        out.append(dict(plan=gmr.Plan.build(g, rows, cols), sched=O.RefSchedule(g.alpha, g.rules(), g.C()),
                        V=g.values(), rows=rows, cols=cols))
    return out


@pytest.mark.parametrize("sr", range(3))
def test_packed_persistent_kernel(pack_grammars, sr):
    """Eight uneven grammars in ONE persistent launch, and in one launch per
    level over all of them (one semiring, each its own B, so every lane layout
    of the kernels' grammar table is used)."""
    torch = pytest.importorskip("torch")
    engines, args = [], []
    for i, gd in enumerate(pack_grammars):
        engines.append(gmr.Engine(gd["plan"]))
        B = PACK_WIDTHS[sr][i]
        X = random_X(sr, gd["cols"], B, 70 + i)
        Xw = engine_inputs(sr, X)
        dX = torch.from_numpy(Xw.view(np.int32)).cuda()
        dY = torch.full((gd["rows"], Xw.shape[1]), 7, dtype=torch.int32, device="cuda")
        args.append((B, X, dX, dY))
    pack = gmr.Pack(engines)
    st = torch.cuda.current_stream().cuda_stream
    max_depth = max(e.depth for e in engines)
    for mode in (gmr.Pack.PERSISTENT, gmr.Pack.LEVELS):
        pack.set_mode(mode)
        for _ in range(2):  # table upload (and capture), then reuse
            for a in args:
                a[3].fill_(7)
            pack.multiply_device([sr] * 8, [a[2].data_ptr() for a in args], [a[3].data_ptr() for a in args],
                                 [a[0] for a in args], stream=st)
            torch.cuda.synchronize()
            if mode == gmr.Pack.PERSISTENT:
                assert pack.status() == (True, 0, 0) and pack.last_launches == 1
            else:
                assert pack.status()[0] is False and pack.last_launches == max_depth + 2
            for gd, (B, X, dX, dY) in zip(pack_grammars, args):
                Yw = dY.cpu().numpy().view({0: np.float32, 1: np.uint32, 2: np.int32}[sr])
                check(sr, engine_outputs(sr, Yw, B), oracle_columns(gd["sched"], sr, gd["V"], X, gd["rows"],
                                                                    gd["cols"]))
    pack.set_mode(gmr.Pack.GRAPH)  # the same call as a graph of branches
    pack.multiply_device([sr] * 8, [a[2].data_ptr() for a in args], [a[3].data_ptr() for a in args],
                         [a[0] for a in args], stream=st)
    torch.cuda.synchronize()
    assert pack.status()[0] is False


def test_packed_persistent_barrier_timeout(pack_grammars):
    """A barrier wait limited to one poll gives up and is reported; the next
    call with the normal limit is correct again."""
    torch = pytest.importorskip("torch")
    engines = [gmr.Engine(gd["plan"]) for gd in pack_grammars]
    B = 8
    Xs = [random_X(0, gd["cols"], B, 90 + i) for i, gd in enumerate(pack_grammars)]
    dXs = [torch.from_numpy(x).cuda() for x in Xs]
    dYs = [torch.zeros((gd["rows"], B), dtype=torch.float32, device="cuda") for gd in pack_grammars]
    pack = gmr.Pack(engines)
    st = torch.cuda.current_stream().cuda_stream
    call = lambda: pack.multiply_device([0] * 8, [x.data_ptr() for x in dXs], [y.data_ptr() for y in dYs],
                                        [B] * 8, stream=st)
    pack.set_mode(gmr.Pack.PERSISTENT, spin_limit=1)
    failures = 0
    for _ in range(3):
        call()
        torch.cuda.synchronize()
        ran, failed, phase = pack.status()
        assert ran
        failures += failed != 0
    assert failures >= 1
    pack.set_mode(gmr.Pack.PERSISTENT)
    call()
    torch.cuda.synchronize()
    assert pack.status() == (True, 0, 0)
    for gd, X, dY in zip(pack_grammars, Xs, dYs):
        check(0, dY.cpu().numpy(), oracle_columns(gd["sched"], 0, gd["V"], X, gd["rows"], gd["cols"]))


@pytest.mark.parametrize("sr", range(3))
def test_chunked_emission_passes(case, sr, monkeypatch):
    """Folding emissions one source chunk at a time (tiny chunks here, so every
    level has several) gives the same results in every emission mode."""
    monkeypatch.setenv("GMR_CHUNK_SLOTS", "7")
    eng = gmr.Engine(case["plan"])
    monkeypatch.delenv("GMR_CHUNK_SLOTS")
    rows, cols = int(case["rows"]), int(case["cols"])
    for B in (1, 32):
        X = random_X(sr, cols, B, 300 + B)
        ref = oracle_columns(case["sched"], sr, case["V"], X, rows, cols)
        # chunked: segmented 16 / 32, row-owned, atomic; 4 CTAs per SM; pushed; interleaved
        for v in (10, 12, 13, 14, 17, 42, 45, 64, 67, 68, 74, 77, 3 + 64):
            eng.set_level_variants(sr, B, np.full(eng.depth + 2, v, dtype=np.uint8))
            Y = engine_outputs(sr, eng.multiply(engine_inputs(sr, X), sr, B=B), B)
            check(sr, Y, ref)
        rng = np.random.default_rng(sr + B)
        for _ in range(3):  # mixed pull / push / interleave chains
            modes = rng.choice([0, gmr.LEVEL_PUSH, gmr.LEVEL_INTERLEAVE], eng.depth + 2)
            eng.set_level_variants(sr, B, rng.integers(0, eng.N_LEVEL_VARIANTS, eng.depth + 2) | modes)
            check(sr, engine_outputs(sr, eng.multiply(engine_inputs(sr, X), sr, B=B), B), ref)
        eng.set_level_variants(sr, B, None)
        for cfg in (dict(push=gmr.PUSH_INTERLEAVE), dict(push=gmr.PUSH_INTERLEAVE, emit_mode=gmr.EMIT_ROWS),
                    dict(push=gmr.PUSH_INTERLEAVE, variant=gmr.VARIANT_FUSED, emit_mode=gmr.EMIT_ATOMIC)):
            check(sr, engine_outputs(sr, eng.multiply(engine_inputs(sr, X), sr, B=B, **cfg), B), ref)
    # the autotuner's chain of pull / push / interleave choices keeps the results
    torch = pytest.importorskip("torch")
    B = 32
    X = random_X(sr, cols, B, 333)
    Xw = engine_inputs(sr, X)
    dX = torch.from_numpy(Xw.view(np.int32)).cuda()
    dY = torch.empty((rows, Xw.shape[1]), dtype=torch.int32, device="cuda")
    eng.autotune(sr, dX.data_ptr(), dY.data_ptr(), B)
    check(sr, engine_outputs(sr, eng.multiply(Xw, sr, B=B), B), oracle_columns(case["sched"], sr, case["V"], X,
                                                                               rows, cols))


def test_allocation_failure_is_reported():
    """A batch whose scratch cannot be allocated returns GMR_ERR_OOM (nothing is
    launched) and the engine keeps working for a normal batch afterwards."""
    torch = pytest.importorskip("torch")
    c = load_case("mosaic_300x64")
    g = gmr.Grammar.from_arrays(int(c["alpha"]), c["rules"], c["C"], c["V"])
    plan = gmr.Plan.build(g, 300, 64)
    eng = gmr.Engine(plan)
    s = plan.stats
    huge_B = 1 << 28
    assert (s["n_ops"] + s["n_terms"]) * huge_B * 4 > 600e9  # beyond the device's memory (288 GB)
    x = torch.zeros(16, dtype=torch.float32, device="cuda")
    with pytest.raises(gmr.GmrError) as e:
        eng.multiply_device(0, x.data_ptr(), x.data_ptr(), huge_B)
    assert e.value.code == 5 and "cudaMalloc" in str(e.value)
    sched = O.RefSchedule(int(c["alpha"]), c["rules"], c["C"])
    X = random_X(0, 64, 4, 1)
    check(0, eng.multiply(X, 0, B=4), oracle_columns(sched, 0, c["V"], X, 300, 64))


@pytest.mark.parametrize("name,sr", [("graph_400", 1), ("graph_w300", 2), ("graph_400", 2)])
def test_fixpoint_reachability_and_distances(name, sr):
    """x <- x (+) M x to the fixpoint on the device == the same iteration with the
    oracle's restatement of the reference sweep, bit for bit."""
    torch = pytest.importorskip("torch")
    c = load_case(name)
    n = int(c["rows"])
    g = gmr.Grammar.from_arrays(int(c["alpha"]), c["rules"], c["C"], c["V"])
    eng = gmr.Engine(gmr.Plan.build(g, n, n))
    sched = O.RefSchedule(int(c["alpha"]), c["rules"], c["C"])
    rng = np.random.default_rng(sr)
    B = 40 if sr == 1 else 3
    if sr == 1:
        X = (rng.random((n, B)) < 0.01).astype(np.float32)
    else:
        X = np.full((n, B), 1e9, dtype=np.float32)
        X[rng.random((n, B)) < 0.01] = 0.0
    ref = X.copy()
    iters_ref = 0
    while True:
        iters_ref += 1
        Y = oracle_columns(sched, sr, c["V"], ref, n, n)
        new = np.maximum(ref, Y) if sr == 1 else np.minimum(ref, Y)
        if np.array_equal(new, ref):
            break
        ref = new
    Xw = engine_inputs(sr, X) if sr == 1 else X.astype(np.int32)  # +inf as 1e9, like the oracle
    dX = torch.from_numpy(Xw.view(np.int32)).cuda()
    dY = torch.empty_like(dX)
    it = eng.fixpoint_device(sr, dX.data_ptr(), dY.data_ptr(), B)
    out = engine_outputs(sr, dX.cpu().numpy().view(np.uint32 if sr == 1 else np.int32), B)
    assert it == iters_ref
    check(sr, out, ref)


@pytest.mark.parametrize("sr", range(3))
@pytest.mark.parametrize("n", [0, 1, 5])
def test_pipelined_host_multiplies(case, sr, n):
    """gmr_engine_multiply_host_many: every hY[i] equals its own multiply."""
    torch = pytest.importorskip("torch")
    rows, cols, B = int(case["rows"]), int(case["cols"]), 33
    eng = gmr.Engine(case["plan"])
    Xs = [engine_inputs(sr, random_X(sr, cols, B, 300 + i)) for i in range(n)]
    Xp = [torch.from_numpy(x.view(np.int32)).pin_memory() for x in Xs]
    Yp = [torch.zeros((rows, x.shape[1]), dtype=torch.int32).pin_memory() for x in Xs]
    eng.multiply_host_many(sr, [x.data_ptr() for x in Xp], [y.data_ptr() for y in Yp], B)
    for i in range(n):
        want = eng.multiply(Xs[i], sr, B=B)
        got = Yp[i].numpy().view(want.dtype)
        if sr == 0:
            assert np.max(np.abs(got - want)) <= 1e-5 * max(1.0, float(np.max(np.abs(want))))
        else:
            np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("sr", [1, 2])
def test_fixpoint_with_staged_levels(sr):
    """The fixpoint loop over multiplies whose levels stage their left-child
    windows in shared memory (GMR_LEVEL_STAGE installed for this (semiring,
    B)): the staged launches' error words do not disturb the loop's change
    flag and iteration count, and the result is the oracle's, bit for bit."""
    torch = pytest.importorskip("torch")
    c = load_case("graph_400" if sr == 1 else "graph_w300")
    n = int(c["rows"])
    g = gmr.Grammar.from_arrays(int(c["alpha"]), c["rules"], c["C"], c["V"])
    eng = gmr.Engine(gmr.Plan.build(g, n, n))
    sched = O.RefSchedule(int(c["alpha"]), c["rules"], c["C"])
    rng = np.random.default_rng(9)
    B = 128 if sr == 1 else 4  # 4 words per slot: 16-byte lanes, so staging applies
    if sr == 1:
        X = (rng.random((n, B)) < 0.01).astype(np.float32)
    else:
        X = np.full((n, B), 1e9, dtype=np.float32)
        X[rng.random((n, B)) < 0.01] = 0.0
    ref, iters_ref = X.copy(), 0
    while True:
        iters_ref += 1
        Y = oracle_columns(sched, sr, c["V"], ref, n, n)
        new = np.maximum(ref, Y) if sr == 1 else np.minimum(ref, Y)
        if np.array_equal(new, ref):
            break
        ref = new
    eng.set_level_variants(sr, B, [128] * (eng.depth + 2))
    Xw = engine_inputs(sr, X) if sr == 1 else X.astype(np.int32)
    dX = torch.from_numpy(Xw.view(np.int32).copy()).cuda()
    dY = torch.empty_like(dX)
    assert eng.fixpoint_device(sr, dX.data_ptr(), dY.data_ptr(), B) == iters_ref
    check(sr, engine_outputs(sr, dX.cpu().numpy().view(np.uint32 if sr == 1 else np.int32), B), ref)
    assert eng.status() == (0, 0)


@pytest.mark.parametrize("sr", [1, 2])
def test_fixpoint_iteration_limit_and_repeat(sr):
    """max_iters caps the device-side loop (0 runs nothing, 1 runs one merge);
    a second call on the same buffers replays the cached loop graph."""
    torch = pytest.importorskip("torch")
    c = load_case("graph_400" if sr == 1 else "graph_w300")
    n = int(c["rows"])
    g = gmr.Grammar.from_arrays(int(c["alpha"]), c["rules"], c["C"], c["V"])
    eng = gmr.Engine(gmr.Plan.build(g, n, n))
    sched = O.RefSchedule(int(c["alpha"]), c["rules"], c["C"])
    rng = np.random.default_rng(5)
    B = 32 if sr == 1 else 2
    if sr == 1:
        X = (rng.random((n, B)) < 0.01).astype(np.float32)
    else:
        X = np.full((n, B), 1e9, dtype=np.float32)
        X[rng.random((n, B)) < 0.01] = 0.0
    Xw = engine_inputs(sr, X) if sr == 1 else X.astype(np.int32)
    dX = torch.from_numpy(Xw.view(np.int32).copy()).cuda()
    dY = torch.empty_like(dX)
    assert eng.fixpoint_device(sr, dX.data_ptr(), dY.data_ptr(), B, max_iters=0) == 0
    np.testing.assert_array_equal(dX.cpu().numpy(), Xw.view(np.int32))
    assert eng.fixpoint_device(sr, dX.data_ptr(), dY.data_ptr(), B, max_iters=1) == 1
    Y = oracle_columns(sched, sr, c["V"], X, n, n)
    one = np.maximum(X, Y) if sr == 1 else np.minimum(X, Y)
    out = engine_outputs(sr, dX.cpu().numpy().view(np.uint32 if sr == 1 else np.int32), B)
    check(sr, out, one)
    total = 1
    for _ in range(200):
        it = eng.fixpoint_device(sr, dX.data_ptr(), dY.data_ptr(), B, max_iters=2)
        total += it
        if it < 2:
            break
    full = engine_outputs(sr, dX.cpu().numpy().view(np.uint32 if sr == 1 else np.int32), B)
    assert eng.fixpoint_device(sr, dX.data_ptr(), dY.data_ptr(), B) == 1  # at the fixpoint: one idle iteration
    np.testing.assert_array_equal(engine_outputs(sr, dX.cpu().numpy().view(np.uint32 if sr == 1 else np.int32), B),
                                  full)


@pytest.mark.parametrize("sr", range(3))
@pytest.mark.parametrize("B", [1, 8, 33])
def test_left_product(case, sr, B):
    """y = x^T M on the GPU against the brute-force transpose product of the expanded matrix."""
    torch = pytest.importorskip("torch")
    rows, cols = int(case["rows"]), int(case["cols"])
    g = gmr.Grammar.from_arrays(int(case["alpha"]), case["rules"], case["C"], case["V"])
    eng = gmr.Engine(case["plan"])
    eng.enable_left(case["plan"])
    X = random_X(sr, rows, B, 900 + B)
    ref = brute_left(O.expand(g.alpha, g.rules(), g.C()), case["V"].astype(np.float32), X, rows, cols, sr)
    Xw = engine_inputs(sr, X)
    dX = torch.from_numpy(Xw.view(np.int32)).cuda()
    dY = torch.zeros((cols, Xw.shape[1]), dtype=torch.int32, device="cuda")
    for _ in range(2):
        eng.multiply_left_device(sr, dX.data_ptr(), dY.data_ptr(), B)
    torch.cuda.synchronize()
    Y = engine_outputs(sr, dY.cpu().numpy().view({0: np.float32, 1: np.uint32, 2: np.int32}[sr]), B)
    check(sr, Y, ref)


@pytest.fixture(scope="module")
def mosaic_mid():
    m = gmr.gen_mosaic(3000, 700, 16, 0.01, 1e-3, 5)
    g = gmr.repair(m)
    plan = gmr.Plan.build(g, 3000, 700)
    eng = gmr.Engine(plan)
    eng.enable_left(plan)
    codes = O.expand(g.alpha, g.rules(), g.C())
    return dict(g=g, plan=plan, eng=eng, codes=codes)


@pytest.mark.parametrize("sr", range(3))
@pytest.mark.parametrize("B", [1, 32, 40])
def test_left_product_straddling_targets(mosaic_mid, sr, B):
    """3,000 x 700 mosaic: symbols with many parents / rows are folded by
    several lane groups (atomic parts into a zeroed value)."""
    torch = pytest.importorskip("torch")
    c = mosaic_mid
    assert len(c["plan"].array("le_split")) > 100
    X = random_X(sr, 3000, B, 70 + B)
    ref = brute_left(c["codes"], c["g"].values().astype(np.float32), X, 3000, 700, sr)
    Xw = engine_inputs(sr, X)
    dX = torch.from_numpy(Xw.view(np.int32)).cuda()
    dY = torch.zeros((700, Xw.shape[1]), dtype=torch.int32, device="cuda")
    for _ in range(2):
        c["eng"].multiply_left_device(sr, dX.data_ptr(), dY.data_ptr(), B)
    torch.cuda.synchronize()
    Y = engine_outputs(sr, dY.cpu().numpy().view({0: np.float32, 1: np.uint32, 2: np.int32}[sr]), B)
    check(sr, Y, ref)


def test_left_product_runlength():
    """Run-length coefficient on the left child: compared with the FP64
    evaluation of the plan's transpose arrays."""
    torch = pytest.importorskip("torch")
    g = gmr.Grammar.from_arrays(5, [[1, 2], [3, 5], [6, 0], [7, 5]], [8, 0, 6, 0], [1.5, 2.5], kinds=[0, 0, 1, 0],
                                reps=[1, 1, 3, 1])
    plan = gmr.Plan.build(g, 2, 3)
    eng = gmr.Engine(plan)
    eng.enable_left(plan)
    X = np.array([[2.0, 0.5], [-1.0, 3.0]], np.float32)
    dX = torch.from_numpy(X).cuda()
    dY = torch.zeros((3, 2), dtype=torch.float32, device="cuda")
    eng.multiply_left_device(0, dX.data_ptr(), dY.data_ptr(), 2)
    torch.cuda.synchronize()
    np.testing.assert_allclose(dY.cpu().numpy(), interp_left(plan, 0, X), rtol=1e-6)


def test_unittest_grammar_runlength():
    """cpu_selftest.cpp:374-467 grammar (run-length rule, coefficient 3)."""
    g = gmr.Grammar.from_arrays(5, [[1, 2], [3, 5], [6, 0], [7, 5]], [8, 0], [1.5, 2.5], kinds=[0, 0, 1, 0],
                                reps=[1, 1, 3, 1])
    eng = gmr.Engine(gmr.Plan.build(g, 2, 3))
    y = eng.multiply(np.array([0.5, -0.5, 1.0], np.float32), 0)[:, 0]
    np.testing.assert_allclose(y, golden_meta()["unittest"]["y_sweep"], atol=1e-6)
    Y = eng.multiply(np.tile(np.array([[0.5], [-0.5], [1.0]], np.float32), (1, 4)), 0)
    np.testing.assert_allclose(Y, [[4.5] * 4, [0.0] * 4], atol=1e-6)


def test_readme_worked_example():
    c = load_case("readme_8x7")
    g = gmr.Grammar.from_arrays(int(c["alpha"]), c["rules"], c["C"], c["V"])
    eng = gmr.Engine(gmr.Plan.build(g, 8, 7))
    y = eng.multiply(np.array(golden_meta()["readme"]["x"], np.float32), 0)[:, 0]
    np.testing.assert_allclose(y, golden_meta()["readme"]["y"], rtol=1e-6)


def test_terminals_only_and_empty_rows():
    g = gmr.Grammar.from_arrays(4, np.zeros((0, 2), np.int32), [1, 3, 0, 0, 2, 0], [1.0])
    eng = gmr.Engine(gmr.Plan.build(g, 4, 3))
    y = eng.multiply(np.array([1.0, 2.0, 4.0], np.float32), 0)[:, 0]
    np.testing.assert_allclose(y, [5.0, 0.0, 2.0, 0.0])
    yt = eng.multiply(np.array([[5], [2**31 - 1], [7]], np.int32), 2)[:, 0]
    np.testing.assert_array_equal(yt, [6, INF, INF, INF])


def test_tropical_int_max_is_infinity():
    # row 0: x0 + 1 and x1 + 1 (value 1) ; x1 = INT_MAX -> only x0 counts
    g = gmr.Grammar.from_arrays(3, [[1, 2]], [3, 0, 2, 0], [1.0])
    eng = gmr.Engine(gmr.Plan.build(g, 3, 2))
    y = eng.multiply(np.array([[10], [2**31 - 1]], np.int32), 2)[:, 0]
    np.testing.assert_array_equal(y, [11, INF, INF])


def test_deterministic_boolean_tropical(case):
    rows, cols, B = int(case["rows"]), int(case["cols"]), 64
    eng = gmr.Engine(case["plan"])
    for sr in (1, 2):
        Xw = engine_inputs(sr, random_X(sr, cols, B, 9))
        a = eng.multiply(Xw, sr, B=B)
        b = eng.multiply(Xw, sr, B=B)
        np.testing.assert_array_equal(a, b)


# ---------------------------------------------------------------- C1 at full size
@pytest.fixture(scope="module")
def c1():
    """Config 1: 20,000 x 5,000 mosaic, 64 founders, seed 0."""
    m = gmr.gen_mosaic(20000, 5000, 64, 0.01, 1e-3, 0)
    g = gmr.repair(m)
    plan = gmr.Plan.build(g, 20000, 5000)
    sched = O.RefSchedule(g.alpha, g.rules(), g.C())
    return dict(g=g, plan=plan, sched=sched, V=g.values(), eng=gmr.Engine(plan))


def test_c1_plain_spmv_vs_fp64(c1):
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, 5000).astype(np.float32)
    ref = c1["sched"].sweep_f64(0, c1["V"], x, 20000, 5000)
    for variant in VARIANTS.values():
        y = c1["eng"].multiply(x, 0, variant=variant)[:, 0]
        err = relmax(y, ref)
        print(f"C1 B=1 variant={variant} rel max-norm error vs FP64 = {err:.3e}")
        assert err <= TOL


@pytest.mark.parametrize("B", [8, 32])
def test_c1_batched_vs_fp64(c1, B):
    rng = np.random.default_rng(B)
    X = rng.uniform(-1, 1, (5000, B)).astype(np.float32)
    refs = {b: c1["sched"].sweep_f64(0, c1["V"], X[:, b], 20000, 5000) for b in range(0, B, max(1, B // 4))}
    for cfg in CONFIGS:
        Y = c1["eng"].multiply(X, 0, B=B, **cfg)
        for b, ref in refs.items():
            assert relmax(Y[:, b], ref) <= TOL, cfg


def test_c1_properties(c1):
    """Size-independent checks at full size: linearity, OR- and min-homomorphism."""
    eng, rng = c1["eng"], np.random.default_rng(5)
    x1, x2 = rng.uniform(-1, 1, (2, 5000)).astype(np.float32)
    y1, y2 = eng.multiply(x1, 0)[:, 0], eng.multiply(x2, 0)[:, 0]
    y12 = eng.multiply((2 * x1 - 3 * x2).astype(np.float32), 0)[:, 0]
    assert relmax(y12, 2 * y1.astype(np.float64) - 3 * y2) < 1e-5
    b1, b2 = (rng.random((2, 5000, 64)) < 0.01)
    Y1, Y2 = eng.multiply(gmr.pack_bits(b1), 1, B=64), eng.multiply(gmr.pack_bits(b2), 1, B=64)
    np.testing.assert_array_equal(eng.multiply(gmr.pack_bits(b1 | b2), 1, B=64), Y1 | Y2)
    t1 = rng.integers(0, 1000, (5000, 4)).astype(np.int32)
    t2 = rng.integers(0, 1000, (5000, 4)).astype(np.int32)
    T1, T2 = eng.multiply(t1, 2), eng.multiply(t2, 2)
    np.testing.assert_array_equal(eng.multiply(np.minimum(t1, t2), 2), np.minimum(T1, T2))


def test_c1_boolean_tropical_bit_exact(c1):
    rng = np.random.default_rng(11)
    for sr, B in ((1, 40), (2, 6)):
        X = random_X(sr, 5000, B, 12)
        Y = engine_outputs(sr, c1["eng"].multiply(engine_inputs(sr, X), sr, B=B), B)
        for b in rng.choice(B, 4, replace=False):
            ref = c1["sched"].cpu_reference(sr, c1["V"].astype(np.float32), X[:, b], 20000, 5000, threads=1)
            np.testing.assert_array_equal(Y[:, b], ref)


def test_lane_width_rule(case):
    """32-byte lanes for (+,x) tiles of 32 words or more, 16-byte lanes for
    (min,+) and narrower tiles, narrower accesses where the width demands."""
    eng = gmr.Engine(case["plan"])
    assert [eng.lane_bytes(0, B) for B in (32, 64, 128, 8, 4, 2, 3)] == [32, 32, 32, 16, 16, 8, 4]
    assert [eng.lane_bytes(2, B) for B in (32, 8)] == [16, 16]
    assert [eng.lane_bytes(1, B) for B in (32, 128, 256)] == [4, 16, 16]
