"""Host-side logic without a GPU: generators, RePair, file format, schedule."""
import numpy as np
import pytest

import gmr
from helpers import INF, SEMIRINGS, brute_left, golden_cases, interp_left, interp_left_edges, interp_plan, load_case
from oracle import oracle as O


# ---------------------------------------------------------------- generators
def test_mosaic_deterministic_across_threads():
    a = gmr.gen_mosaic(500, 300, 16, 0.01, 0.001, 42, threads=1).codes()
    b = gmr.gen_mosaic(500, 300, 16, 0.01, 0.001, 42, threads=7).codes()
    np.testing.assert_array_equal(a, b)
    c = gmr.gen_mosaic(500, 300, 16, 0.01, 0.001, 43, threads=7).codes()
    assert not np.array_equal(a, c)


def test_mosaic_shape_and_density():
    m = gmr.gen_mosaic(2000, 500, 64, 0.01, 1e-3, 0, threads=4)
    codes = m.codes()
    assert (codes == 0).sum() == 2000
    dens = m.nnz / (2000 * 500)
    assert 0.35 < dens < 0.65  # Beta(1/2,1/2) allele frequency: mean 1/2
    # columns strictly increasing within each row
    rows = np.split(codes, np.flatnonzero(codes == 0) + 1)[:-1]
    for r in rows[:50]:
        assert np.all(np.diff(r[:-1]) > 0)


def test_copy_graph_deterministic_sorted_dedup():
    a = gmr.gen_copy_graph(1000, 8, 0.7, True, 3, threads=1)
    b = gmr.gen_copy_graph(1000, 8, 0.7, True, 3, threads=5)
    np.testing.assert_array_equal(a.codes(), b.codes())
    codes = a.codes()
    assert (codes == 0).sum() == 1000
    assert np.array_equal(a.values(), np.arange(1, 101))
    for r in np.split(codes, np.flatnonzero(codes == 0) + 1)[:-1][:100]:
        cols = (r[:-1] - 1) % 1000
        assert np.all(np.diff(cols) > 0)  # sorted, no duplicate targets


# ---------------------------------------------------------------- RePair
@pytest.mark.parametrize("kind", ["mosaic", "graph", "wgraph", "dense"])
def test_repair_round_trip(kind):
    if kind == "mosaic":
        m = gmr.gen_mosaic(400, 200, 8, 0.02, 0.01, 5, threads=3)
    elif kind == "graph":
        m = gmr.gen_copy_graph(800, 10, 0.8, False, 9, threads=3)
    elif kind == "wgraph":
        m = gmr.gen_copy_graph(500, 7, 0.6, True, 2, threads=3)
    else:
        rng = np.random.default_rng(1)
        M = rng.choice([0.0, 1.0, 2.5], size=(30, 17))
        M[3] = 0.0
        m = gmr.Csrv.from_dense(M)
    g = gmr.repair(m, 3)
    vc = O.expand(g.alpha, g.rules(), g.C())
    np.testing.assert_array_equal(vc, m.codes())
    # topological numbering, binary rules never spanning a row end
    r = g.rules()
    idx = np.arange(len(r)) + g.alpha
    assert np.all(r[:, 0] < idx) and np.all(r[:, 1] < idx) and np.all(r >= 1)
    # every pair replaced occurs at least twice at creation -> no dead rules
    used = np.zeros(len(r), bool)
    Cs = g.C()
    used[Cs[Cs >= g.alpha] - g.alpha] = True
    for i in range(len(r) - 1, -1, -1):
        if used[i]:
            for c in r[i]:
                if c >= g.alpha:
                    used[c - g.alpha] = True
    assert used.all()
    assert len(Cs) + 2 * len(r) < len(vc)  # it compresses


def test_repair_thread_count_independent():
    m = gmr.gen_mosaic(300, 100, 8, 0.02, 0.01, 5, threads=2)
    g1, g2 = gmr.repair(m, 1), gmr.repair(m, 1)
    np.testing.assert_array_equal(g1.rules(), g2.rules())
    g4 = gmr.repair(m, 4)
    vc = O.expand(g4.alpha, g4.rules(), g4.C())
    np.testing.assert_array_equal(vc, m.codes())


def test_grammar_file_round_trip(tmp_path):
    c = load_case("mosaic_300x64")
    g = gmr.Grammar.from_arrays(int(c["alpha"]), c["rules"], c["C"], c["V"])
    g.save(tmp_path / "m")
    h = gmr.Grammar.load(tmp_path / "m")
    np.testing.assert_array_equal(h.rules(), c["rules"])
    np.testing.assert_array_equal(h.C(), c["C"])
    np.testing.assert_array_equal(h.values(), c["V"])
    raw = np.fromfile(tmp_path / "m.vc.R", dtype=np.int32)
    assert raw[0] == c["alpha"] and np.array_equal(raw[1:], c["rules"].reshape(-1))


# ---------------------------------------------------------------- error paths
def test_truncated_rules_file(tmp_path):
    c = load_case("graph_400")
    g = gmr.Grammar.from_arrays(int(c["alpha"]), c["rules"], c["C"], c["V"])
    g.save(tmp_path / "g")
    raw = (tmp_path / "g.vc.R").read_bytes()
    (tmp_path / "g.vc.R").write_bytes(raw[:-4])
    with pytest.raises(gmr.GmrError) as e:
        gmr.Grammar.load(tmp_path / "g")
    assert e.value.code == 2


def test_out_of_range_child_rejected():
    with pytest.raises(gmr.GmrError) as e:
        gmr.Grammar.from_arrays(5, [[1, 2], [3, 7]], [6, 0], [1.0])  # rule 1 refers to itself (7 = alpha+2)
    assert e.value.code == 2
    with pytest.raises(gmr.GmrError):
        gmr.Grammar.from_arrays(5, [[0, 2]], [5, 0], [1.0])  # the row delimiter as a child


def test_alpha_overflow_rejected():
    with pytest.raises(gmr.GmrError) as e:
        gmr.Grammar.from_arrays(2**31 - 2, [[1, 2], [1, 2], [1, 2]], [0], [1.0])
    assert e.value.code == 6


def test_more_rows_than_declared_rejected():
    g = gmr.Grammar.from_arrays(4, [[1, 2]], [4, 0, 3, 0, 1, 0], [1.0])
    gmr.Plan.build(g, 3, 3)
    with pytest.raises(gmr.GmrError):
        gmr.Plan.build(g, 2, 3)


def test_terminal_without_value_rejected():
    g = gmr.Grammar.from_arrays(10, [[1, 9]], [10, 0], [1.0])  # code 9 -> value index 2 of 1
    with pytest.raises(gmr.GmrError):
        gmr.Plan.build(g, 1, 4)


def test_corrupt_layered_schedule_rejected():
    c = load_case("mosaic_300x64")
    s = O.RefSchedule(int(c["alpha"]), c["rules"], c["C"])
    vi, ci = s.terminal_tables(int(c["cols"]))
    rules = s.rules_lrc()
    k = int(s.level_offsets[2])
    rules["l"][k] = int(s.level_widths[2]) + 5  # beyond the previous frontier
    with pytest.raises(gmr.GmrError) as e:
        gmr.Plan.from_layered(int(c["rows"]), int(c["cols"]), s.alpha, rules, vi, ci, c["V"], s.gpu_schedule())
    assert e.value.code == 2
    sched = s.gpu_schedule()
    sched["emit_row"] = sched["emit_row"].copy()
    sched["emit_row"][0] = int(c["rows"])
    with pytest.raises(gmr.GmrError):
        gmr.Plan.from_layered(int(c["rows"]), int(c["cols"]), s.alpha, s.rules_lrc(), vi, ci, c["V"], sched)


# ---------------------------------------------------------------- plan
@pytest.fixture(params=golden_cases())
def case(request):
    return load_case(request.param)


def test_plan_reference_figures(case):
    """L, w*, |R|, +pt, E, E_T, U as the reference's build_schedule computes them."""
    g = gmr.Grammar.from_arrays(int(case["alpha"]), case["rules"], case["C"], case["V"])
    st = gmr.Plan.build(g, int(case["rows"]), int(case["cols"])).stats
    alpha, depth, max_width, n_raw, n_lay, n_pt, n_em, n_te = case["ref_head"].tolist()
    assert (st["depth"], st["ref_max_width"], st["ref_raw"], st["ref_layered"], st["ref_passthrough"],
            st["ref_emit"], st["ref_term_emit"], st["ref_alpha"]) == (depth, max_width, n_raw, n_lay, n_pt, n_em,
                                                                       n_te, alpha)
    assert st["n_ops"] == n_raw  # every raw rule evaluated once, no pass-through copies


def test_plan_level_ops_match_host_scheduler(case):
    g = gmr.Grammar.from_arrays(int(case["alpha"]), case["rules"], case["C"], case["V"])
    ops = gmr.Plan.build(g, int(case["rows"]), int(case["cols"])).level_ops()
    np.testing.assert_array_equal(ops[1:], case["host_scheduler_widths"])


@pytest.mark.parametrize("sr", range(3))
def test_plan_interpretation_matches_reference(case, sr):
    """The plan, evaluated level by level, gives the reference's y."""
    name = SEMIRINGS[sr]
    g = gmr.Grammar.from_arrays(int(case["alpha"]), case["rules"], case["C"], case["V"])
    p = gmr.Plan.build(g, int(case["rows"]), int(case["cols"]))
    y = interp_plan(p, sr, case[f"x_{name}"])
    ref = case[f"y64_{name}"]
    if sr == 0:  # V is held as float32, as the reference engine holds it (gpu_engine_test.cu:305-308)
        np.testing.assert_allclose(y, ref, rtol=1e-7, atol=1e-6)
    else:
        np.testing.assert_array_equal(y, ref.astype(np.int64))


@pytest.mark.parametrize("sr", range(3))
def test_plan_from_layered_matches_reference(case, sr):
    """The legacy boundary: the reference's layered schedule relaid out."""
    name = SEMIRINGS[sr]
    s = O.RefSchedule(int(case["alpha"]), case["rules"], case["C"])
    vi, ci = s.terminal_tables(int(case["cols"]))
    p = gmr.Plan.from_layered(int(case["rows"]), int(case["cols"]), s.alpha, s.rules_lrc(), vi, ci, case["V"],
                              s.gpu_schedule())
    st = p.stats
    assert st["ref_passthrough"] == s.num_pt and st["n_ops"] == s.num_raw
    y = interp_plan(p, sr, case[f"x_{name}"])
    ref = case[f"y64_{name}"]
    if sr == 0:
        np.testing.assert_allclose(y, ref, rtol=1e-7, atol=1e-6)
    else:
        np.testing.assert_array_equal(y, ref.astype(np.int64))


def test_plan_child_sorted_and_row_sorted(case):
    g = gmr.Grammar.from_arrays(int(case["alpha"]), case["rules"], case["C"], case["V"])
    p = gmr.Plan.build(g, int(case["rows"]), int(case["cols"]))
    lvl, em = p.array("lvl_off"), p.array("em_off")
    L, R = p.array("op_l"), p.array("op_r")
    for k in range(1, len(lvl)):
        a, b = lvl[k - 1], lvl[k]
        key = L[a:b].astype(np.int64) * (1 << 32) + R[a:b]
        assert np.all(np.diff(key) >= 0)
        assert np.all(L[a:b] < a) and np.all(R[a:b] < a)  # children strictly below
    rows = p.array("em_row")
    for k in range(len(em) - 1):
        assert np.all(np.diff(rows[em[k]:em[k + 1]]) >= 0)


def test_unittest_grammar_plan():
    """Run-length rule: the plan keeps a coefficient array (cpu_selftest.cpp:374-467)."""
    g = gmr.Grammar.from_arrays(5, [[1, 2], [3, 5], [6, 0], [7, 5]], [8, 0], [1.5, 2.5], kinds=[0, 0, 1, 0],
                                reps=[1, 1, 3, 1])
    p = gmr.Plan.build(g, 2, 3)
    st = p.stats
    assert st["depth"] == 4 and st["ref_passthrough"] == 5 and st["has_coeff"] == 1
    y = interp_plan(p, 0, np.array([0.5, -0.5, 1.0], np.float32))
    np.testing.assert_allclose(y, [4.5, 0.0], atol=1e-12)


def test_empty_grammar_terminals_only():
    g = gmr.Grammar.from_arrays(4, np.zeros((0, 2), np.int32), [1, 3, 0, 0, 2, 0], [1.0])
    p = gmr.Plan.build(g, 3, 3)
    assert p.stats["depth"] == 0 and p.stats["n_ops"] == 0
    y = interp_plan(p, 0, np.array([1.0, 2.0, 4.0], np.float32))
    np.testing.assert_allclose(y, [5.0, 0.0, 2.0])


def test_describe_lists_levels(case):
    g = gmr.Grammar.from_arrays(int(case["alpha"]), case["rules"], case["C"], case["V"])
    d = gmr.Plan.build(g, int(case["rows"]), int(case["cols"])).describe()
    assert d.startswith("Max depth (L): ")
    levels, windows = d.split("Left-child windows")
    assert len([ln for ln in levels.splitlines() if ln[:1].isdigit()]) == case["ref_head"][1] + 1
    assert len([ln for ln in windows.splitlines() if ln[:1].isdigit()]) == case["ref_head"][1]


def test_alg_bytes_formula(case):
    g = gmr.Grammar.from_arrays(int(case["alpha"]), case["rules"], case["C"], case["V"])
    p = gmr.Plan.build(g, int(case["rows"]), int(case["cols"]))
    alpha, depth, mw, n_raw, n_lay, n_pt, n_em, n_te = case["ref_head"].tolist()
    rows, cols, nv = int(case["rows"]), int(case["cols"]), len(case["V"])
    for B in (1, 32):
        want = 12 * n_lay + 8 * n_em + 8 * n_te + 8 * (alpha - 1) + 4 * nv + 4 * cols * B + 4 * rows * B
        assert p.alg_bytes(0, B) == want
    assert p.alg_bytes(1, 64) == 12 * n_lay + 8 * n_em + 8 * n_te + 8 * (alpha - 1) + 4 * nv + 8 * cols + 8 * rows


@pytest.mark.parametrize("sr", range(3))
def test_left_product_structures(case, sr):
    """The transpose arrays, evaluated top-down, give y = x^T M of the expanded matrix."""
    g = gmr.Grammar.from_arrays(int(case["alpha"]), case["rules"], case["C"], case["V"])
    rows, cols = int(case["rows"]), int(case["cols"])
    p = gmr.Plan.build(g, rows, cols)
    p.prepare_left()
    assert len(p.array("par_src")) == 2 * p.stats["n_ops"]
    assert p.array("erow_off")[-1] == p.stats["n_emit"] + p.stats["n_term_emit"]
    rng = np.random.default_rng(sr)
    if sr == 0:
        X = rng.uniform(-1, 1, (rows, 3))
    elif sr == 1:
        X = (rng.random((rows, 3)) < 0.3).astype(np.float64)
    else:
        X = rng.integers(0, 1000, (rows, 3)).astype(np.float64)
        X[rng.random(X.shape) < 0.3] = 1e9
    codes = O.expand(g.alpha, g.rules(), g.C())
    ref = brute_left(codes, case["V"].astype(np.float32), X, rows, cols, sr)
    for Y in (interp_left(p, sr, X), interp_left_edges(p, sr, X)):
        if sr == 0:
            np.testing.assert_allclose(Y, ref, rtol=1e-6, atol=1e-6)
        else:
            np.testing.assert_array_equal(Y, ref)


@pytest.mark.parametrize("sr", range(3))
def test_left_edge_lists_straddling_chunks(sr):
    """A mosaic grammar whose popular symbols have far more than one chunk of
    edges: the flat edge lists still give x^T M, and le_split is exact."""
    m = gmr.gen_mosaic(400, 120, 6, 0.02, 1e-3, 4)
    g = gmr.repair(m)
    p = gmr.Plan.build(g, 400, 120)
    p.prepare_left()
    assert len(p.array("le_split")) > 10
    rng = np.random.default_rng(sr)
    X = rng.uniform(-1, 1, (400, 2)) if sr == 0 else (rng.random((400, 2)) < 0.3).astype(np.float64) \
        if sr == 1 else rng.integers(0, 1000, (400, 2)).astype(np.float64)
    ref = brute_left(O.expand(g.alpha, g.rules(), g.C()), g.values().astype(np.float32), X, 400, 120, sr)
    Y = interp_left_edges(p, sr, X)
    if sr == 0:
        np.testing.assert_allclose(Y, ref, rtol=1e-6, atol=1e-6)
    else:
        np.testing.assert_array_equal(Y, ref)


def test_left_edge_lists_runlength():
    g = gmr.Grammar.from_arrays(5, [[1, 2], [3, 5], [6, 0], [7, 5]], [8, 0], [1.5, 2.5], kinds=[0, 0, 1, 0],
                                reps=[1, 1, 3, 1])
    p = gmr.Plan.build(g, 2, 3)
    p.prepare_left()
    X = np.array([[2.0], [-1.0]])
    np.testing.assert_allclose(interp_left_edges(p, 0, X), interp_left(p, 0, X), atol=1e-12)


def test_window_stats_match_numpy_restatement():
    """The plan's left-child window statistics (shared-memory staging) equal a
    direct numpy computation over the plan arrays."""
    m = gmr.gen_mosaic(4000, 900, 32, 0.02, 0.002, 5, threads=4)
    g = gmr.repair(m, 4)
    plan = gmr.Plan.build(g, 4000, 900)
    R, words = 64, 8
    got = plan.window_stats(R, words)
    lvl, opl = plan.array("lvl_off"), plan.array("op_l")
    assert got.shape == (plan.stats["depth"], 5)
    for k in range(1, plan.stats["depth"] + 1):
        a, b = int(lvl[k - 1]), int(lvl[k])
        fits, dens, runs = np.zeros(3), [], 0
        for r0 in range(a, b, R):
            c = opl[r0:min(r0 + R, b)]
            c = c[c >= 0]
            runs += 1
            win = (int(c[-1]) - int(c[0]) + 1) if len(c) else 0
            fits += np.array([win * words * 4 <= x * 1024 for x in (64, 128, 200)])
            if len(c):
                dens.append(len(np.unique(c)) / win)
        exp = [*(fits / max(runs, 1)), np.mean(dens) if dens else 0.0, (opl[a:b] >= 0).mean() if b > a else 0.0]
        np.testing.assert_allclose(got[k - 1], exp, rtol=1e-12, atol=1e-12)
    assert "Left-child windows" in plan.describe()


def test_window_stats_rejects_bad_arguments():
    m = gmr.gen_mosaic(500, 200, 8, 0.02, 0.002, 3, threads=2)
    plan = gmr.Plan.build(gmr.repair(m, 2), 500, 200)
    with pytest.raises(gmr.GmrError):
        plan.window_stats(0, 32)
    with pytest.raises(gmr.GmrError):
        plan.window_stats(64, 0)


def test_interleave_eligibility_follows_level_widths():
    """A level can be interleaved when it spans two source chunks or more."""
    from gmr import learn

    m = gmr.gen_mosaic(3000, 700, 16, 0.02, 0.002, 4, threads=2)
    plan = gmr.Plan.build(gmr.repair(m, 2), 3000, 700)
    lvl = plan.array("lvl_off")  # lvl_off[k] = end of level k, lvl_off[0] = 0
    widths = np.diff(lvl)        # widths[k - 1] = rules of level k
    cs = int(np.median(widths[widths > 0]))
    ok = learn.interleave_allowed(plan, chunk_slots=cs)
    assert not ok[0] and not ok[-1]
    for k in range(1, plan.stats["depth"] + 1):
        assert ok[k] == (widths[k - 1] > cs)
