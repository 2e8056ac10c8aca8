"""Schedule builder on the GPU: every plan array and figure equals the host
builder's (integer work, compared exactly), and the errors are the same."""
import numpy as np
import pytest

import gmr
from helpers import golden_cases, load_case

ARRAYS = ["op_l", "op_r", "op_c", "lvl_off", "em_off", "em_src", "em_row", "term_val", "term_col", "V",
          "seg_off", "seg_row", "seg_start"]


def assert_same_plan(g, rows, cols):
    host = gmr.Plan.build(g, rows, cols)
    devp = gmr.Plan.build(g, rows, cols, device=0, validate=True)
    assert devp.stats == host.stats
    for name in ARRAYS:
        np.testing.assert_array_equal(devp.array(name), host.array(name), err_msg=name)
    return host, devp


def random_grammar(seed, alpha=40, n=300, rows=25, runlen=0.2, dead=0.2):
    """Children-first rules over alpha terminals (some run-length, some never
    referenced from C) and a top sequence of `rows` rows."""
    rng = np.random.default_rng(seed)
    rules = np.zeros((n, 2), np.int32)
    kinds = (rng.random(n) < runlen).astype(np.int32)
    reps = np.where(kinds == 1, rng.integers(2, 9, n), 1).astype(np.int32)
    for i in range(n):
        hi = alpha + i
        # lean towards recent rules so the grammar gets deep
        pick = lambda: int(rng.integers(max(1, hi - 30), hi)) if rng.random() < 0.7 else int(rng.integers(1, hi))
        rules[i] = (pick(), pick() if kinds[i] == 0 else 0)
    referenced = rng.random(n) >= dead
    C = []
    for _ in range(rows):
        k = int(rng.integers(0, 12))
        for _ in range(k):
            if rng.random() < 0.3:
                C.append(int(rng.integers(1, alpha)))
            else:
                cand = np.flatnonzero(referenced)
                C.append(alpha + int(rng.choice(cand)) if cand.size else int(rng.integers(1, alpha)))
        C.append(0)
    cols = 4
    nv = (alpha - 2) // cols + 1
    V = rng.integers(1, 50, nv).astype(np.float64)
    return gmr.Grammar.from_arrays(alpha, rules, np.array(C, np.int32), V, kinds=kinds, reps=reps), rows, cols


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_cases())
def test_golden_grammars(name):
    c = load_case(name)
    g = gmr.Grammar.from_arrays(int(c["alpha"]), c["rules"], c["C"], c["V"])
    assert_same_plan(g, int(c["rows"]), int(c["cols"]))


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(12))
def test_random_grammars_with_runlength_and_dead_rules(seed):
    g, rows, cols = random_grammar(seed, n=50 + 97 * seed, runlen=0.1 + 0.03 * seed)
    host, _ = assert_same_plan(g, rows, cols)
    assert host.stats["n_ops"] > 0


@pytest.mark.gpu
def test_unittest_grammar_runlength():
    g = gmr.Grammar.from_arrays(5, [[1, 2], [3, 5], [6, 0], [7, 5]], [8, 0], [1.5, 2.5], kinds=[0, 0, 1, 0],
                                reps=[1, 1, 3, 1])
    _, d = assert_same_plan(g, 2, 3)
    assert d.stats["depth"] == 4 and d.stats["ref_passthrough"] == 5 and d.stats["has_coeff"] == 1


@pytest.mark.gpu
@pytest.mark.parametrize("C,rows", [([], 0), ([], 3), ([0, 0, 0], 3), ([1, 3, 0, 0, 2, 0], 3), ([2, 0], 4)])
def test_terminals_only_and_empty_rows(C, rows):
    g = gmr.Grammar.from_arrays(4, np.zeros((0, 2), np.int32), np.array(C, np.int32), [1.0])
    _, d = assert_same_plan(g, rows, 3)
    assert d.stats["depth"] == 0


@pytest.mark.gpu
def test_unreferenced_rules_only():
    g = gmr.Grammar.from_arrays(4, [[1, 2], [4, 3]], [1, 0], [1.0])
    _, d = assert_same_plan(g, 1, 3)
    assert d.stats["n_ops"] == 0 and d.stats["ref_raw"] == 2


@pytest.mark.gpu
def test_mosaic_and_graph_grammars():
    g = gmr.repair(gmr.gen_mosaic(3000, 700, 16, 0.01, 1e-3, 5))
    assert_same_plan(g, 3000, 700)
    g = gmr.repair(gmr.gen_copy_graph(20000, 12, 0.7, True, 9))
    assert_same_plan(g, 20000, 20000)


@pytest.mark.gpu
def test_c1_grammar_and_multiply():
    """20,000 x 5,000 mosaic: identical plan; engines on the two plans agree
    bit for bit in (OR,AND) and within 1e-5 relative in (+,x), whose fp32
    atomics make the summation order vary from run to run."""
    g = gmr.repair(gmr.gen_mosaic(20000, 5000, 64, 0.01, 1e-3, 0))
    host, devp = assert_same_plan(g, 20000, 5000)
    eh, ed = gmr.Engine(host), gmr.Engine(devp)
    X = np.random.default_rng(1).uniform(-1, 1, (5000, 8)).astype(np.float32)
    a, b = eh.multiply(X, "plustimes", B=8), ed.multiply(X, "plustimes", B=8)
    assert np.max(np.abs(a - b)) <= 1e-5 * np.max(np.abs(a))
    Xb = gmr.pack_bits(np.random.default_rng(2).random((5000, 64)) < 0.01)
    np.testing.assert_array_equal(eh.multiply(Xb, "boolean", B=64), ed.multiply(Xb, "boolean", B=64))


@pytest.mark.gpu
def test_same_errors_as_host():
    g = gmr.Grammar.from_arrays(4, [[1, 2]], [4, 0, 3, 0, 1, 0], [1.0])
    assert_same_plan(g, 3, 3)
    for build in (lambda: gmr.Plan.build(g, 2, 3), lambda: gmr.Plan.build(g, 2, 3, device=0)):
        with pytest.raises(gmr.GmrError) as e:
            build()
        assert e.value.code == 2 and "more rows" in str(e.value)
    g = gmr.Grammar.from_arrays(10, [[1, 9]], [10, 0], [1.0])  # code 9 -> value index 2 of 1
    msgs = []
    for build in (lambda: gmr.Plan.build(g, 1, 4), lambda: gmr.Plan.build(g, 1, 4, device=0)):
        with pytest.raises(gmr.GmrError) as e:
            build()
        msgs.append((e.value.code, str(e.value)))
    assert msgs[0] == msgs[1]


def test_device_build_rejects_bad_arguments():
    g = gmr.Grammar.from_arrays(4, [[1, 2]], [4, 0], [1.0])
    with pytest.raises(gmr.GmrError) as e:
        gmr.Plan.build(g, -1, 3, device=0)
    assert e.value.code == 1
