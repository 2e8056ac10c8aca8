"""The oracle (oracle/oracle.c) against the reference's own outputs.

tests/golden holds what the reference code produced on these grammars
(tests/golden/make_golden.py): its BuiltSchedule arrays, its FP64 cpu_sweep and
brute force (cpu_selftest.cpp), and its float/int sequential CPU sweep
(gpu_engine_test.cu:49-104)."""
import numpy as np
import pytest

from helpers import SEMIRINGS, golden_cases, golden_meta, load_case
from oracle import oracle as O


@pytest.fixture(params=golden_cases())
def case(request):
    return load_case(request.param)


def sched_of(c):
    return O.RefSchedule(int(c["alpha"]), c["rules"], c["C"])


def test_schedule_identical_to_reference(case):
    s = sched_of(case)
    head = case["ref_head"]
    assert [s.alpha, s.depth, s.max_width, s.num_raw, s.num_layered, s.num_pt, s.emit_total,
            s.num_term] == head.tolist()
    np.testing.assert_array_equal(s.left, case["ref_left"])
    np.testing.assert_array_equal(s.right, case["ref_right"])
    np.testing.assert_array_equal(s.coeff, case["ref_coeff"])
    np.testing.assert_array_equal(s.level_offsets, case["ref_level_offsets"])
    np.testing.assert_array_equal(s.emit_offsets, case["ref_emit_offsets"])
    np.testing.assert_array_equal(s.emit_pos, case["ref_emit_pos"])
    np.testing.assert_array_equal(s.emit_row, case["ref_emit_row"])
    np.testing.assert_array_equal(s.term_emit_sym, case["ref_term_sym"])
    np.testing.assert_array_equal(s.term_emit_row, case["ref_term_row"])
    np.testing.assert_array_equal(s.term_orig, case["ref_term_orig"])


@pytest.mark.parametrize("sr", range(3))
def test_sweep_f64_bit_identical(case, sr):
    s = sched_of(case)
    name = SEMIRINGS[sr]
    y = s.sweep_f64(sr, case["V"], case[f"x_{name}"], int(case["rows"]), int(case["cols"]))
    np.testing.assert_array_equal(y, case[f"y64_{name}"])


@pytest.mark.parametrize("sr", range(3))
def test_brute_force_matches(case, sr):
    name = SEMIRINGS[sr]
    vc = O.expand(int(case["alpha"]), case["rules"], case["C"])
    y = O.brute_force(vc, sr, case["V"], case[f"x_{name}"], int(case["rows"]), int(case["cols"]))
    if sr == 0:
        np.testing.assert_allclose(y, case[f"ybf_{name}"], rtol=0, atol=1e-12)
    else:
        np.testing.assert_array_equal(y, case[f"ybf_{name}"])
    assert bool(case["selftest_passed"])


@pytest.mark.parametrize("sr", range(3))
def test_cpu_reference_bit_identical(case, sr):
    """float / int sequential sweep == the reference's, bit for bit."""
    s = sched_of(case)
    name = SEMIRINGS[sr]
    y = s.cpu_reference(sr, case["V"].astype(np.float32), case[f"x_{name}"], int(case["rows"]),
                        int(case["cols"]), threads=1)
    np.testing.assert_array_equal(y.view(np.int32), case[f"y32_{name}"].view(np.int32))


def test_unittest_grammar_known_answer():
    """cpu_selftest.cpp:374-467: T/T, T/NT, run-length and NT/NT rules."""
    meta = golden_meta()["unittest"]
    assert meta["passed"]
    rules = np.array([[1, 2], [3, 5], [6, -1], [7, 5]])
    kinds = np.array([0, 0, 1, 0])
    reps = np.array([1, 1, 3, 1])
    s = O.RefSchedule(5, rules, np.array([8, 0]), kinds, reps)
    assert s.depth == meta["max_depth"] == 4
    assert s.num_pt == meta["num_passthrough"] == 5
    y = s.sweep_f64(0, np.array([1.5, 2.5]), np.array([0.5, -0.5, 1.0], np.float32), 2, 3)
    np.testing.assert_allclose(y, meta["y_sweep"], atol=1e-12)


def test_readme_known_answer():
    meta = golden_meta()["readme"]
    c = load_case("readme_8x7")
    np.testing.assert_array_equal(c["x_plustimes"], np.array(meta["x"], np.float32))
    np.testing.assert_allclose(c["y64_plustimes"], meta["y"], atol=1e-5)
    s = sched_of(c)
    y = s.sweep_f64(0, c["V"], c["x_plustimes"], 8, 7)
    np.testing.assert_allclose(y, meta["y"], atol=1e-5)


def test_planted_mistake_is_caught():
    """A wrong oracle must fail the golden check: perturb one rule."""
    c = load_case("mosaic_300x64")
    rules = c["rules"].copy()
    rules[5, 1] = rules[4, 1] if rules[4, 1] != rules[5, 1] else rules[6, 1]
    s = O.RefSchedule(int(c["alpha"]), rules, c["C"])
    y = s.sweep_f64(0, c["V"], c["x_plustimes"], int(c["rows"]), int(c["cols"]))
    assert not np.array_equal(y, c["y64_plustimes"])
