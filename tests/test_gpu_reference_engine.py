"""The reference's own GPU engine (its kernels from gpu-engine/gpu_engine.cu,
run by oracle/ref/ref_gpu.cpp with its host sequence) on this GPU: its results
match the oracle and this engine, so it can stand as the plain-sweep baseline."""
import numpy as np
import pytest

import gmr
from helpers import golden_cases, load_case
from oracle import oracle as O
from test_gpu_parity import check, engine_inputs, engine_outputs, oracle_columns, random_X

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref_gpu():
    why = O.RefGpu.available()
    if why:
        pytest.skip(why)
    return O.RefGpu(0)


@pytest.mark.parametrize("name", golden_cases())
@pytest.mark.parametrize("sr", range(3))
@pytest.mark.parametrize("B", [1, 5])
def test_reference_kernels_match_oracle_and_engine(ref_gpu, name, sr, B):
    c = load_case(name)
    rows, cols = int(c["rows"]), int(c["cols"])
    sched = O.RefSchedule(int(c["alpha"]), c["rules"], c["C"])
    X = random_X(sr, cols, B, 40 + B)
    Y, ms = ref_gpu.run(sched, sr, c["V"], X, rows, cols, iters=2)
    assert ms > 0
    ref = oracle_columns(sched, sr, c["V"], X, rows, cols)
    check(sr, Y.astype(np.float64) if sr == 0 else Y, ref)
    g = gmr.Grammar.from_arrays(int(c["alpha"]), c["rules"], c["C"], c["V"])
    eng = gmr.Engine(gmr.Plan.build(g, rows, cols))
    ours = engine_outputs(sr, eng.multiply(engine_inputs(sr, X), sr, B=B), B)
    if sr == 0:
        assert np.max(np.abs(ours - Y)) <= 1e-5 * max(1.0, float(np.max(np.abs(ref))))
    else:
        np.testing.assert_array_equal(np.asarray(ours, np.int64), np.asarray(Y, np.int64))
