"""RePair on the GPU: the same grammar as the host compressor, rule for rule
and symbol for symbol (integer work, compared exactly)."""
import numpy as np
import pytest

import gmr
from oracle import oracle as O


def assert_same_grammar(m):
    host = gmr.repair(m)
    devg = gmr.repair(m, device=0)
    assert devg.alpha == host.alpha
    np.testing.assert_array_equal(devg.rules(), host.rules())
    np.testing.assert_array_equal(devg.C(), host.C())
    np.testing.assert_array_equal(devg.values(), host.values())
    return host, devg


def csrv(rows, cols, codes, V=(1.0,)):
    return gmr.Csrv.from_codes(rows, cols, np.asarray(codes, np.int32), np.asarray(V, np.float64))


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(4))
def test_mosaic(seed):
    m = gmr.gen_mosaic(600 + 500 * seed, 128 + 100 * seed, 8, 0.02, 1e-3, seed)
    host, devg = assert_same_grammar(m)
    assert len(host.rules()) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("weighted", [False, True])
def test_copy_graph(weighted):
    assert_same_grammar(gmr.gen_copy_graph(30000, 10, 0.7, weighted, 4))


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(6))
def test_runs_and_repeats(seed):
    """Arbitrary strings with runs "aaa...": the counts skip overlapping
    occurrences and the greedy choices alternate inside runs."""
    rng = np.random.default_rng(seed)
    rows, alpha = 60, 9
    codes = []
    for _ in range(rows):
        row = []
        while len(row) < rng.integers(0, 40):
            sym = int(rng.integers(1, alpha))
            row += [sym] * int(rng.choice([1, 1, 2, 3, 5, 8]))
        if rng.random() < 0.5:
            row += row[: len(row) // 2]
        codes += row + [0]
    m = csrv(rows, alpha - 1, codes)
    host, devg = assert_same_grammar(m)
    # the grammar still expands to the input
    np.testing.assert_array_equal(O.expand(devg.alpha, devg.rules(), devg.C()), np.asarray(codes))


@pytest.mark.gpu
@pytest.mark.parametrize("codes,rows", [([], 0), ([0, 0], 2), ([1, 0], 1), ([1, 2, 0, 1, 2, 0], 2),
                                        ([3, 3, 3, 3, 0, 3, 3, 3, 0], 2)])
def test_small_edge_cases(codes, rows):
    assert_same_grammar(csrv(rows, 4, codes))


@pytest.mark.gpu
def test_c1_mosaic_and_plan():
    """20,000 x 5,000 mosaic: identical grammar, hence an identical plan."""
    m = gmr.gen_mosaic(20000, 5000, 64, 0.01, 1e-3, 0)
    host, devg = assert_same_grammar(m)
    a, b = gmr.Plan.build(host, 20000, 5000), gmr.Plan.build(devg, 20000, 5000, device=0)
    assert a.stats == b.stats


def test_device_repair_rejects_null():
    h = gmr.C.c_void_p()
    assert gmr.lib().gmr_repair_compress_device(None, 0, gmr.C.byref(h)) == 1
