"""The rules the GPU RePair uses to run a round without a sequential scan,
restated in numpy and checked against the host compressor on many random
strings (the GPU tests check the kernels; these check the argument):

* counting: inside a run of equal symbols a pair counts when its distance to
  the run's first symbol is even (non-overlapping occurrences);
* the greedy choice "replace at i when rank(i) <= rank(i+1), then skip i+1"
  is want(i) and not chosen(i-1), i.e. alternating from the start of each
  maximal run of wanting positions;
* after the first round only pairs that hold a symbol made by the previous
  round, or were candidates in it, can reach a count of two.
"""
import numpy as np
import pytest

import gmr

NONE = np.iinfo(np.int64).max


def run_starts(flag_start):
    """Index of the latest True at or before each position (a running maximum)."""
    idx = np.where(flag_start, np.arange(len(flag_start)), 0)
    return np.maximum.accumulate(idx) if len(idx) else idx


def parallel_repair(codes, alpha, restrict=True):
    s = np.asarray(codes, np.int64)
    rules = []
    cand_prev = None
    fresh = alpha
    for rnd in range(100000):
        n = len(s)
        if n < 2:
            break
        x, y = s[:-1], s[1:]
        valid = (x != 0) & (y != 0)
        eq_start = run_starts(np.r_[True, s[1:] != s[:-1]])[:-1]
        counted = valid & ((x != y) | (((np.arange(n - 1) - eq_start) & 1) == 0))
        rel = valid if (not restrict or cand_prev is None) else valid & (
            (x >= fresh) | (y >= fresh) | cand_prev[:-1])
        keys = x * (1 << 32) + y
        pos = np.flatnonzero(rel)
        if len(pos) < 2:
            break
        uk, inv = np.unique(keys[pos], return_inverse=True)
        cnt = np.bincount(inv, weights=counted[pos].astype(np.int64), minlength=len(uk)).astype(np.int64)
        cand = np.flatnonzero(cnt >= 2)
        if len(cand) == 0:
            break
        order = cand[np.lexsort((uk[cand], -cnt[cand]))]     # count desc, key asc
        rank_of = np.full(len(uk), NONE, np.int64)
        rank_of[order] = np.arange(len(order))
        rank = np.full(n, NONE, np.int64)
        rank[pos] = rank_of[inv]
        rn = np.r_[rank[1:], NONE]
        want = (rank != NONE) & (rank <= rn)
        wstart = run_starts(want & ~np.r_[False, want[:-1]])
        chosen = want & (((np.arange(n) - wstart) & 1) == 0)
        uses = np.bincount(rank[chosen], minlength=len(order))
        acc = uses >= 2
        if not acc.any():
            break
        maxsym = alpha + len(rules)
        newsym = np.full(len(order), -1, np.int64)
        newsym[acc] = maxsym + np.arange(acc.sum())
        for r in np.flatnonzero(acc):
            k = uk[order[r]]
            rules.append((int(k >> 32), int(k & 0xFFFFFFFF)))
        here = chosen & (rank != NONE)
        here[here] = acc[rank[here]]
        gone = np.r_[False, here[:-1]]
        sym = np.where(here, newsym[np.where(here, rank, 0)], s)
        keep = ~gone
        cand_prev = (rank != NONE)[keep]
        fresh = maxsym
        s = sym[keep]
    return np.array(rules, np.int64).reshape(-1, 2), s


def random_codes(rng, rows, alpha):
    codes = []
    for _ in range(rows):
        row = []
        while len(row) < rng.integers(0, 30):
            row += [int(rng.integers(1, alpha))] * int(rng.choice([1, 1, 2, 3, 5]))
        if rng.random() < 0.5:
            row += row[: len(row) // 2]
        codes += row + [0]
    return np.asarray(codes, np.int32)


@pytest.mark.parametrize("seed", range(20))
@pytest.mark.parametrize("restrict", [False, True])
def test_parallel_rules_give_the_host_grammar(seed, restrict):
    rng = np.random.default_rng(seed)
    alpha = int(rng.integers(3, 12))
    codes = random_codes(rng, int(rng.integers(5, 80)), alpha)
    g = gmr.repair(gmr.Csrv.from_codes(len(codes), alpha - 1, codes, np.asarray([1.0])))
    rules, C = parallel_repair(codes, g.alpha, restrict=restrict)
    np.testing.assert_array_equal(rules, g.rules().astype(np.int64))
    np.testing.assert_array_equal(C, g.C().astype(np.int64))


@pytest.mark.parametrize("seed", range(3))
def test_parallel_rules_on_a_mosaic(seed):
    m = gmr.gen_mosaic(300, 64, 6, 0.03, 1e-3, seed)
    g = gmr.repair(m)
    rules, C = parallel_repair(m.codes(), g.alpha)
    np.testing.assert_array_equal(rules, g.rules().astype(np.int64))
    np.testing.assert_array_equal(C, g.C().astype(np.int64))
