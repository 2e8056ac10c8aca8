"""Test helpers: fixture loading and a numpy interpreter of a plan.

The interpreter evaluates the plan arrays exactly as the kernels are meant to
(values by level in an arena, emissions folded per level) so the schedule
builder can be checked on a machine without a GPU.  It is test code only."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
SEMIRINGS = ("plustimes", "boolean", "tropical")
INF = 1_000_000_000


def golden_cases():
    meta = json.loads((GOLDEN / "golden.json").read_text())
    return [c["name"] for c in meta["cases"]]


def load_case(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def golden_meta():
    return json.loads((GOLDEN / "golden.json").read_text())


def interp_plan(plan, semiring: int, x: np.ndarray) -> np.ndarray:
    """FP64 / int evaluation of a gmr.Plan for one right-hand side x (float)."""
    s = plan.stats
    op_l, op_r, op_c = plan.array("op_l"), plan.array("op_r"), plan.array("op_c")
    lvl, em_off = plan.array("lvl_off"), plan.array("em_off")
    src, row = plan.array("em_src"), plan.array("em_row")
    tv, tc, V = plan.array("term_val"), plan.array("term_col"), plan.array("V")
    x = np.asarray(x, dtype=np.float64)
    if semiring == 0:
        T = np.concatenate([[0.0], V[tv].astype(np.float64) * x[tc]])
        zero, op = 0.0, np.add
    elif semiring == 1:
        T = np.concatenate([[0], ((V[tv] != 0) & (x[tc] != 0)).astype(np.int64)])
        zero, op = 0, np.bitwise_or
    else:
        iv = np.trunc(V[tv]).astype(np.int64)
        ix = np.trunc(np.minimum(x[tc], 2**31 - 1)).astype(np.int64)
        leaf = np.where((iv >= INF) | (ix >= INF), INF, iv + ix)
        T = np.concatenate([[INF], leaf])
        zero, op = INF, np.minimum
    A = np.zeros(s["n_ops"], dtype=T.dtype)

    def val(refs):
        refs = np.asarray(refs, dtype=np.int64)
        out = np.empty(len(refs), dtype=T.dtype)
        m = refs >= 0
        out[m] = A[refs[m]]
        out[~m] = T[-refs[~m] - 1]
        return out

    y = np.full(s["rows"], zero, dtype=T.dtype)
    for k in range(0, s["depth"] + 1):
        if k >= 1:
            a, b = lvl[k - 1], lvl[k]
            lv = val(op_l[a:b])
            if semiring == 0 and len(op_c):
                lv = lv * op_c[a:b]
            A[a:b] = op(lv, val(op_r[a:b]))
        e0, e1 = em_off[k], em_off[k + 1]
        if e1 > e0:
            v = val(src[e0:e1])
            if semiring == 0:
                np.add.at(y, row[e0:e1], v)
            elif semiring == 1:
                np.bitwise_or.at(y, row[e0:e1], v)
            else:
                np.minimum.at(y, row[e0:e1], v)
    return y


def brute_left(codes, V, X, rows, cols, semiring):
    """y = x^T M from the CSRV string (codes val*cols+col+1, 0 = row end), per column of X [rows][B]."""
    X = np.asarray(X, dtype=np.float64)
    B = X.shape[1]
    ends = np.flatnonzero(codes == 0)
    r = np.repeat(np.arange(len(ends)), np.diff(np.concatenate([[-1], ends])) - 1)
    nz = codes[codes != 0].astype(np.int64) - 1
    c, v = nz % cols, np.asarray(V, dtype=np.float64)[nz // cols]
    if semiring == 0:
        Y = np.zeros((cols, B))
        np.add.at(Y, c, v[:, None] * X[r])
        return Y
    if semiring == 1:
        Y = np.zeros((cols, B), dtype=np.int64)
        np.bitwise_or.at(Y, c, ((v[:, None] != 0) & (X[r] != 0)).astype(np.int64))
        return Y
    iv = np.trunc(v).astype(np.int64)[:, None]
    ix = np.trunc(np.minimum(X[r], 2**31 - 1)).astype(np.int64)
    leaf = np.where((iv >= INF) | (ix >= INF), INF, iv + ix)
    Y = np.full((cols, B), INF, dtype=np.int64)
    np.minimum.at(Y, c, leaf)
    return Y


def interp_left(plan, semiring, X):
    """FP64 / int evaluation of the left product from the plan's transpose arrays."""
    s = plan.stats
    n = s["n_ops"]
    lvl = plan.array("lvl_off")
    po, ps = plan.array("par_off"), plan.array("par_src")
    eo, er = plan.array("erow_off"), plan.array("erow_row")
    to, tq = plan.array("tcol_off"), plan.array("tcol_q")
    tv, V, op_c = plan.array("term_val"), plan.array("V"), plan.array("op_c")
    X = np.asarray(X, dtype=np.float64)
    B = X.shape[1]
    zero = {0: 0.0, 1: 0, 2: INF}[semiring]
    op = {0: np.add, 1: np.bitwise_or, 2: np.minimum}[semiring]
    dt = np.float64 if semiring == 0 else np.int64
    Xs = X if semiring == 0 else (X != 0).astype(np.int64) if semiring == 1 else np.minimum(X, INF).astype(np.int64)
    down = np.full((n, B), zero, dtype=dt)

    def node_down(u):
        acc = np.full(B, zero, dtype=dt)
        for p in ps[po[u]:po[u + 1]]:
            pp = p if p >= 0 else ~p
            v = down[pp]
            if semiring == 0 and len(op_c) and p >= 0:
                v = v * op_c[pp]
            acc = op(acc, v)
        for r in er[eo[u]:eo[u + 1]]:
            acc = op(acc, Xs[r])
        return acc

    for k in range(s["depth"], 0, -1):
        for u in range(lvl[k - 1], lvl[k]):
            down[u] = node_down(u)
    Y = np.full((s["cols"], B), zero, dtype=dt)
    for c in range(s["cols"]):
        for q in tq[to[c]:to[c + 1]]:
            d = node_down(n + q)
            v = V[tv[q - 1]]
            if semiring == 0:
                l = v * d
            elif semiring == 1:
                l = d if v != 0 else np.zeros(B, dtype=dt)
            else:
                l = np.where((int(v) >= INF) | (d >= INF), INF, int(v) + d)
            Y[c] = op(Y[c], l)
    return Y


def interp_left_edges(plan, semiring, X, chunk=16):
    """The left product evaluated from the flat edge lists (le_*), level by
    level from the top, as the chunked fold does; also checks that le_split
    holds exactly the targets whose edges straddle a chunk."""
    s = plan.stats
    n, D = s["n_ops"], s["depth"]
    lo, src, tgt, split = (plan.array(a) for a in ("le_off", "le_src", "le_tgt", "le_split"))
    to, tq = plan.array("tcol_off"), plan.array("tcol_q")
    tv, V, op_c = plan.array("term_val"), plan.array("V"), plan.array("op_c")
    X = np.asarray(X, dtype=np.float64)
    B = X.shape[1]
    zero = {0: 0.0, 1: 0, 2: INF}[semiring]
    op = {0: np.add, 1: np.bitwise_or, 2: np.minimum}[semiring]
    dt = np.float64 if semiring == 0 else np.int64
    Xs = X if semiring == 0 else (X != 0).astype(np.int64) if semiring == 1 else np.minimum(X, INF).astype(np.int64)
    down = np.full((n, B), zero, dtype=dt)
    tdown = np.full((s["n_terms"], B), zero, dtype=dt)
    want_split = []
    for k in list(range(D, 0, -1)) + [D + 1]:
        a, b = int(lo[k - 1]), int(lo[k])
        t = tgt[a:b]
        assert np.all(np.diff(t) >= 0), "targets ascending within a level"
        starts = np.flatnonzero(np.r_[True, t[1:] != t[:-1]])
        ends = np.r_[starts[1:], len(t)] - 1
        for s0, s1 in zip(starts, ends):
            if s0 // chunk != s1 // chunk:
                want_split.append(int(t[s0]) if k <= D else n + int(t[s0]))
        out = tdown if k == D + 1 else down
        for e in range(a, b):
            sv = int(src[e])
            if sv >= n:
                v = Xs[sv - n]
            else:
                pp = sv if sv >= 0 else ~sv
                v = down[pp]
                if semiring == 0 and len(op_c) and sv >= 0:
                    v = v * op_c[pp]
            out[tgt[e]] = op(out[tgt[e]], v)
    assert sorted(want_split) == sorted(int(x) for x in split)
    Y = np.full((s["cols"], B), zero, dtype=dt)
    for c in range(s["cols"]):
        for q in tq[to[c]:to[c + 1]]:
            d = tdown[q]
            v = V[tv[q - 1]]
            if semiring == 0:
                l = v * d
            elif semiring == 1:
                l = d if v != 0 else np.zeros(B, dtype=dt)
            else:
                l = np.where((int(v) >= INF) | (d >= INF), INF, int(v) + d)
            Y[c] = op(Y[c], l)
    return Y
