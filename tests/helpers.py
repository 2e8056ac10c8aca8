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
