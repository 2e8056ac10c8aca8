"""Generates the golden fixtures in tests/golden from the REFERENCE's own code.

Run in a container that holds the reference tree (g-mm-repair); its root is
taken from the environment variable GMR_REFERENCE (default /root/reference):

    GMR_REFERENCE=/path/to/g-mm-repair python tests/golden/make_golden.py

It builds the reference's sources where they lie (oracle/Makefile -> oracle/_ref:
cpu_selftest, host_scheduler and ref_tool, a harness that calls the
reference's cpu_sweep / brute_force / run_cpu_reference_layered), produces
small grammars with this project's seeded generators and RePair compressor,
runs the reference binaries on them and stores inputs and reference outputs
as .npz fixtures.  Nothing here runs at test time; the tests only read the
fixtures.

Known-answer cases that come from the reference's own tests and docs:
  * the cpu_selftest --unittest grammar (cpu_selftest.cpp:374-467):
    depth 4, 5 pass-throughs, y = [4.5, 0];
  * the README worked example (README.md:145-181): the 8x7 matrix with
    x = [2,1,1,2,1,1,1] gives y = [12.9, 20.7, 20.7, 12.9, 20.7, 19.3, 19.3, 12.9].
"""
from __future__ import annotations

import json
import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "g-mm-repair_gb300"))
sys.path.insert(0, str(REPO))

import gmr  # noqa: E402
from gmr import build as gbuild  # noqa: E402

REF_DIR = REPO / "oracle" / "_ref"

# README.md worked example (matrix rows as in the README)
README_M = np.array([
    [2.3, 0, 1.2, 1.2, 1.2, 2.3, 1.2],
    [1.2, 4.5, 3.4, 1.2, 1.2, 2.3, 4.5],
    [1.2, 4.5, 3.4, 1.2, 1.2, 2.3, 4.5],
    [2.3, 0, 1.2, 1.2, 1.2, 2.3, 1.2],
    [1.2, 4.5, 3.4, 1.2, 1.2, 2.3, 4.5],
    [0, 4.5, 3.4, 2.3, 2.3, 0, 4.5],
    [0, 4.5, 3.4, 2.3, 2.3, 0, 4.5],
    [2.3, 0, 1.2, 1.2, 1.2, 2.3, 1.2],
])
README_X = np.array([2, 1, 1, 2, 1, 1, 1], dtype=np.float32)
README_Y = np.array([12.9, 20.7, 20.7, 12.9, 20.7, 19.3, 19.3, 12.9])


def xs_for(cols: int, seed: int) -> dict:
    rng = np.random.default_rng(seed)
    trop = rng.integers(0, 1000, cols).astype(np.float32)
    trop[rng.random(cols) < 0.1] = 1e9
    return {
        "plustimes": rng.uniform(-1, 1, cols).astype(np.float32),
        "boolean": (rng.random(cols) < 0.5).astype(np.float32),
        "tropical": trop,
    }


def run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd} failed:\n{r.stdout}\n{r.stderr}")
    return r.stdout


def make_case(name: str, g: "gmr.Grammar", rows: int, cols: int, xs: dict, tmp: Path) -> dict:
    base = tmp / name
    g.save(base)
    for s, x in xs.items():
        x.astype(np.float32).tofile(f"{base}.x.{s}.x")
    run([str(REF_DIR / "ref_tool"), str(base), str(rows), str(cols), f"{base}.x", f"{base}.out"])
    out = dict(rows=rows, cols=cols, alpha=g.alpha, rules=g.rules(), C=g.C(), V=g.values())
    for s, x in xs.items():
        out[f"x_{s}"] = x
        out[f"y64_{s}"] = np.fromfile(f"{base}.out.{s}.y64", dtype=np.float64)
        out[f"ybf_{s}"] = np.fromfile(f"{base}.out.{s}.ybf", dtype=np.float64)
        y32 = np.fromfile(f"{base}.out.{s}.y32", dtype=np.int32)
        out[f"y32_{s}"] = y32.view(np.float32) if s == "plustimes" else y32
    raw = open(f"{base}.out.sched", "rb").read()
    head = np.frombuffer(raw[:64], dtype=np.int64)
    alpha, depth, max_width, n_raw, n_lay, n_pt, n_em, n_te = (int(v) for v in head)
    off = 64

    def take(n, dt):
        nonlocal off
        a = np.frombuffer(raw[off:off + n * 4], dtype=dt).copy()
        off += n * 4
        return a

    out["ref_head"] = head.copy()
    out["ref_left"], out["ref_right"], out["ref_coeff"] = take(n_lay, np.int32), take(n_lay, np.int32), take(
        n_lay, np.float32)
    out["ref_level_offsets"] = take(depth + 1, np.int32)
    out["ref_emit_offsets"] = take(depth + 1, np.int32)
    out["ref_emit_pos"], out["ref_emit_row"] = take(n_em, np.int32), take(n_em, np.int32)
    out["ref_term_sym"], out["ref_term_row"] = take(n_te, np.int32), take(n_te, np.int32)
    out["ref_term_orig"] = take(alpha, np.int32)
    assert off == len(raw), (off, len(raw))
    # the reference self-test on the same files (sweep vs brute force, 3 semirings)
    st = run([str(REF_DIR / "cpu_selftest"), str(base), str(rows), str(cols)])
    out["selftest_passed"] = np.array("REPAIR FILE-TEST PASSED" in st)
    # the reference inspector: raw level widths
    hs = run([str(REF_DIR / "host_scheduler"), str(base)])
    widths = [int(m.group(2)) for m in re.finditer(r"^(\d+)\t(\d+)$", hs, re.M)]
    out["host_scheduler_widths"] = np.array(widths, dtype=np.int64)
    np.savez_compressed(HERE / f"{name}.npz", **out)
    return {"name": name, "rows": rows, "cols": cols, "rules": int(g.n_rules), "C": int(len(out["C"])),
            "selftest_passed": bool(out["selftest_passed"]), "depth": depth, "passthrough": n_pt}


def main():
    gbuild.build()
    run(["make", "-s", "-C", str(REPO / "oracle"), "ref"])
    cases = []
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        # small mosaic genotype matrix (value 1)
        m = gmr.gen_mosaic(300, 64, 8, 0.05, 0.01, 7, threads=4)
        cases.append(make_case("mosaic_300x64", gmr.repair(m, 4), 300, 64, xs_for(64, 11), tmp))
        # copy-model graphs: unweighted (Boolean) and weighted (tropical)
        m = gmr.gen_copy_graph(400, 6, 0.7, False, 3, threads=4)
        cases.append(make_case("graph_400", gmr.repair(m, 4), 400, 400, xs_for(400, 12), tmp))
        m = gmr.gen_copy_graph(300, 5, 0.7, True, 5, threads=4)
        cases.append(make_case("graph_w300", gmr.repair(m, 4), 300, 300, xs_for(300, 13), tmp))
        # README worked example, with the README's x
        m = gmr.Csrv.from_dense(README_M)
        xs = xs_for(7, 14)
        xs["plustimes"] = README_X
        cases.append(make_case("readme_8x7", gmr.repair(m, 1), 8, 7, xs, tmp))
        # empty rows, a single-entry row, a dense row, several distinct values
        M = np.zeros((12, 9))
        M[1, 3] = 2.0
        M[4, :] = 1.5
        M[5, ::2] = 1.5
        M[7, ::2] = 1.5
        M[9, :] = 1.5
        M[11, 8] = -3.0
        cases.append(make_case("ragged_12x9", gmr.repair(gmr.Csrv.from_dense(M), 1), 12, 9, xs_for(9, 15), tmp))
    # the reference's own unit test (run-length rule; not expressible in .vc.R)
    ut = run([str(REF_DIR / "cpu_selftest"), "--unittest"])
    unit = {
        "max_depth": int(re.search(r"max_depth: (\d+)", ut).group(1)),
        "num_passthrough": int(re.search(r"num_passthrough: (\d+)", ut).group(1)),
        "y_sweep": [float(v) for v in re.search(r"y_sweep: \[([^\]]*)\]", ut).group(1).split(",")],
        "passed": "UNIT TEST PASSED" in ut,
    }
    meta = {"cases": cases, "unittest": unit,
            "readme": {"x": README_X.tolist(), "y": README_Y.tolist()}}
    (HERE / "golden.json").write_text(json.dumps(meta, indent=1) + "\n")
    print(json.dumps(meta, indent=1))


if __name__ == "__main__":
    main()
