"""bench.py stays runnable: every name it loads is defined, and --help works."""
import ast
import builtins
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

BENCH = Path(__file__).resolve().parent.parent / "bench.py"


def test_bench_has_no_undefined_names():
    tree = ast.parse(BENCH.read_text())
    loaded = {n.id for n in ast.walk(tree) if isinstance(n, ast.Name) and isinstance(n.ctx, ast.Load)}
    known = set(dir(builtins)) | {"__file__"}
    for n in ast.walk(tree):
        if isinstance(n, (ast.FunctionDef, ast.ClassDef)):
            known.add(n.name)
        elif isinstance(n, ast.Name) and isinstance(n.ctx, ast.Store):
            known.add(n.id)
        elif isinstance(n, ast.arguments):
            known |= {a.arg for a in n.args + n.kwonlyargs + n.posonlyargs}
            known |= {a.arg for a in (n.vararg, n.kwarg) if a is not None}
        elif isinstance(n, (ast.Import, ast.ImportFrom)):
            known |= {(a.asname or a.name).split(".")[0] for a in n.names}
        elif isinstance(n, ast.ExceptHandler) and n.name:
            known.add(n.name)
    assert sorted(loaded - known) == []


def test_bench_help_runs():
    r = subprocess.run([sys.executable, str(BENCH), "--help"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "--impl" in r.stdout and "--steps" in r.stdout


@pytest.mark.gpu
def test_cusparse_generic_baseline_small():
    """The direct cuSPARSE baseline (generic SpMM / SpMV through ctypes, int32
    CSR) on a small random 0/1 matrix: every algorithm it reports as run
    matches the dense product."""
    torch = pytest.importorskip("torch")
    import bench

    rng = np.random.default_rng(3)
    rows, cols, B = 700, 300, 8
    M = rng.random((rows, cols)) < 0.05
    crow = np.concatenate([[0], np.cumsum(M.sum(axis=1))]).astype(np.int64)
    colv = np.nonzero(M)[1].astype(np.int32)
    X = torch.rand((cols, B), device="cuda") * 2 - 1
    Y_ref = torch.from_numpy(M.astype(np.float32)).cuda() @ X
    out = bench.cusparse_generic(torch, crow, colv, rows, cols, X, B, 3, Y_ref.cpu())
    ran = {k: v for k, v in out["spmm_vps"].items() if isinstance(v, float)}
    assert ran, out
    assert all(e < 1e-5 for e in out["spmm_rel_err_vs_torch"].values()), out
    assert any(isinstance(v, float) for v in out["spmv_vps"].values()), out
