"""bench.py stays runnable: every name it loads is defined, and --help works."""
import ast
import builtins
import subprocess
import sys
from pathlib import Path

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
