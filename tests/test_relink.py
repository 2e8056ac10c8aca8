"""Drop-in at link level: the reference's own gpu_test driver, unchanged,
links against libgmr.so (gpu-engine/Makefile:41-42 with gpu_engine.cu
replaced by the library; callers gpu_engine_test.cu:200-204, 225-228), and
the reference's header and include/gmr.h declare the same two entry points.

Needs the reference tree ($GMR_REFERENCE, default /root/reference) and nvcc;
skipped where either is absent.  Builds only (no GPU is used).
"""
import os
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO))
from oracle.oracle import reference_root  # noqa: E402

GPU_ENGINE = reference_root() / "gpu-engine"
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
ENTRY = ("run_gpu_right_multiply_layered", "run_gpu_right_multiply_batched")

pytestmark = pytest.mark.skipif(not (GPU_ENGINE / "gpu_engine_test.cu").exists() or not Path(NVCC).exists(),
                                reason="reference tree or nvcc absent")


def test_reference_header_and_gmr_h_agree(tmp_path):
    """Both headers in one C++ translation unit: two extern "C" declarations
    of one function with different parameters, or two different definitions
    of LayeredRule / GPUSchedule, would not compile."""
    tu = tmp_path / "both.cu"
    tu.write_text('#include "gmr.h"\n#include "gpu_engine.h"\n'
                  'static_assert(sizeof(LayeredRule) == 12, "LayeredRule");\n'
                  'auto* f1 = &run_gpu_right_multiply_layered;\nauto* f2 = &run_gpu_right_multiply_batched;\n')
    r = subprocess.run([NVCC, "-std=c++17", "-arch=sm_103a", f"-I{REPO / 'include'}", f"-I{GPU_ENGINE}", "-c",
                        str(tu), "-o", str(tmp_path / "both.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_unchanged_reference_driver_links_against_libgmr(tmp_path):
    sys.path.insert(0, str(REPO / "g-mm-repair_gb300"))
    from gmr import build as gbuild

    gbuild.build()
    out = tmp_path / "gpu_test"
    env = dict(os.environ, NVCC=NVCC)
    r = subprocess.run(["make", "-s", "-f", str(REPO / "g-mm-repair_gb300" / "gpu_test.mk"),
                        f"GMR_REFERENCE={reference_root()}", f"OUT={out}"], capture_output=True, text=True, env=env,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert out.exists()
    undefined = subprocess.run(["nm", "-D", "--undefined-only", str(out)], capture_output=True, text=True).stdout
    for name in ENTRY:  # resolved from libgmr.so at load time, not compiled into the driver
        assert name in undefined, name
    deps = subprocess.run(["ldd", str(out)], capture_output=True, text=True).stdout
    assert "libgmr.so" in deps
