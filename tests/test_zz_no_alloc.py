"""The multiply entry point that allocates nothing (gmr_multiply_noalloc).

It serves callers that may not allocate device memory while they run (a
serving loop inside a fixed memory budget, a pool that must not grow): its
scratch lives in a static device array of the library, and the caller passes
the schedule, X and Y in device memory it owns.  This test plays such a caller:
it places the plan arrays in its own (torch) buffers, calls the entry point
through the C-ABI twice in a row with different inputs, and compares each
result with the engine's normal entry point (gmr_engine_multiply): (+,x) within
the parity tests' tolerance (relative max-norm 1e-5), (OR,AND) and (min,+)
bit-exact.  Collected last on purpose (file name), so a stop at the first
failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

import gmr
from gmr import _lib as L

pytestmark = pytest.mark.gpu
TOL = 1e-5


def relmax(y, ref):
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.abs(np.asarray(y, np.float64) - ref).max() / max(np.abs(ref).max(), 1e-30))


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    m = gmr.gen_mosaic(3000, 700, 32, 0.02, 0.002, 21, threads=4)
    plan = gmr.Plan.build(gmr.repair(m, 4), 3000, 700)
    eng = gmr.Engine(plan)
    dev = torch.device("cuda")

    def d(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    ops = np.stack([plan.array("op_l"), plan.array("op_r")], axis=1).reshape(-1)
    keep = {  # caller-owned device copies of the plan
        "ops": d(ops), "em_src": d(plan.array("em_src")), "seg_row": d(plan.array("seg_row")),
        "seg_start": d(plan.array("seg_start")), "term_val": d(plan.array("term_val")),
        "term_col": d(plan.array("term_col")), "V": d(plan.array("V")),
    }
    host = {"lvl_off": plan.array("lvl_off"), "seg_off": plan.array("seg_off")}
    st = plan.stats
    dp = L.DevicePlan()
    dp.rows, dp.cols, dp.depth = st["rows"], st["cols"], st["depth"]
    dp.n_ops, dp.n_terms = st["n_ops"], st["n_terms"]
    dp.lvl_off = host["lvl_off"].ctypes.data
    dp.seg_off = host["seg_off"].ctypes.data
    dp.ops = keep["ops"].data_ptr()
    dp.op_c = None
    for k in ("em_src", "seg_row", "seg_start", "term_val", "term_col", "V"):
        setattr(dp, k, keep[k].data_ptr())
    return dict(torch=torch, eng=eng, dp=dp, keep=keep, host=host, rows=st["rows"], cols=st["cols"])


def run_both(s, sr, X, B):
    torch = s["torch"]
    stream = torch.cuda.current_stream()
    dX = torch.from_numpy(np.ascontiguousarray(X).view(np.int32)).cuda()
    words = X.shape[1]
    y_new = torch.zeros((s["rows"], words), dtype=torch.int32, device="cuda")
    y_ref = torch.zeros((s["rows"], words), dtype=torch.int32, device="cuda")
    rc = gmr.lib().gmr_multiply_noalloc(C.byref(s["dp"]), sr, C.c_void_p(dX.data_ptr()),
                                        C.c_void_p(y_new.data_ptr()), B, C.c_void_p(stream.cuda_stream))
    assert rc == 0, gmr.lib().gmr_last_error().decode()
    s["eng"].multiply_device(sr, dX.data_ptr(), y_ref.data_ptr(), B, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    dt = {0: np.float32, 1: np.uint32, 2: np.int32}[sr]
    return y_new.cpu().numpy().view(dt), y_ref.cpu().numpy().view(dt)


@pytest.mark.parametrize("B", [1, 8, 32])
def test_noalloc_matches_engine_plustimes(setup, B):
    rng = np.random.default_rng(B)
    for call in range(2):  # two calls in a row share the static scratch
        X = rng.uniform(-1, 1, (setup["cols"], B)).astype(np.float32)
        y_new, y_ref = run_both(setup, 0, X, B)
        assert relmax(y_new, y_ref) <= TOL, (call, relmax(y_new, y_ref))


def test_noalloc_matches_engine_boolean_tropical(setup):
    rng = np.random.default_rng(7)
    for call in range(2):
        Xb = gmr.pack_bits(rng.random((setup["cols"], 64)) < 0.05)
        a, b = run_both(setup, 1, Xb, 64)
        np.testing.assert_array_equal(a, b)
        Xt = rng.integers(0, 1000, (setup["cols"], 4)).astype(np.int32)
        Xt[rng.random(Xt.shape) < 0.3] = 2**31 - 1
        a, b = run_both(setup, 2, Xt, 4)
        np.testing.assert_array_equal(a, b)


def test_noalloc_rejects_oversize(setup):
    dp = L.DevicePlan.from_buffer_copy(setup["dp"])
    big = np.array([0, 1 << 30], dtype=np.int64)  # a level of 2^30 rules: far beyond 64 MiB of scratch
    dp.lvl_off = big.ctypes.data
    dp.depth, dp.n_ops = 1, 1 << 30
    rc = gmr.lib().gmr_multiply_noalloc(C.byref(dp), 0, C.c_void_p(16), C.c_void_p(16), 32, None)
    assert rc == 6 and b"exceeds the static" in gmr.lib().gmr_last_error()
