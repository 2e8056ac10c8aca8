"""The multiply entry point that allocates nothing (gmr_multiply_noalloc).

It serves callers that may not allocate device memory while they run (a
serving loop inside a fixed memory budget, a pool that must not grow): its
scratch lives in a static device array of the library, and the caller passes
the schedule, X and Y in device memory it owns.  This test plays such a caller:
it places the plan arrays in its own (torch) buffers, calls the entry point
through the C-ABI twice in a row with different inputs, and compares each
result with the oracle (the FP64 sweep for (+,x), the reference's int sweep for
(OR,AND) and (min,+)) and with the engine's normal entry point
(gmr_engine_multiply): (+,x) within the parity tests' tolerance (relative
max-norm 1e-5), (OR,AND) and (min,+) bit-exact.  It also checks that the
device's free memory does not change across calls.  Collected last on purpose
(file name), so a stop at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

import gmr
from gmr import _lib as L
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-5
DT = {0: np.float32, 1: np.uint32, 2: np.int32}


def relmax(y, ref):
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.abs(np.asarray(y, np.float64) - ref).max() / max(np.abs(ref).max(), 1e-30))


def device_plan(torch, plan):
    """The plan's arrays in caller-owned device memory, as gmr_device_plan."""
    dev = torch.device("cuda")

    def d(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    ops = np.stack([plan.array("op_l"), plan.array("op_r")], axis=1).reshape(-1)
    st = plan.stats
    keep = {"ops": d(ops), "em_src": d(plan.array("em_src")), "seg_row": d(plan.array("seg_row")),
            "seg_start": d(plan.array("seg_start")), "term_val": d(plan.array("term_val")),
            "term_col": d(plan.array("term_col")), "V": d(plan.array("V"))}
    if st["has_coeff"]:
        keep["op_c"] = d(plan.array("op_c"))
    host = {"lvl_off": plan.array("lvl_off"), "seg_off": plan.array("seg_off")}
    dp = L.DevicePlan()
    dp.rows, dp.cols, dp.depth = st["rows"], st["cols"], st["depth"]
    dp.n_ops, dp.n_terms = st["n_ops"], st["n_terms"]
    dp.lvl_off = host["lvl_off"].ctypes.data
    dp.seg_off = host["seg_off"].ctypes.data
    for k in ("ops", "em_src", "seg_row", "seg_start", "term_val", "term_col", "V"):
        setattr(dp, k, keep[k].data_ptr())
    dp.op_c = keep["op_c"].data_ptr() if "op_c" in keep else None
    return dp, keep, host


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    m = gmr.gen_mosaic(3000, 700, 32, 0.02, 0.002, 21, threads=4)
    g = gmr.repair(m, 4)
    plan = gmr.Plan.build(g, 3000, 700)
    dp, keep, host = device_plan(torch, plan)
    st = plan.stats
    return dict(torch=torch, eng=gmr.Engine(plan), dp=dp, keep=keep, host=host, rows=st["rows"], cols=st["cols"],
                sched=O.RefSchedule(g.alpha, g.rules(), g.C()), V=g.values())


def noalloc(s, sr, dX, dY, B):
    torch = s["torch"]
    rc = gmr.lib().gmr_multiply_noalloc(C.byref(s["dp"]), sr, C.c_void_p(dX.data_ptr()), C.c_void_p(dY.data_ptr()),
                                        B, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, gmr.lib().gmr_last_error().decode()


def run_both(s, sr, X, B):
    torch = s["torch"]
    stream = torch.cuda.current_stream()
    dX = torch.from_numpy(np.ascontiguousarray(X).view(np.int32)).cuda()
    words = X.shape[1]
    y_new = torch.zeros((s["rows"], words), dtype=torch.int32, device="cuda")
    y_ref = torch.zeros((s["rows"], words), dtype=torch.int32, device="cuda")
    noalloc(s, sr, dX, y_new, B)
    s["eng"].multiply_device(sr, dX.data_ptr(), y_ref.data_ptr(), B, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    return y_new.cpu().numpy().view(DT[sr]), y_ref.cpu().numpy().view(DT[sr])


def oracle_plustimes(s, X):
    V = s["V"].astype(np.float32).astype(np.float64)
    return np.stack([s["sched"].sweep_f64(0, V, X[:, b], s["rows"], s["cols"]) for b in range(X.shape[1])], axis=1)


@pytest.mark.parametrize("B", [1, 3, 8, 12, 32])
def test_noalloc_matches_oracle_and_engine_plustimes(setup, B):
    """B = 3 and 12 take the generic lane-count kernels, 1 / 8 / 32 the shifted ones."""
    rng = np.random.default_rng(B)
    for call in range(2):  # two calls in a row share the static scratch
        X = rng.uniform(-1, 1, (setup["cols"], B)).astype(np.float32)
        y_new, y_ref = run_both(setup, 0, X, B)
        assert relmax(y_new, oracle_plustimes(setup, X)) <= TOL, call
        assert relmax(y_new, y_ref) <= TOL, (call, relmax(y_new, y_ref))


def test_noalloc_matches_oracle_and_engine_boolean_tropical(setup):
    rng = np.random.default_rng(7)
    V32 = setup["V"].astype(np.float32)
    for call in range(2):
        bits = rng.random((setup["cols"], 64)) < 0.05
        a, b = run_both(setup, 1, gmr.pack_bits(bits), 64)
        np.testing.assert_array_equal(a, b)
        got = gmr.unpack_bits(a, 64)
        for c in (0, 17, 63):
            ref = setup["sched"].cpu_reference(1, V32, bits[:, c].astype(np.float32), setup["rows"], setup["cols"])
            np.testing.assert_array_equal(got[:, c], ref)
        Xt = rng.integers(0, 1000, (setup["cols"], 4)).astype(np.int32)
        Xt[rng.random(Xt.shape) < 0.3] = 2**31 - 1
        a, b = run_both(setup, 2, Xt, 4)
        np.testing.assert_array_equal(a, b)
        for c in range(4):
            x = np.minimum(Xt[:, c].astype(np.float64), 1e9).astype(np.float32)
            np.testing.assert_array_equal(a[:, c], setup["sched"].cpu_reference(2, V32, x, setup["rows"],
                                                                                setup["cols"]))


def test_noalloc_runlength_coefficients():
    """A plan with a run-length rule passes its coefficients (op_c)."""
    torch = pytest.importorskip("torch")
    g = gmr.Grammar.from_arrays(5, [[1, 2], [3, 5], [6, 0], [7, 5]], [8, 0], [1.5, 2.5], kinds=[0, 0, 1, 0],
                                reps=[1, 1, 3, 1])
    plan = gmr.Plan.build(g, 2, 3)
    assert plan.stats["has_coeff"]
    dp, keep, host = device_plan(torch, plan)
    s = dict(torch=torch, dp=dp)
    X = np.array([[0.5, 1.0], [-0.5, 2.0], [1.0, -1.0]], np.float32)
    dX = torch.from_numpy(X).cuda()
    dY = torch.zeros((2, 2), dtype=torch.float32, device="cuda")
    for _ in range(2):
        noalloc(s, 0, dX, dY, 2)
        torch.cuda.synchronize()
        np.testing.assert_allclose(dY.cpu().numpy(), gmr.Engine(plan).multiply(X, 0), rtol=1e-6)
    np.testing.assert_allclose(dY.cpu().numpy()[:, 0], [4.5, 0.0], atol=1e-6)  # cpu_selftest unit grammar


def test_noalloc_leaves_free_memory_unchanged(setup):
    """After the first call on the device (the set-up), calls change the
    device's free memory by nothing: no allocation, no code loading."""
    torch = setup["torch"]
    rng = np.random.default_rng(11)
    B = 8
    dX = torch.from_numpy(rng.uniform(-1, 1, (setup["cols"], B)).astype(np.float32)).cuda()
    dY = torch.zeros((setup["rows"], B), dtype=torch.float32, device="cuda")
    noalloc(setup, 0, dX, dY, B)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for sr, b in ((0, B), (0, 3), (2, 8), (1, 64), (0, 1)):  # other semirings and widths too
        noalloc(setup, sr, dX, dY, b)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_oversize(setup):
    dp = L.DevicePlan.from_buffer_copy(setup["dp"])
    big = np.array([0, 1 << 30], dtype=np.int64)  # a level of 2^30 rules: far beyond 64 MiB of scratch
    dp.lvl_off = big.ctypes.data
    dp.depth, dp.n_ops = 1, 1 << 30
    rc = gmr.lib().gmr_multiply_noalloc(C.byref(dp), 0, C.c_void_p(16), C.c_void_p(16), 32, None)
    assert rc == 6 and b"exceeds the static" in gmr.lib().gmr_last_error()
