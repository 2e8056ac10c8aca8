// Runs the reference's own GPU kernels on this GPU: a baseline, test
// infrastructure only.
//
// The device code is the reference's gpu-engine/gpu_engine.cu compiled to
// PTX where it lies (oracle/Makefile target _ref/gpu_engine.ptx); the CUDA
// driver loads and compiles it (cuModuleLoad).  This file restates the
// reference's host sequence around those kernels:
//   single vector  gpu_engine.cu:224-264  fill y; init_T_terminals;
//                  emit_terminals; fill W1, W2; per level eval_level_layered
//                  then emit_level; swap W
//   batched        gpu_engine.cu:516-545  the same with the *_batched kernels
// with the same kernels, grid sizes (256 threads per block) and order, timed
// with events around the `iters` repetitions as the reference times them.
// Kernels are found by the names the driver reports for the module
// (cuModuleEnumerateFunctions / cuFuncGetName).  One deliberate difference:
// buffers are device memory (cuMemAlloc) where the reference uses managed
// memory (written for unified-memory parts); device memory is the
// reference's best case on a discrete-memory GPU.
#include <cuda.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_err;

struct Fail {
    std::string msg;
};

void check(CUresult r, const char* what) {
    if (r != CUDA_SUCCESS) {
        const char* s = nullptr;
        cuGetErrorString(r, &s);
        throw Fail{std::string(what) + ": " + (s ? s : "unknown error")};
    }
}

struct Kernels {
    CUfunction fill = nullptr, init_T = nullptr, eval = nullptr, emit = nullptr, emit_term = nullptr;
    CUfunction init_T_b = nullptr, eval_b = nullptr, emit_b = nullptr, emit_term_b = nullptr;
};

struct Ref {
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    CUdevice dev = 0;
    Kernels k[3];  // PlusTimes, Boolean, Tropical (gpu_engine.h:46-97)
};

Ref* g_ref = nullptr;

// Mangled-name pieces: <len><identifier>I<len><semiring> for the templates.
const char* kSemiring[3] = {"9PlusTimes", "7Boolean", "8Tropical"};

bool has(const std::string& name, const std::string& kernel, const std::string& arg) {
    return name.find(kernel + "I" + arg) != std::string::npos;
}

struct Buf {
    CUdeviceptr p = 0;
    explicit Buf(size_t bytes) {
        if (bytes) check(cuMemAlloc(&p, bytes), "cuMemAlloc");
    }
    Buf(const void* h, size_t bytes) : Buf(bytes) {
        if (bytes) check(cuMemcpyHtoD(p, h, bytes), "cuMemcpyHtoD");
    }
    ~Buf() {
        if (p) cuMemFree(p);
    }
};

void launch(CUfunction f, long work, void** args) {
    const unsigned blocks = (unsigned)((work + 255) / 256);
    if (blocks == 0) return;
    check(cuLaunchKernel(f, blocks, 1, 1, 256, 1, 1, 0, nullptr, args, nullptr), "cuLaunchKernel");
}

}  // namespace

extern "C" const char* refgpu_error() { return g_err.c_str(); }

extern "C" int refgpu_open(const char* ptx_path, int device) {
    try {
        if (g_ref) return 0;
        auto* r = new Ref();
        check(cuInit(0), "cuInit");
        check(cuDeviceGet(&r->dev, device), "cuDeviceGet");
        check(cuDevicePrimaryCtxRetain(&r->ctx, r->dev), "cuDevicePrimaryCtxRetain");
        check(cuCtxSetCurrent(r->ctx), "cuCtxSetCurrent");
        check(cuModuleLoad(&r->mod, ptx_path), "cuModuleLoad");
        unsigned n = 0;
        check(cuModuleGetFunctionCount(&n, r->mod), "cuModuleGetFunctionCount");
        std::vector<CUfunction> fs(n);
        check(cuModuleEnumerateFunctions(fs.data(), n, r->mod), "cuModuleEnumerateFunctions");
        for (CUfunction f : fs) {
            const char* c = nullptr;
            check(cuFuncGetName(&c, f), "cuFuncGetName");
            const std::string name = c ? c : "";
            for (int s = 0; s < 3; ++s) {
                Kernels& k = r->k[s];
                const std::string S = kSemiring[s];
                if (has(name, "17fill_array_kernel", s == 0 ? "f" : "i")) k.fill = f;
                if (has(name, "16init_T_terminals", S)) k.init_T = f;
                if (has(name, "18eval_level_layered", S)) k.eval = f;
                if (has(name, "10emit_level", S)) k.emit = f;
                if (has(name, "14emit_terminals", S)) k.emit_term = f;
                if (has(name, "14init_T_batched", S)) k.init_T_b = f;
                if (has(name, "18eval_level_batched", S)) k.eval_b = f;
                if (has(name, "18emit_level_batched", S)) k.emit_b = f;
                if (has(name, "22emit_terminals_batched", S)) k.emit_term_b = f;
            }
        }
        for (auto& k : r->k)
            if (!k.fill || !k.init_T || !k.eval || !k.emit || !k.emit_term || !k.init_T_b || !k.eval_b || !k.emit_b ||
                !k.emit_term_b)
                throw Fail{"a reference kernel is missing from the module"};
        g_ref = r;
        return 0;
    } catch (const Fail& f) {
        g_err = f.msg;
        return 1;
    }
}

// One reference multiply, repeated `iters` times; Y receives the last one.
// rules: (left, right, coeff) x n_rules, the reference's LayeredRule layout
// (layered_types.h:45-49).  X: cols x B floats, Y: rows x B words (float for
// semiring 0, int otherwise).  B == 1 runs the single-vector kernels.
extern "C" int refgpu_run(int semiring, int rows, int cols, int alpha, int n_rules, const void* rules,
                          const int* val_idx, const int* col_idx, const float* V, int n_vals, int depth,
                          int max_width, const int* level_offsets, const int* emit_offsets, const int* emit_pos,
                          const int* emit_row, int emit_total, const int* term_sym, const int* term_row,
                          int n_term, const float* X, void* Y, int B, int iters, float* ms_total) {
    try {
        if (!g_ref) throw Fail{"refgpu_open first"};
        if (semiring < 0 || semiring > 2 || B < 1 || iters < 1) throw Fail{"bad argument"};
        check(cuCtxSetCurrent(g_ref->ctx), "cuCtxSetCurrent");
        const Kernels& k = g_ref->k[semiring];
        const size_t w = 4;  // float or int
        const long Bl = B;
        Buf dT((size_t)alpha * Bl * w), dRules(rules, (size_t)n_rules * 12);
        Buf dVi(val_idx, (size_t)(alpha - 1) * 4), dCi(col_idx, (size_t)(alpha - 1) * 4);
        Buf dV(V, (size_t)n_vals * 4), dX(X, (size_t)cols * Bl * 4), dY((size_t)rows * Bl * w);
        Buf dW1((size_t)max_width * Bl * w), dW2((size_t)max_width * Bl * w);
        Buf dEp(emit_pos, (size_t)emit_total * 4), dEr(emit_row, (size_t)emit_total * 4);
        Buf dTs(term_sym, (size_t)n_term * 4), dTr(term_row, (size_t)n_term * 4);
        // S::zero() (gpu_engine.h:48, 61, 79)
        const float zf = 0.0f;
        const int zi = semiring == 2 ? 1000000000 : 0;
        const void* zero = semiring == 0 ? (const void*)&zf : (const void*)&zi;
        auto fill = [&](CUdeviceptr p, long n) {
            if (n <= 0) return;
            void* args[] = {&p, const_cast<void*>(zero), &n};
            launch(k.fill, n, args);
        };
        CUevent e0, e1;
        check(cuEventCreate(&e0, CU_EVENT_DEFAULT), "cuEventCreate");
        check(cuEventCreate(&e1, CU_EVENT_DEFAULT), "cuEventCreate");
        check(cuEventRecord(e0, nullptr), "cuEventRecord");
        for (int it = 0; it < iters; ++it) {
            CUdeviceptr T = dT.p, Vp = dV.p, Xp = dX.p, vi = dVi.p, ci = dCi.p, y = dY.p;
            CUdeviceptr ts = dTs.p, tr = dTr.p;
            fill(y, (long)rows * Bl);
            int a = alpha, nt = n_term, b = B;
            if (B == 1) {
                void* ai[] = {&T, &Vp, &Xp, &vi, &ci, &a};
                launch(k.init_T, alpha, ai);
                if (n_term > 0) {
                    void* at[] = {&ts, &tr, &T, &y, &nt};
                    launch(k.emit_term, n_term, at);
                }
            } else {
                void* ai[] = {&T, &Vp, &Xp, &vi, &ci, &a, &b};
                launch(k.init_T_b, (long)alpha * Bl, ai);
                if (n_term > 0) {
                    void* at[] = {&ts, &tr, &T, &y, &nt, &b};
                    launch(k.emit_term_b, (long)n_term * Bl, at);
                }
            }
            CUdeviceptr rd = dW1.p, wr = dW2.p;
            fill(rd, (long)max_width * Bl);
            fill(wr, (long)max_width * Bl);
            for (int lv = 1; lv <= depth; ++lv) {
                int nr = level_offsets[lv] - level_offsets[lv - 1];
                int ne = emit_offsets[lv] - emit_offsets[lv - 1];
                CUdeviceptr rp = dRules.p + (CUdeviceptr)level_offsets[lv - 1] * 12;
                CUdeviceptr ep = dEp.p + (CUdeviceptr)emit_offsets[lv - 1] * 4;
                CUdeviceptr er = dEr.p + (CUdeviceptr)emit_offsets[lv - 1] * 4;
                if (nr > 0) {
                    if (B == 1) {
                        void* ae[] = {&rp, &rd, &wr, &T, &nr};
                        launch(k.eval, nr, ae);
                    } else {
                        void* ae[] = {&rp, &rd, &wr, &T, &nr, &b};
                        launch(k.eval_b, (long)nr * Bl, ae);
                    }
                }
                if (ne > 0) {
                    if (B == 1) {
                        void* am[] = {&ep, &er, &wr, &y, &ne};
                        launch(k.emit, ne, am);
                    } else {
                        void* am[] = {&ep, &er, &wr, &y, &ne, &b};
                        launch(k.emit_b, (long)ne * Bl, am);
                    }
                }
                CUdeviceptr t = rd;
                rd = wr;
                wr = t;
            }
        }
        check(cuEventRecord(e1, nullptr), "cuEventRecord");
        check(cuEventSynchronize(e1), "cuEventSynchronize");
        float ms = 0.0f;
        check(cuEventElapsedTime(&ms, e0, e1), "cuEventElapsedTime");
        cuEventDestroy(e0);
        cuEventDestroy(e1);
        check(cuMemcpyDtoH(Y, dY.p, (size_t)rows * Bl * w), "cuMemcpyDtoH");
        if (ms_total) *ms_total = ms;
        return 0;
    } catch (const Fail& f) {
        g_err = f.msg;
        return 1;
    }
}
