// Learned cost model for the per-launch kernel-variant choice.
//
// Per launch slot (the launch of level k: rules of level k + emissions of
// level k-1) the plan yields GMR_N_BASE_FEATURES features: rule count,
// emission and row-segment counts, emissions per segment, emission fan-out
// (emissions per distinct source), the child-distance histogram of the
// level's rules, the size of the previous level's values at this B, the
// semiring, the position in the sweep and whether terminals are evaluated
// in place.  The model input is those features
// plus a one-hot of the kernel variant; the output is log(time in us).
//
// The model is a fully connected ReLU network, in -> 64 -> 64 -> 64 -> 1, in
// fp32.  Forward, backward (mean squared error), Adam and inference are the
// kernels below; training runs on the GPU.  It only chooses schedules: every
// variant computes the same Y.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "gmr_internal.h"

namespace gmr {

#define GMR_LCUDA(call)                                                                                \
    do {                                                                                               \
        cudaError_t err_ = (call);                                                                     \
        if (err_ != cudaSuccess)                                                                       \
            throw ::gmr::Error(GMR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(err_));   \
    } while (0)

// ------------------------------------------------------------------ kernels
// Z = A W^T + b, A: [N][in], W: [out][in]; relu != 0 applies max(0, .).
__global__ void k_dense_fwd(const float* __restrict__ A, const float* __restrict__ W, const float* __restrict__ b,
                            float* __restrict__ Z, int N, int in, int out, int relu) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)N * out) return;
    const int n = (int)(t / out), o = (int)(t % out);
    const float* a = A + (int64_t)n * in;
    const float* w = W + (int64_t)o * in;
    float acc = b[o];
    for (int i = 0; i < in; ++i) acc = fmaf(a[i], w[i], acc);
    Z[t] = relu ? fmaxf(acc, 0.0f) : acc;
}

// dY = 2 (Y - T) / N and per-thread squared errors (for the loss).
__global__ void k_mse_grad(const float* Y, const float* T, float* dY, float* sq, int N) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const float d = Y[n] - T[n];
    dY[n] = 2.0f * d / (float)N;
    sq[n] = d * d;
}

// dA[n][i] = sum_o dZ[n][o] W[o][i], masked by the ReLU of A (A > 0).
__global__ void k_dense_bwd_data(const float* __restrict__ dZ, const float* __restrict__ W,
                                 const float* __restrict__ A, float* __restrict__ dA, int N, int in, int out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)N * in) return;
    const int n = (int)(t / in), i = (int)(t % in);
    float acc = 0.0f;
    for (int o = 0; o < out; ++o) acc = fmaf(dZ[(int64_t)n * out + o], W[(int64_t)o * in + i], acc);
    dA[t] = A[t] > 0.0f ? acc : 0.0f;
}

// dW[o][i] = sum_n dZ[n][o] A[n][i], db[o] = sum_n dZ[n][o]; block per (o, i-chunk).
__global__ void k_dense_bwd_weight(const float* __restrict__ dZ, const float* __restrict__ A, float* __restrict__ dW,
                                   float* __restrict__ db, int N, int in, int out) {
    const int o = blockIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;  // i == in: the bias
    float acc = 0.0f;
    if (i <= in) {
        for (int n = threadIdx.x; n < N; n += blockDim.x) {
            const float g = dZ[(int64_t)n * out + o];
            acc = fmaf(g, i < in ? A[(int64_t)n * in + i] : 1.0f, acc);
        }
    }
    for (int d = 16; d > 0; d >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, d);
    if (threadIdx.x == 0 && i <= in) {
        if (i < in) dW[(int64_t)o * in + i] = acc;
        else db[o] = acc;
    }
}

__global__ void k_adam(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float gt = g[t];
    const float mt = b1 * m[t] + (1.0f - b1) * gt;
    const float vt = b2 * v[t] + (1.0f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    p[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
}

__global__ void k_gather_rows(const float* X, const float* T, const int* idx, float* Xb, float* Tb, int n, int in) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)n * (in + 1)) return;
    const int r = (int)(t / (in + 1)), c = (int)(t % (in + 1));
    const int src = idx[r];
    if (c < in) Xb[(int64_t)r * in + c] = X[(int64_t)src * in + c];
    else Tb[r] = T[src];
}

// (x - mean) / std per feature, in place.
__global__ void k_normalize(float* X, const float* mean, const float* inv_std, int N, int in) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)N * in) return;
    const int c = (int)(t % in);
    X[t] = (X[t] - mean[c]) * inv_std[c];
}

static int nblk(int64_t n, int tpb = 256) { return (int)std::max<int64_t>(1, (n + tpb - 1) / tpb); }

struct DBuf {
    float* p = nullptr;
    size_t n = 0;
    void ensure(size_t k) {
        if (k <= n) return;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        GMR_LCUDA(cudaMalloc(&p, std::max<size_t>(k, 1) * sizeof(float)));
        n = k;
    }
    ~DBuf() {
        if (p) cudaFree(p);
    }
};

static uint32_t crc32(const unsigned char* d, size_t n) {  // IEEE 802.3 polynomial, bitwise
    uint32_t c = 0xffffffffu;
    for (size_t i = 0; i < n; ++i) {
        c ^= d[i];
        for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xedb88320u & (0u - (c & 1u)));
    }
    return ~c;
}

}  // namespace gmr

// ------------------------------------------------------------------ model
struct gmr_mlp {
    int in = 0, hidden = 64, layers = 3;  // hidden layers
    std::vector<float> params;            // [W1 b1 W2 b2 ... Wout bout]
    std::vector<float> mean, inv_std;     // input normalisation
    std::vector<int> dims() const {
        std::vector<int> d{in};
        for (int l = 0; l < layers; ++l) d.push_back(hidden);
        d.push_back(1);
        return d;
    }
    // offsets of W_l and b_l in params
    std::vector<size_t> offsets() const {
        auto d = dims();
        std::vector<size_t> off;
        size_t o = 0;
        for (size_t l = 0; l + 1 < d.size(); ++l) {
            off.push_back(o);
            o += (size_t)d[l] * d[l + 1];
            off.push_back(o);
            o += d[l + 1];
        }
        off.push_back(o);
        return off;
    }
};

namespace gmr {

// Device-side forward (and optionally backward) over N rows of normalised input.
struct MlpRun {
    const gmr_mlp& m;
    std::vector<int> d;
    std::vector<size_t> off;
    DBuf P, G, acts, grads;
    std::vector<size_t> act_off;
    explicit MlpRun(const gmr_mlp& mm) : m(mm), d(mm.dims()), off(mm.offsets()) {
        P.ensure(m.params.size());
        G.ensure(m.params.size());
        GMR_LCUDA(cudaMemcpy(P.p, m.params.data(), m.params.size() * 4, cudaMemcpyHostToDevice));
    }
    void layout(int N) {
        act_off.clear();
        size_t o = 0;
        for (int w : d) {
            act_off.push_back(o);
            o += (size_t)N * w;
        }
        acts.ensure(o);
        grads.ensure(o);
    }
    // X (device, normalised) -> acts; returns pointer to outputs [N]
    float* forward(const float* X, int N) {
        layout(N);
        GMR_LCUDA(cudaMemcpy(acts.p, X, (size_t)N * d[0] * 4, cudaMemcpyDeviceToDevice));
        for (size_t l = 0; l + 1 < d.size(); ++l) {
            const bool last = l + 2 == d.size();
            k_dense_fwd<<<nblk((int64_t)N * d[l + 1]), 256>>>(acts.p + act_off[l], P.p + off[2 * l], P.p + off[2 * l + 1],
                                                             acts.p + act_off[l + 1], N, d[l], d[l + 1], last ? 0 : 1);
        }
        GMR_LCUDA(cudaGetLastError());
        return acts.p + act_off.back();
    }
    // after forward: gradients of mean squared error against T into G
    float backward(const float* T, int N, DBuf& sq, bool want_loss = true) {
        sq.ensure(N);
        float* Y = acts.p + act_off.back();
        float* dY = grads.p + act_off.back();
        k_mse_grad<<<nblk(N), 256>>>(Y, T, dY, sq.p, N);
        for (size_t l = d.size() - 1; l >= 1; --l) {
            const int in = d[l - 1], out = d[l];
            float* dZ = grads.p + act_off[l];
            dim3 blk(32, 8), grd(out, (in + 1 + 7) / 8);
            k_dense_bwd_weight<<<grd, blk>>>(dZ, acts.p + act_off[l - 1], G.p + off[2 * (l - 1)],
                                             G.p + off[2 * (l - 1) + 1], N, in, out);
            if (l >= 2)
                k_dense_bwd_data<<<nblk((int64_t)N * in), 256>>>(dZ, P.p + off[2 * (l - 1)], acts.p + act_off[l - 1],
                                                                 grads.p + act_off[l - 1], N, in, out);
        }
        GMR_LCUDA(cudaGetLastError());
        if (!want_loss) return 0.0f;
        std::vector<float> h(N);
        GMR_LCUDA(cudaMemcpy(h.data(), sq.p, (size_t)N * 4, cudaMemcpyDeviceToHost));
        double s = 0;
        for (float v : h) s += v;
        return (float)(s / std::max(N, 1));
    }
};

static void upload_normalised(const gmr_mlp& m, const float* hX, int N, DBuf& X) {
    X.ensure((size_t)N * m.in);
    GMR_LCUDA(cudaMemcpy(X.p, hX, (size_t)N * m.in * 4, cudaMemcpyHostToDevice));
    DBuf mu, is;
    mu.ensure(m.in);
    is.ensure(m.in);
    GMR_LCUDA(cudaMemcpy(mu.p, m.mean.data(), (size_t)m.in * 4, cudaMemcpyHostToDevice));
    GMR_LCUDA(cudaMemcpy(is.p, m.inv_std.data(), (size_t)m.in * 4, cudaMemcpyHostToDevice));
    k_normalize<<<nblk((int64_t)N * m.in), 256>>>(X.p, mu.p, is.p, N, m.in);
    GMR_LCUDA(cudaGetLastError());
}

}  // namespace gmr

using namespace gmr;

extern "C" int gmr_mlp_create(int in_dim, int hidden, int layers, uint64_t seed, gmr_mlp** out) {
    return guarded([&] {
        if (!out || in_dim < 1 || hidden < 1 || layers < 1 || in_dim > 4096 || hidden > 1024 || layers > 8)
            throw Error(GMR_ERR_ARG, "bad model shape");
        auto m = std::make_unique<gmr_mlp>();
        m->in = in_dim;
        m->hidden = hidden;
        m->layers = layers;
        auto d = m->dims();
        auto off = m->offsets();
        m->params.assign(off.back(), 0.0f);
        std::mt19937_64 rng(seed);
        for (size_t l = 0; l + 1 < d.size(); ++l) {  // He initialisation, zero biases
            std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (float)d[l]));
            for (size_t k = off[2 * l]; k < off[2 * l + 1]; ++k) m->params[k] = nd(rng);
        }
        m->mean.assign(in_dim, 0.0f);
        m->inv_std.assign(in_dim, 1.0f);
        *out = m.release();
    });
}

extern "C" void gmr_mlp_free(gmr_mlp* m) { delete m; }

extern "C" int gmr_mlp_info(const gmr_mlp* m, int* in_dim, int* hidden, int* layers, int64_t* n_params) {
    return guarded([&] {
        if (!m) throw Error(GMR_ERR_ARG, "null model");
        if (in_dim) *in_dim = m->in;
        if (hidden) *hidden = m->hidden;
        if (layers) *layers = m->layers;
        if (n_params) *n_params = (int64_t)m->params.size();
    });
}

extern "C" int gmr_mlp_params(gmr_mlp* m, float* get, const float* set, int64_t n) {
    return guarded([&] {
        if (!m || n != (int64_t)m->params.size()) throw Error(GMR_ERR_ARG, "parameter count mismatch");
        if (set) std::copy(set, set + n, m->params.begin());
        if (get) std::copy(m->params.begin(), m->params.end(), get);
    });
}

extern "C" int gmr_mlp_set_norm(gmr_mlp* m, const float* mean, const float* std) {
    return guarded([&] {
        if (!m || !mean || !std) throw Error(GMR_ERR_ARG, "null argument");
        for (int i = 0; i < m->in; ++i) {
            m->mean[i] = mean[i];
            m->inv_std[i] = std[i] > 1e-12f ? 1.0f / std[i] : 1.0f;
        }
    });
}

extern "C" int gmr_mlp_predict(const gmr_mlp* m, const float* X, int N, float* Y) {
    return guarded([&] {
        if (!m || (N > 0 && (!X || !Y)) || N < 0) throw Error(GMR_ERR_ARG, "bad argument");
        if (N == 0) return;
        DBuf dX;
        upload_normalised(*m, X, N, dX);
        MlpRun run(*m);
        float* out = run.forward(dX.p, N);
        GMR_LCUDA(cudaMemcpy(Y, out, (size_t)N * 4, cudaMemcpyDeviceToHost));
    });
}

extern "C" int gmr_mlp_gradients(gmr_mlp* m, const float* X, const float* T, int N, float* grad, int64_t n,
                                 float* loss) {
    return guarded([&] {
        if (!m || !X || !T || !grad || N < 1 || n != (int64_t)m->params.size()) throw Error(GMR_ERR_ARG, "bad argument");
        DBuf dX, dT, sq;
        upload_normalised(*m, X, N, dX);
        dT.ensure(N);
        GMR_LCUDA(cudaMemcpy(dT.p, T, (size_t)N * 4, cudaMemcpyHostToDevice));
        MlpRun run(*m);
        run.forward(dX.p, N);
        float l = run.backward(dT.p, N, sq);
        GMR_LCUDA(cudaMemcpy(grad, run.G.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
        if (loss) *loss = l;
    });
}

extern "C" int gmr_mlp_train(gmr_mlp* m, const float* X, const float* T, int N, int epochs, int batch, float lr,
                             uint64_t seed, float* loss_out) {
    return guarded([&] {
        if (!m || !X || !T || N < 1 || epochs < 1 || batch < 1) throw Error(GMR_ERR_ARG, "bad argument");
        batch = std::min(batch, N);
        DBuf dX, dT, Xb, Tb, M, Vv, sq;
        DBuf idx_f;  // int indices stored in a float-sized buffer
        upload_normalised(*m, X, N, dX);
        dT.ensure(N);
        GMR_LCUDA(cudaMemcpy(dT.p, T, (size_t)N * 4, cudaMemcpyHostToDevice));
        Xb.ensure((size_t)batch * m->in);
        Tb.ensure(batch);
        const size_t np = m->params.size();
        M.ensure(np);
        Vv.ensure(np);
        GMR_LCUDA(cudaMemset(M.p, 0, np * 4));
        GMR_LCUDA(cudaMemset(Vv.p, 0, np * 4));
        idx_f.ensure(N);
        MlpRun run(*m);
        std::vector<int> perm(N);
        std::iota(perm.begin(), perm.end(), 0);
        std::mt19937_64 rng(seed);
        const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
        int64_t step = 0;
        for (int ep = 0; ep < epochs; ++ep) {
            std::shuffle(perm.begin(), perm.end(), rng);
            GMR_LCUDA(cudaMemcpy(idx_f.p, perm.data(), (size_t)N * 4, cudaMemcpyHostToDevice));
            for (int s = 0; s + batch <= N; s += batch) {
                k_gather_rows<<<nblk((int64_t)batch * (m->in + 1)), 256>>>(
                    dX.p, dT.p, reinterpret_cast<const int*>(idx_f.p) + s, Xb.p, Tb.p, batch, m->in);
                run.forward(Xb.p, batch);
                run.backward(Tb.p, batch, sq, false);
                ++step;
                const float c1 = 1.0f - std::pow(b1, (float)step), c2 = 1.0f - std::pow(b2, (float)step);
                k_adam<<<nblk((int64_t)np), 256>>>(run.P.p, run.G.p, M.p, Vv.p, (int)np, lr, b1, b2, eps, c1, c2);
            }
        }
        GMR_LCUDA(cudaMemcpy(m->params.data(), run.P.p, np * 4, cudaMemcpyDeviceToHost));
        if (loss_out) {
            MlpRun ev(*m);
            ev.forward(dX.p, N);
            *loss_out = ev.backward(dT.p, N, sq);
        }
    });
}

// File: magic "GMRMLP01", int32 in, hidden, layers, n_params, then mean[in],
// inv_std[in], params[n], then CRC-32 of everything before it.
extern "C" int gmr_mlp_save(const gmr_mlp* m, const char* path) {
    return guarded([&] {
        if (!m || !path) throw Error(GMR_ERR_ARG, "null argument");
        std::vector<unsigned char> buf;
        auto put = [&](const void* p, size_t n) {
            const unsigned char* c = static_cast<const unsigned char*>(p);
            buf.insert(buf.end(), c, c + n);
        };
        put("GMRMLP01", 8);
        int32_t h[4] = {m->in, m->hidden, m->layers, (int32_t)m->params.size()};
        put(h, sizeof h);
        put(m->mean.data(), m->mean.size() * 4);
        put(m->inv_std.data(), m->inv_std.size() * 4);
        put(m->params.data(), m->params.size() * 4);
        uint32_t c = crc32(buf.data(), buf.size());
        put(&c, 4);
        FILE* f = std::fopen(path, "wb");
        if (!f) throw Error(GMR_ERR_IO, std::string("cannot create ") + path);
        bool ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
        if (std::fclose(f) != 0 || !ok) throw Error(GMR_ERR_IO, std::string("short write on ") + path);
    });
}

extern "C" int gmr_mlp_load(const char* path, gmr_mlp** out) {
    return guarded([&] {
        if (!path || !out) throw Error(GMR_ERR_ARG, "null argument");
        FILE* f = std::fopen(path, "rb");
        if (!f) throw Error(GMR_ERR_IO, std::string("cannot open ") + path);
        std::vector<unsigned char> buf;
        unsigned char tmp[65536];
        size_t r;
        while ((r = std::fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + r);
        std::fclose(f);
        if (buf.size() < 8 + 16 + 4 || std::memcmp(buf.data(), "GMRMLP01", 8) != 0)
            throw Error(GMR_ERR_FORMAT, "not a gmr cost-model file");
        uint32_t c;
        std::memcpy(&c, buf.data() + buf.size() - 4, 4);
        if (crc32(buf.data(), buf.size() - 4) != c) throw Error(GMR_ERR_FORMAT, "cost-model checksum mismatch");
        int32_t h[4];
        std::memcpy(h, buf.data() + 8, 16);
        auto m = std::make_unique<gmr_mlp>();
        m->in = h[0];
        m->hidden = h[1];
        m->layers = h[2];
        if (m->in < 1 || m->hidden < 1 || m->layers < 1 || m->in > 4096 || m->hidden > 1024 || m->layers > 8)
            throw Error(GMR_ERR_FORMAT, "bad model shape");
        const size_t np = m->offsets().back();
        if ((size_t)h[3] != np || buf.size() != 8 + 16 + (size_t)(2 * m->in + np) * 4 + 4)
            throw Error(GMR_ERR_FORMAT, "cost-model size mismatch");
        const float* fp = reinterpret_cast<const float*>(buf.data() + 24);
        m->mean.assign(fp, fp + m->in);
        m->inv_std.assign(fp + m->in, fp + 2 * m->in);
        m->params.assign(fp + 2 * m->in, fp + 2 * m->in + np);
        *out = m.release();
    });
}

extern "C" int gmr_engine_choose_learned(gmr_engine* e, const gmr_plan* p, const gmr_mlp* m, int semiring, int B,
                                         float* pred, int cap) {
    return guarded([&] {
        if (!e || !p || !m) throw Error(GMR_ERR_ARG, "null argument");
        const int nf = GMR_N_BASE_FEATURES, nv = GMR_N_LEVEL_VARIANTS;
        if (m->in != nf + nv) throw Error(GMR_ERR_FORMAT, "model input size does not match the feature set");
        int slots = 0;
        std::vector<float> base((size_t)(p->depth + 2) * nf);
        int rc = gmr_plan_launch_features(p, semiring, B, base.data(), (int)base.size(), &slots);
        if (rc != GMR_OK) throw Error(rc, gmr_last_error());
        std::vector<float> X((size_t)slots * nv * (nf + nv), 0.0f), Y((size_t)slots * nv);
        for (int s = 0; s < slots; ++s)
            for (int v = 0; v < nv; ++v) {
                float* row = X.data() + ((size_t)s * nv + v) * (nf + nv);
                std::copy(base.begin() + (size_t)s * nf, base.begin() + (size_t)(s + 1) * nf, row);
                row[nf + v] = 1.0f;
            }
        rc = gmr_mlp_predict(m, X.data(), slots * nv, Y.data());
        if (rc != GMR_OK) throw Error(rc, gmr_last_error());
        std::vector<uint8_t> table(slots, 0);
        for (int s = 1; s < slots; ++s) {
            int b = 0;
            for (int v = 1; v < nv; ++v)
                if (Y[(size_t)s * nv + v] < Y[(size_t)s * nv + b]) b = v;
            table[s] = (uint8_t)b;
        }
        rc = gmr_engine_set_level_variants(e, semiring, B, table.data(), slots);
        if (rc != GMR_OK) throw Error(rc, gmr_last_error());
        if (pred) {
            if (cap < slots * nv) throw Error(GMR_ERR_RANGE, "prediction buffer too small");
            std::copy(Y.begin(), Y.end(), pred);
        }
    });
}
