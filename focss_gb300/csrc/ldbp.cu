// ldbp.cu -- learned digital back-propagation: forward and backward kernels.
//
// Model (per realization, field at 2 samples/symbol, N samples):
//   for each span s:   x *= span_scale                         (Amplifier::drop_power)
//     for each step i: x = FIR(x, h[s,i])                       (learned dispersion filter)
//                      x = x * exp(i xi[s,i] |x|^2)             (learned nonlinear gain)
//   y = FIR(x, h_mf);  symbols = y[0::2]                          (learned matched filter)
// FIR(x, h)[n] = sum_{t<T} h[t] x[(n + t - c) mod N], c = (T-1)/2 (circular).
// It replaces the many-step split-step DBP of backward_propagation
// (src/tasks/systems.cpp:73-91) with few learned steps per span; plain DBP is
// its initialisation, its fallback and the yardstick of its Q.
//
// Gradients use the Wirtinger convention g = dL/d(conj z) for complex values;
// for real parameters dL/dxi is returned.  Loss: L = mean_k |symbols_k - t_k|^2.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace fg {

constexpr int FIR_THREADS = 128;                    // fir_kernel
constexpr int FIR_GRAD_THREADS = 256;               // fir_grad_taps_kernel: 8 warps x 8 taps
constexpr int FIR_OUT = 4;                          // consecutive outputs per thread
constexpr int FIR_TILE = FIR_THREADS * FIR_OUT;     // outputs per CTA of fir_kernel
constexpr int FIR_GRAD_TILE = 2048;                 // samples per CTA of fir_grad_taps_kernel
constexpr int FIR_MAX_TAPS = 255;
constexpr int FIR_TAPS_PAD = (FIR_MAX_TAPS + 7) / 8 * 8;
// Shared-memory sample windows keep one padding slot after every R samples,
// R the run a thread reads from a multiple of R: runs of 4 (forward) start
// 40 bytes apart across a half-warp and runs of 8 (tap gradient) 72 bytes
// apart, both on distinct bank pairs.
template <int R>
__device__ __forceinline__ int fir_pad(int i) { return i + i / R; }
constexpr int FIR_XS = (FIR_TILE + FIR_TAPS_PAD + 8) * (FIR_OUT + 1) / FIR_OUT;
constexpr int FIR_GRAD_XS = (FIR_GRAD_TILE + FIR_TAPS_PAD + 8) * 9 / 8;

// Loads samples [n0 - c, n0 - c + span) of one realization (circular) into
// the padded window: all of a thread's loads are issued before the first
// store (a load-store loop would wait for one load latency per iteration).
template <int THREADS, int TILE, int R>
__device__ __forceinline__ void fir_load_window(float2* xs, const float2* __restrict__ xb, int n0, int c, int span,
                                                int N) {
    constexpr int K = (TILE + FIR_TAPS_PAD + THREADS - 1) / THREADS;
    float2 v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int i = threadIdx.x + k * THREADS;
        if (i < span) {
            int s = n0 - c + i;
            if (s < 0 || s >= N) {
                s %= N;
                if (s < 0) s += N;
            }
            v[k] = xb[s];
        }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int i = threadIdx.x + k * THREADS;
        if (i < span) xs[fir_pad<R>(i)] = v[k];
    }
}

// y = FIR(x, h) for every realization; conj_rev: use h'[t] = conj(h[T-1-t])
// (the adjoint filter, for the input gradient).  Register-blocked: a thread
// computes 4 consecutive outputs from an 11-sample register window per 8 taps
// (taps zero-padded to a multiple of 8), so a product costs 19/32 of a
// shared-memory load instead of two; each output still sums its taps in
// ascending order with the same fused multiply-adds.
//
// Inference epilogue (both optional): the output is multiplied by `gain`
// (the span's drop_power factor, moved past the linear filter) and then
// rotated by exp(i xi |.|^2) (the step's nonlinear phase, as nl_kernel), so
// one launch does a whole learned step.
__global__ void __launch_bounds__(FIR_THREADS) fir_kernel(const float2* __restrict__ x, const float2* __restrict__ h,
                                                          int T, int conj_rev, float2* __restrict__ y, int N,
                                                          float gain, const float* __restrict__ xi) {
    __shared__ float2 xs[FIR_XS];
    __shared__ float2 hs[FIR_TAPS_PAD];
    const int b = blockIdx.y;
    const int n0 = blockIdx.x * FIR_TILE;
    const int c = (T - 1) / 2;
    const int Tp = (T + 7) & ~7;
    for (int t = threadIdx.x; t < Tp; t += blockDim.x) {
        float2 v = make_float2(0.f, 0.f);
        if (t < T) {
            v = conj_rev ? h[T - 1 - t] : h[t];
            if (conj_rev) v.y = -v.y;
        }
        hs[t] = v;
    }
    fir_load_window<FIR_THREADS, FIR_TILE, FIR_OUT>(xs, x + (size_t)b * N, n0, c, FIR_TILE + Tp, N);
    __syncthreads();
    const int o0 = threadIdx.x * FIR_OUT;
    float2 acc[FIR_OUT];
#pragma unroll
    for (int i = 0; i < FIR_OUT; ++i) acc[i] = make_float2(0.f, 0.f);
    for (int tb = 0; tb < Tp; tb += 8) {
        constexpr int WN = FIR_OUT + 7;  // window of 8 taps x FIR_OUT outputs
        float2 w[WN], hv[8];
        const int base = ((o0 + tb) / FIR_OUT) * (FIR_OUT + 1);
#pragma unroll
        for (int j = 0; j < WN; ++j) w[j] = xs[base + j + j / FIR_OUT];
#pragma unroll
        for (int u = 0; u < 8; ++u) hv[u] = hs[tb + u];
#pragma unroll
        for (int u = 0; u < 8; ++u)
#pragma unroll
            for (int i = 0; i < FIR_OUT; ++i) {
                const float2 xv = w[i + u];
                acc[i].x = fmaf(hv[u].x, xv.x, fmaf(-hv[u].y, xv.y, acc[i].x));
                acc[i].y = fmaf(hv[u].x, xv.y, fmaf(hv[u].y, xv.x, acc[i].y));
            }
    }
    if (gain != 1.0f) {
#pragma unroll
        for (int i = 0; i < FIR_OUT; ++i) acc[i] = cscale(acc[i], gain);
    }
    if (xi) {
        const float k = *xi;
#pragma unroll
        for (int i = 0; i < FIR_OUT; ++i) acc[i] = cmul(acc[i], phase_rotation(k * cnorm(acc[i])));
    }
    float2* yb = y + (size_t)b * N + n0 + o0;
#pragma unroll
    for (int i = 0; i < FIR_OUT; ++i)
        if (n0 + o0 + i < N) yb[i] = acc[i];
}

// g_h[t] += sum_n g_y[n] conj(x[(n + t - c) mod N]) over all realizations.
// Warp w takes taps 8w .. 8w + 7 (+ 64 per round for longer filters), lane l
// the 8 consecutive samples 8l .. 8l + 7 of each 256-sample chunk of the
// 2048-sample tile: per (chunk, 8 taps) a 15-sample register window and 8 gradient
// samples give 64 products; lanes meet in a warp sum, CTAs in atomics.
__global__ void __launch_bounds__(FIR_GRAD_THREADS) fir_grad_taps_kernel(const float2* __restrict__ x,
                                                                         const float2* __restrict__ gy, int T,
                                                                         float2* __restrict__ gh, int N) {
    __shared__ float2 xs[FIR_GRAD_XS];
    __shared__ float2 gs[FIR_GRAD_TILE * 9 / 8];
    const int b = blockIdx.y;
    const int n0 = blockIdx.x * FIR_GRAD_TILE;
    const int c = (T - 1) / 2;
    const int Tp = (T + 7) & ~7;
    fir_load_window<FIR_GRAD_THREADS, FIR_GRAD_TILE, 8>(xs, x + (size_t)b * N, n0, c, FIR_GRAD_TILE + Tp, N);
    {
        constexpr int K = FIR_GRAD_TILE / FIR_GRAD_THREADS;
        float2 v[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int i = threadIdx.x + k * FIR_GRAD_THREADS;
            v[k] = (n0 + i < N) ? gy[(size_t)b * N + n0 + i] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int k = 0; k < K; ++k) gs[fir_pad<8>(threadIdx.x + k * FIR_GRAD_THREADS)] = v[k];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t0 = warp * 8; t0 < Tp; t0 += 64) {
        float2 acc[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[j] = make_float2(0.f, 0.f);
        for (int q = 0; q < FIR_GRAD_TILE; q += 256) {
            const int nl = q + 8 * lane;  // first local sample of this lane
            float2 g[8], w[16];
            const int gb = (nl >> 3) * 9, xb = ((nl + t0) >> 3) * 9;
#pragma unroll
            for (int i = 0; i < 8; ++i) g[i] = gs[gb + i];
#pragma unroll
            for (int k = 0; k < 15; ++k) w[k] = xs[xb + k + (k >> 3)];
#pragma unroll
            for (int j = 0; j < 8; ++j)
#pragma unroll
                for (int i = 0; i < 8; ++i) acc[j] = cadd(acc[j], cmulc(g[i], w[i + j]));
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float sx = warp_sum(acc[j].x), sy = warp_sum(acc[j].y);
            if (lane == 0 && t0 + j < T) {
                atomicAdd(&gh[t0 + j].x, sx);
                atomicAdd(&gh[t0 + j].y, sy);
            }
        }
    }
}

// y = x exp(i xi |x|^2)
__global__ void nl_kernel(const float2* __restrict__ x, const float* __restrict__ xi, float2* __restrict__ y,
                          size_t n) {
    const float k = *xi;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        y[i] = cmul(x[i], phase_rotation(k * cnorm(x[i])));
}

// Backward of y = x e^{i phi}, phi = xi |x|^2:
//   g_x = g_y e^{-i phi} (1 - i xi p) + conj(g_y) i xi x^2 e^{i phi}
//   dL/dxi = 2 Re(conj(g_y) i p y)
__global__ void nl_grad_kernel(const float2* __restrict__ x, const float* __restrict__ xi,
                               const float2* __restrict__ gy, float2* __restrict__ gx, float* __restrict__ gxi,
                               size_t n) {
    const float k = *xi;
    float acc = 0.f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 xv = x[i], g = gy[i];
        const float p = cnorm(xv);
        const float2 e = phase_rotation(k * p);                  // e^{i phi}
        const float2 y = cmul(xv, e);
        const float2 t1 = cmul(g, make_float2(e.x, -e.y));       // g e^{-i phi}
        const float2 a = cmul(t1, make_float2(1.f, -k * p));     // (1 - i xi p)
        const float2 x2 = cmul(xv, xv);
        const float2 b = cmul(cmul(make_float2(g.x, -g.y), x2), e);  // conj(g) x^2 e^{i phi}
        gx[i] = make_float2(a.x - k * b.y, a.y + k * b.x);       // + i xi b
        // 2 Re(conj(g) * i p y) = -2 p Im(conj(g) y)
        const float2 gy_ = cmul(make_float2(g.x, -g.y), y);
        acc += -2.f * p * gy_.y;
    }
    __shared__ float red[64];
    float dummy = 0.f;
    float s = acc;
    block_max_sum(dummy, s, red);
    if (threadIdx.x == 0) atomicAdd(gxi, s);
}

// symbols = y[0::2]; loss = mean |symbols - t|^2, g_y = 0 at odd samples.
__global__ void mse_decimate_kernel(const float2* __restrict__ y, const float2* __restrict__ tx, int N,
                                    size_t n_sym_total, float inv_count, float2* __restrict__ sym,
                                    float2* __restrict__ gy, double* __restrict__ loss) {
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n_sym_total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t b = i / (N / 2), k = i % (N / 2);
        const float2 v = y[b * N + 2 * k];
        if (sym) sym[i] = v;
        if (gy) {
            const float2 d = csub(v, tx[i]);
            gy[b * N + 2 * k] = cscale(d, inv_count);
            gy[b * N + 2 * k + 1] = make_float2(0.f, 0.f);
            acc += (double)cnorm(d);
        }
    }
    __shared__ double sd[32];
    acc = block_sum_d(acc, sd);
    if (threadIdx.x == 0 && loss) atomicAdd(loss, acc * inv_count);
}

// Adam on n real parameters (complex parameters as interleaved pairs; the
// real gradient of a complex z = a + ib is (2 Re g, 2 Im g)).  Parameters in
// [alt_lo, alt_hi) (the nonlinear gains) use the learning rate lr_alt.
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                            float* __restrict__ m2, int n, float lr, float b1, float b2, float eps, float c1,
                            float c2, float gscale, int alt_lo, int alt_hi, float lr_alt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i] * gscale;
        const float a = b1 * m1[i] + (1.f - b1) * gi;
        const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = v;
        const float r = (i >= alt_lo && i < alt_hi) ? lr_alt : lr;
        p[i] -= r * (a * c1) / (sqrtf(v * c2) + eps);
    }
}

}  // namespace fg

// ---------------------------------------------------------------- model object
namespace {
struct LdbpModel {
    focss_ctx* ctx = nullptr;
    int spans = 0, steps = 0, taps = 0, mf_taps = 0, samples = 0, batch = 0;
    float span_scale = 1.f;
    int n_params = 0;        // real parameter count
    float* params = nullptr; // [h: spans*steps*taps*2][xi: spans*steps][hmf: mf_taps*2]
    float* grads = nullptr;
    float* m1 = nullptr;
    float* m2 = nullptr;
    int adam_t = 0;
    float2* acts = nullptr;  // (2*spans*steps + 1) activations of batch*samples
    float2* work = nullptr;  // 2 work buffers of batch*samples
    float2* sym = nullptr;   // batch*samples/2
    double* loss = nullptr;
    size_t field_n() const { return (size_t)batch * samples; }
    float2* h(int k) const { return (float2*)params + (size_t)k * taps; }
    float* xi(int k) const { return params + (size_t)spans * steps * taps * 2 + k; }
    // the gain section is padded to an even count so the taps after it stay 8-byte aligned
    int xi_count() const { return (spans * steps + 1) & ~1; }
    float2* hmf() const { return (float2*)(params + (size_t)spans * steps * taps * 2 + xi_count()); }
    float2* gh(int k) const { return (float2*)grads + (size_t)k * taps; }
    float* gxi(int k) const { return grads + (size_t)spans * steps * taps * 2 + k; }
    float2* ghmf() const { return (float2*)(grads + (size_t)spans * steps * taps * 2 + xi_count()); }
};

inline int gridn(size_t n) {
    size_t g = (n + 255) / 256;
    return (int)std::max<size_t>(1, std::min<size_t>(g, (size_t)fg::sm_count() * 16));
}
}  // namespace

struct focss_ldbp : LdbpModel {};

using fg::count_launch;

static focss_status ldbp_err(focss_ctx* c, cudaError_t e, const char* what) { return fg::cuda_check(c, e, what); }

static cudaError_t fir(const LdbpModel& M, const float2* x, const float2* h, int T, int conj_rev, float2* y,
                       float gain = 1.0f, const float* xi = nullptr) {
    dim3 g((M.samples + fg::FIR_TILE - 1) / fg::FIR_TILE, M.batch);
    fg::fir_kernel<<<g, fg::FIR_THREADS, 0, M.ctx->stream>>>(x, h, T, conj_rev, y, M.samples, gain, xi);
    count_launch();
    return cudaGetLastError();
}

// Inference forward pass: one launch per learned step (FIR, the span's
// drop_power factor applied to the filter output, nonlinear phase), reading
// the input field directly, then the matched filter into work[1].
static cudaError_t ldbp_infer(LdbpModel& M, const float2* in) {
    const size_t n = M.field_n();
    float2* bufs[2] = {M.work, M.work + n};
    const int layers = M.spans * M.steps;
    int w = (layers - 1) & 1;  // the last step lands in work[0]
    const float2* src = in;
    cudaError_t e = cudaSuccess;
    for (int sp = 0; sp < M.spans && e == cudaSuccess; ++sp)
        for (int st = 0; st < M.steps && e == cudaSuccess; ++st) {
            const int k = sp * M.steps + st;
            e = fir(M, src, M.h(k), M.taps, 0, bufs[w], st == 0 ? M.span_scale : 1.0f, M.xi(k));
            src = bufs[w];
            w ^= 1;
        }
    if (e == cudaSuccess) e = fir(M, src, M.hmf(), M.mf_taps, 0, M.work + n);
    return e;
}

// Forward pass; keeps every layer input in M.acts when `keep`.
static cudaError_t ldbp_forward(LdbpModel& M, const float2* in, bool keep) {
    if (!keep && M.steps > 0) return ldbp_infer(M, in);
    cudaStream_t s = M.ctx->stream;
    const size_t n = M.field_n();
    float2* cur = M.work;
    float2* nxt = M.work + n;
    cudaError_t e = cudaMemcpyAsync(cur, in, sizeof(float2) * n, cudaMemcpyDeviceToDevice, s);
    int a = 0;
    for (int sp = 0; sp < M.spans && e == cudaSuccess; ++sp) {
        e = fg::launch_scale(cur, n, make_float2(M.span_scale, 0.f), s);
        for (int st = 0; st < M.steps && e == cudaSuccess; ++st) {
            const int k = sp * M.steps + st;
            if (keep) e = cudaMemcpyAsync(M.acts + (size_t)(a++) * n, cur, sizeof(float2) * n, cudaMemcpyDeviceToDevice, s);
            if (e == cudaSuccess) e = fir(M, cur, M.h(k), M.taps, 0, nxt);
            std::swap(cur, nxt);
            if (keep && e == cudaSuccess)
                e = cudaMemcpyAsync(M.acts + (size_t)(a++) * n, cur, sizeof(float2) * n, cudaMemcpyDeviceToDevice, s);
            if (e == cudaSuccess) {
                fg::nl_kernel<<<gridn(n), 256, 0, s>>>(cur, M.xi(k), nxt, n);
                count_launch();
                e = cudaGetLastError();
            }
            std::swap(cur, nxt);
        }
    }
    if (keep && e == cudaSuccess)
        e = cudaMemcpyAsync(M.acts + (size_t)(a++) * n, cur, sizeof(float2) * n, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = fir(M, cur, M.hmf(), M.mf_taps, 0, nxt);
    // result (2 sps, before decimation) is left in work[1] when the layer count is even
    if (nxt != M.work + n && e == cudaSuccess)
        e = cudaMemcpyAsync(M.work + n, nxt, sizeof(float2) * n, cudaMemcpyDeviceToDevice, s);
    return e;
}

extern "C" {

FOCSS_API focss_status focss_ldbp_create(focss_ctx* c, int spans, int steps_per_span, int taps, int mf_taps,
                                         int samples, int batch, double span_scale, focss_ldbp** out) {
    if (!c || !out || spans <= 0 || steps_per_span <= 0 || taps <= 0 || mf_taps <= 0 || samples <= 0 || batch <= 0 ||
        samples % 2)
        return FOCSS_ERR_INVALID_ARG;
    if (taps % 2 == 0 || mf_taps % 2 == 0 || taps > fg::FIR_MAX_TAPS || mf_taps > fg::FIR_MAX_TAPS)
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "ldbp: tap counts must be odd and <= 255");
    focss_ldbp* m = new (std::nothrow) focss_ldbp();
    if (!m) return FOCSS_ERR_OOM;
    m->ctx = c;
    m->spans = spans;
    m->steps = steps_per_span;
    m->taps = taps;
    m->mf_taps = mf_taps;
    m->samples = samples;
    m->batch = batch;
    m->span_scale = (float)span_scale;
    m->n_params = spans * steps_per_span * 2 * taps + m->xi_count() + 2 * mf_taps;
    const size_t n = m->field_n();
    const size_t n_acts = (size_t)2 * spans * steps_per_span + 1;
    cudaError_t e = cudaMalloc(&m->params, sizeof(float) * 4 * (size_t)m->n_params);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->params, 0, sizeof(float) * 4 * (size_t)m->n_params, c->stream);
    m->grads = m->params + m->n_params;
    m->m1 = m->grads + m->n_params;
    m->m2 = m->m1 + m->n_params;
    if (e == cudaSuccess) e = cudaMalloc(&m->acts, sizeof(float2) * n * n_acts);
    if (e == cudaSuccess) e = cudaMalloc(&m->work, sizeof(float2) * n * 3);
    m->sym = m->work + 2 * n;
    if (e == cudaSuccess) e = cudaMalloc(&m->loss, sizeof(double) * 2);
    if (e != cudaSuccess) {
        cudaFree(m->params);
        cudaFree(m->acts);
        cudaFree(m->work);
        cudaFree(m->loss);
        delete m;
        return ldbp_err(c, e, "ldbp alloc");
    }
    *out = m;
    return FOCSS_OK;
}

FOCSS_API focss_status focss_ldbp_destroy(focss_ldbp* m) {
    if (!m) return FOCSS_OK;
    cudaStreamSynchronize(m->ctx->stream);
    cudaFree(m->params);
    cudaFree(m->acts);
    cudaFree(m->work);
    cudaFree(m->loss);
    delete m;
    return FOCSS_OK;
}

FOCSS_API int focss_ldbp_num_params(const focss_ldbp* m) { return m ? m->n_params : 0; }

FOCSS_API focss_status focss_ldbp_set_params(focss_ldbp* m, const float* host, int n) {
    if (!m || !host || n != m->n_params) return FOCSS_ERR_INVALID_ARG;
    cudaError_t e = cudaMemcpyAsync(m->params, host, sizeof(float) * n, cudaMemcpyHostToDevice, m->ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->m1, 0, sizeof(float) * 2 * n, m->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->ctx->stream);
    m->adam_t = 0;
    return ldbp_err(m->ctx, e, "ldbp set params");
}

FOCSS_API focss_status focss_ldbp_get_params(focss_ldbp* m, float* host, float* grads, int n) {
    if (!m || n != m->n_params) return FOCSS_ERR_INVALID_ARG;
    cudaError_t e = cudaSuccess;
    if (host) e = cudaMemcpyAsync(host, m->params, sizeof(float) * n, cudaMemcpyDeviceToHost, m->ctx->stream);
    if (grads && e == cudaSuccess)
        e = cudaMemcpyAsync(grads, m->grads, sizeof(float) * n, cudaMemcpyDeviceToHost, m->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->ctx->stream);
    return ldbp_err(m->ctx, e, "ldbp get params");
}

FOCSS_API focss_status focss_ldbp_forward(focss_ldbp* m, const focss_field* in, focss_field* symbols) {
    if (!m || !in || !symbols) return FOCSS_ERR_INVALID_ARG;
    if (in->modes != 1 || in->samples != m->samples || in->batch != m->batch || symbols->modes != 1 ||
        symbols->samples != m->samples / 2 || symbols->batch != m->batch)
        return fg::set_error(m->ctx, FOCSS_ERR_INVALID_ARG, "ldbp_forward: shapes");
    cudaError_t e = ldbp_forward(*m, in->d, false);
    const size_t ns = (size_t)m->batch * (m->samples / 2);
    if (e == cudaSuccess) {
        fg::mse_decimate_kernel<<<gridn(ns), 256, 0, m->ctx->stream>>>(m->work + m->field_n(), nullptr, m->samples, ns,
                                                                       1.f, symbols->d, nullptr, nullptr);
        count_launch();
        e = cudaGetLastError();
    }
    return ldbp_err(m->ctx, e, "ldbp forward");
}

// One forward + backward over the batch: gradients into the model (overwritten),
// loss (mean |symbols - tx|^2) returned.
FOCSS_API focss_status focss_ldbp_loss_grad(focss_ldbp* m, const focss_field* in, const focss_field* tx,
                                            double* loss) {
    if (!m || !in || !tx) return FOCSS_ERR_INVALID_ARG;
    if (in->modes != 1 || in->samples != m->samples || in->batch != m->batch || tx->modes != 1 ||
        tx->samples != m->samples / 2 || tx->batch != m->batch)
        return fg::set_error(m->ctx, FOCSS_ERR_INVALID_ARG, "ldbp_loss_grad: shapes");
    cudaStream_t s = m->ctx->stream;
    const size_t n = m->field_n();
    const size_t ns = (size_t)m->batch * (m->samples / 2);
    cudaError_t e = ldbp_forward(*m, in->d, true);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->grads, 0, sizeof(float) * m->n_params, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->loss, 0, sizeof(double), s);
    float2* g = m->work;           // gradient w.r.t. the current layer output
    float2* g2 = m->work + n;      // (work[1] holds y; reused after the loss)
    float2* ybuf = m->work + n;
    if (e == cudaSuccess) {
        // y lives in work[1]; write the output gradient into work[0]
        fg::mse_decimate_kernel<<<gridn(ns), 256, 0, s>>>(ybuf, tx->d, m->samples, ns, 1.f / (float)ns, m->sym, g,
                                                          m->loss);
        count_launch();
        e = cudaGetLastError();
    }
    const int L = m->spans * m->steps;
    int a = 2 * L;  // index of the matched filter's input activation
    dim3 gg((m->samples + fg::FIR_GRAD_TILE - 1) / fg::FIR_GRAD_TILE, m->batch);
    // matched filter
    if (e == cudaSuccess) {
        fg::fir_grad_taps_kernel<<<gg, fg::FIR_GRAD_THREADS, 0, s>>>(m->acts + (size_t)a * n, g, m->mf_taps, m->ghmf(), m->samples);
        count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = fir(*m, g, m->hmf(), m->mf_taps, 1, g2);
    std::swap(g, g2);
    for (int sp = m->spans - 1; sp >= 0 && e == cudaSuccess; --sp) {
        for (int st = m->steps - 1; st >= 0 && e == cudaSuccess; --st) {
            const int k = sp * m->steps + st;
            --a;  // NL input
            fg::nl_grad_kernel<<<gridn(n), 256, 0, s>>>(m->acts + (size_t)a * n, m->xi(k), g, g2, m->gxi(k), n);
            count_launch();
            e = cudaGetLastError();
            std::swap(g, g2);
            --a;  // FIR input
            if (e == cudaSuccess) {
                fg::fir_grad_taps_kernel<<<gg, fg::FIR_GRAD_THREADS, 0, s>>>(m->acts + (size_t)a * n, g, m->taps, m->gh(k), m->samples);
                count_launch();
                e = cudaGetLastError();
            }
            if (e == cudaSuccess) e = fir(*m, g, m->h(k), m->taps, 1, g2);
            std::swap(g, g2);
        }
        if (e == cudaSuccess) e = fg::launch_scale(g, n, make_float2(m->span_scale, 0.f), s);
    }
    double h_loss = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_loss, m->loss, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (loss) *loss = h_loss;
    return ldbp_err(m->ctx, e, "ldbp loss/grad");
}

FOCSS_API focss_status focss_ldbp_adam_step(focss_ldbp* m, double lr, double lr_gain, double beta1, double beta2,
                                            double eps) {
    if (!m) return FOCSS_ERR_INVALID_ARG;
    m->adam_t += 1;
    const float c1 = (float)(1.0 / (1.0 - std::pow(beta1, m->adam_t)));
    const float c2 = (float)(1.0 / (1.0 - std::pow(beta2, m->adam_t)));
    // complex gradients g = dL/dconj(z) -> real gradient 2 g; xi gradients are already real:
    // the factor 2 is applied uniformly (Adam is invariant to gradient scale).
    const int xi_lo = m->spans * m->steps * m->taps * 2;
    fg::adam_kernel<<<gridn(m->n_params), 256, 0, m->ctx->stream>>>(
        m->params, m->grads, m->m1, m->m2, m->n_params, (float)lr, (float)beta1, (float)beta2, (float)eps, c1, c2,
        1.f, xi_lo, xi_lo + m->spans * m->steps, (float)lr_gain);
    count_launch();
    return ldbp_err(m->ctx, cudaGetLastError(), "ldbp adam");
}

}  // extern "C"
