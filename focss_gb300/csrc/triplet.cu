// triplet.cu -- first-order perturbation (triplet) sum and equalizer.
//
//   y_mode[k] = sum_{(m,n)} C_mn A_mode[k+m] sum_p A_p[k+n] conj(A_p[k+m+n])
//
// for k in [R, N-R), zero elsewhere (SINO::term / SINO::cubic,
// src/focss/equalizer/sino.cpp:161-171, 203-220), and the equalizer
// (rx - y) / linear_weight (:193-196).  Samples outside [0, N) count as zero,
// so box-shaped term sets (|m|, |n| <= R) are accepted as well as the
// reference's diamond |m| + |n| <= R.
//
// Kernel: one CTA per tile of TK = T*NT consecutive outputs.  Terms are
// grouped by m on the host into dense n-runs (zero-padded to multiples of T).
// Per m the CTA hoists Q_m[j] = sum_p A_p[j] conj(A_p[j+m]) for the tile into
// shared memory; each thread then owns T consecutive outputs and slides a
// register window over Q_m along n, so one shared-memory load feeds T complex
// multiply-adds (FP32 CUDA cores; the sum has no GEMM structure).  Shared
// arrays use a padded index j + j/T so the per-thread stride T+1 is odd and
// reads are conflict-free.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace fg {
namespace {

constexpr int TT = 8;     // outputs per thread and n-steps per window refill
constexpr int NT = 128;   // threads per CTA
constexpr int TK = TT * NT;

__device__ __forceinline__ int padi(int j) { return j + (j >> 3); }

struct TripletArgs {
    const float2* in;       // batch realizations, `in_bstride` apart, modes x N each
    size_t in_bstride;
    const float2* rx;       // equalizer: batch x modes x N, or null
    float2* out;
    float2 inv_lw;          // 1 / linear_weight (equalizer)
    int modes, samples, radius;
    int groups;
    const int* g_m;         // m of each group
    const int* g_nlo;       // first n of each group's dense run
    const int* g_off;       // groups+1 offsets into coef (each run a multiple of TT long)
    const float2* coef;     // dense C_mn runs
    int halo_q;             // max |n| + TT over groups (Q range beyond the tile)
    int halo_a;             // halo_q + max |m| (A range beyond the tile)
};

template <int MODES>
__global__ void __launch_bounds__(NT) triplet_kernel(const TripletArgs a) {
    extern __shared__ float2 sh[];
    const int N = a.samples;
    const int b = blockIdx.y;
    const int k0 = blockIdx.x * TK;
    const int alen = TK + 2 * a.halo_a;
    const int qlen = TK + 2 * a.halo_q;
    float2* As = sh;                           // MODES x padi(alen)
    const int astride = padi(alen) + 1;
    float2* Qs = As + MODES * astride;         // padi(qlen)
    const float2* in = a.in + (size_t)b * a.in_bstride;

    // A tile: index i <-> sample k0 - halo_a + i (zero outside [0, N))
    for (int p = 0; p < MODES; ++p)
        for (int i = threadIdx.x; i < alen; i += NT) {
            const int s = k0 - a.halo_a + i;
            As[p * astride + padi(i)] = (s >= 0 && s < N) ? in[(size_t)p * N + s] : make_float2(0.f, 0.f);
        }

    float2 acc[MODES][TT];
#pragma unroll
    for (int p = 0; p < MODES; ++p)
#pragma unroll
        for (int r = 0; r < TT; ++r) acc[p][r] = make_float2(0.f, 0.f);

    const int kl = threadIdx.x * TT;  // first local output of this thread
    for (int g = 0; g < a.groups; ++g) {
        const int m = a.g_m[g];
        const int nlo = a.g_nlo[g];
        const int off = a.g_off[g], len = a.g_off[g + 1] - off;
        __syncthreads();  // previous Q consumed (and A tile ready on g = 0)
        // Q tile: index i <-> j = k0 - halo_q + i
        for (int i = threadIdx.x; i < qlen; i += NT) {
            const int ia = i + (a.halo_a - a.halo_q);  // A index of j
            float2 q = make_float2(0.f, 0.f);
#pragma unroll
            for (int p = 0; p < MODES; ++p)
                q = cadd(q, cmulc(As[p * astride + padi(ia)], As[p * astride + padi(ia + m)]));
            Qs[padi(i)] = q;
        }
        __syncthreads();
        float2 s[TT];
#pragma unroll
        for (int r = 0; r < TT; ++r) s[r] = make_float2(0.f, 0.f);
        // window w[x] = Q at local output index kl + n + x
        const int qbase = kl + a.halo_q;  // Q index of local output kl at n = 0
        float2 w[2 * TT];
#pragma unroll
        for (int x = 0; x < TT; ++x) w[x] = Qs[padi(qbase + nlo + x)];
        for (int d0 = 0; d0 < len; d0 += TT) {
#pragma unroll
            for (int x = 0; x < TT; ++x) w[TT + x] = Qs[padi(qbase + nlo + d0 + TT + x)];
#pragma unroll
            for (int d = 0; d < TT; ++d) {
                const float2 c = __ldg(a.coef + off + d0 + d);
#pragma unroll
                for (int r = 0; r < TT; ++r) {
                    const float2 q = w[r + d];
                    s[r].x = fmaf(c.x, q.x, fmaf(-c.y, q.y, s[r].x));
                    s[r].y = fmaf(c.x, q.y, fmaf(c.y, q.x, s[r].y));
                }
            }
#pragma unroll
            for (int x = 0; x < TT; ++x) w[x] = w[TT + x];
        }
        // acc_p[k] += A_p[k + m] * s[k]
#pragma unroll
        for (int p = 0; p < MODES; ++p)
#pragma unroll
            for (int r = 0; r < TT; ++r)
                acc[p][r] = cadd(acc[p][r], cmul(As[p * astride + padi(kl + r + m + a.halo_a)], s[r]));
    }

    const float2* rx = a.rx ? a.rx + (size_t)b * MODES * N : nullptr;
    float2* out = a.out + (size_t)b * MODES * N;
#pragma unroll
    for (int p = 0; p < MODES; ++p)
#pragma unroll
        for (int r = 0; r < TT; ++r) {
            const int k = k0 + kl + r;
            if (k >= N) continue;
            const bool valid = k >= a.radius && k < N - a.radius;
            float2 y = valid ? acc[p][r] : make_float2(0.f, 0.f);
            if (rx) y = cmul(csub(rx[(size_t)p * N + k], y), a.inv_lw);
            out[(size_t)p * N + k] = y;
        }
}

struct Terms {
    std::vector<int> gm, gnlo, goff;
    std::vector<float2> coef;
    int halo_q = 0, halo_a = 0;
};

bool build_terms(int n_terms, const int32_t* m, const int32_t* n, const double* c, Terms& t) {
    std::map<int, std::map<int, std::pair<double, double>>> by_m;
    for (int i = 0; i < n_terms; ++i) {
        auto& slot = by_m[m[i]][n[i]];
        slot.first += c[2 * i];
        slot.second += c[2 * i + 1];
    }
    int max_n = 0, max_m = 0;
    t.goff.push_back(0);
    for (auto& kv : by_m) {
        const int mm = kv.first;
        const int nlo = kv.second.begin()->first, nhi = kv.second.rbegin()->first;
        int len = nhi - nlo + 1;
        len = (len + TT - 1) / TT * TT;
        t.gm.push_back(mm);
        t.gnlo.push_back(nlo);
        const size_t base = t.coef.size();
        t.coef.resize(base + len, make_float2(0.f, 0.f));
        for (auto& e : kv.second) t.coef[base + (e.first - nlo)] = make_float2((float)e.second.first, (float)e.second.second);
        t.goff.push_back((int)t.coef.size());
        max_m = std::max(max_m, std::abs(mm));
        max_n = std::max({max_n, std::abs(nlo), std::abs(nlo + len - 1)});
    }
    t.halo_q = max_n + TT;
    t.halo_a = t.halo_q + max_m;
    return true;
}

// Device term tables of recent term lists, per context: an equalizer applied
// again with the same coefficients skips the host grouping and the upload.
// The device buffer lives in ctx->tables (freed with the context); its
// layout is {gm[ng], gnlo[ng], goff[ng+1], pad to 16 B, coef runs}.
struct TermPlan {
    int ng = 0, halo_q = 0, halo_a = 0;
    size_t coef_offset = 0;
};
std::mutex g_term_mutex;
std::map<std::pair<const Ctx*, std::string>, TermPlan> g_term_plans;
constexpr int kMaxTermPlans = 16;

uint64_t fnv1a(const void* p, size_t n, uint64_t h) {
    const unsigned char* b = (const unsigned char*)p;
    for (size_t i = 0; i < n; ++i) {
        h ^= b[i];
        h *= 1099511628211ull;
    }
    return h;
}

std::string term_key(int n_terms, const int32_t* m, const int32_t* n, const double* c) {
    uint64_t h1 = 1469598103934665603ull, h2 = 0x9E3779B97F4A7C15ull;
    h1 = fnv1a(&n_terms, sizeof n_terms, h1);
    h1 = fnv1a(m, sizeof(int32_t) * n_terms, h1);
    h1 = fnv1a(n, sizeof(int32_t) * n_terms, h1);
    h1 = fnv1a(c, sizeof(double) * 2 * n_terms, h1);
    h2 = fnv1a(c, sizeof(double) * 2 * n_terms, h2);
    h2 = fnv1a(n, sizeof(int32_t) * n_terms, h2);
    h2 = fnv1a(m, sizeof(int32_t) * n_terms, h2);
    char buf[64];
    std::snprintf(buf, sizeof buf, "triplet:%016llx%016llx:%d", (unsigned long long)h1, (unsigned long long)h2,
                  n_terms);
    return buf;
}

// The cached device tables of a term list (built and uploaded on a miss).
focss_status term_plan(Ctx* c, int n_terms, const int32_t* m, const int32_t* n, const double* coef,
                       const char** dev, TermPlan* plan) {
    const std::string key = term_key(n_terms, m, n, coef);
    std::lock_guard<std::mutex> lock(g_term_mutex);
    auto it = g_term_plans.find({c, key});
    auto tt = c->tables.find(key);
    if (it != g_term_plans.end() && tt != c->tables.end()) {
        *dev = (const char*)tt->second;
        *plan = it->second;
        return FOCSS_OK;
    }
    int cached = 0;
    for (auto& kv : c->tables) cached += kv.first.compare(0, 8, "triplet:") == 0;
    if (cached >= kMaxTermPlans) {  // drop them all (in-flight kernels finish first)
        cudaStreamSynchronize(c->stream);
        for (auto kv = c->tables.begin(); kv != c->tables.end();) {
            if (kv->first.compare(0, 8, "triplet:") == 0) {
                cudaFree(kv->second);
                g_term_plans.erase({c, kv->first});
                kv = c->tables.erase(kv);
            } else {
                ++kv;
            }
        }
    }
    Terms t;
    build_terms(n_terms, m, n, coef, t);
    TermPlan p;
    p.ng = (int)t.gm.size();
    p.halo_q = t.halo_q;
    p.halo_a = t.halo_a;
    const size_t bytes_i = sizeof(int) * (3 * (size_t)p.ng + 1);
    p.coef_offset = (bytes_i + 15) / 16 * 16;
    std::vector<char> host(p.coef_offset + sizeof(float2) * t.coef.size(), 0);
    int* hi = (int*)host.data();
    std::copy(t.gm.begin(), t.gm.end(), hi);
    std::copy(t.gnlo.begin(), t.gnlo.end(), hi + p.ng);
    std::copy(t.goff.begin(), t.goff.end(), hi + 2 * p.ng);
    std::copy(t.coef.begin(), t.coef.end(), (float2*)(host.data() + p.coef_offset));
    void* d = nullptr;
    cudaError_t e = cudaMalloc(&d, host.size());
    if (e != cudaSuccess) return cuda_check(c, e, "triplet tables");
    e = cudaMemcpy(d, host.data(), host.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_check(c, e, "triplet upload");
    }
    c->tables[key] = d;
    g_term_plans[{c, key}] = p;
    *dev = (const char*)d;
    *plan = p;
    return FOCSS_OK;
}

}  // namespace

// The triplet sum over `modes` consecutive rows of each realization of `in`
// (realizations in_bstride apart), written to `out` (batch x modes x N);
// with rx, the equalizer (rx - y) / linear_weight instead.
focss_status run_triplet_rows(Ctx* c, const float2* in, size_t in_bstride, int modes, int samples, int batch,
                              const float2* rx, int radius, int n_terms, const int32_t* m, const int32_t* n,
                              const double* coef, float2 inv_lw, float2* out) {
    if (modes < 1 || modes > 2)
        return set_error(c, FOCSS_ERR_UNSUPPORTED, "triplet: 1 or 2 modes");
    if (n_terms <= 0 || !m || !n || !coef) return set_error(c, FOCSS_ERR_INVALID_ARG, "triplet: empty term list");
    for (int i = 0; i < n_terms; ++i)
        if (std::abs(m[i]) > 4096 || std::abs(n[i]) > 4096)
            return set_error(c, FOCSS_ERR_INVALID_ARG, "triplet: |m|, |n| must be <= 4096");
    const char* d = nullptr;
    TermPlan t;
    focss_status st = term_plan(c, n_terms, m, n, coef, &d, &t);
    if (st != FOCSS_OK) return st;
    const size_t ng = (size_t)t.ng;
    const float2* dcoef = (const float2*)(d + t.coef_offset);
    cudaStream_t s = c->stream;
    cudaError_t e = cudaSuccess;
    TripletArgs a{};
    a.in = in;
    a.in_bstride = in_bstride;
    a.rx = rx;
    a.out = out;
    a.inv_lw = inv_lw;
    a.modes = modes;
    a.samples = samples;
    a.radius = radius;
    a.groups = (int)ng;
    a.g_m = (const int*)d;
    a.g_nlo = (const int*)d + ng;
    a.g_off = (const int*)d + 2 * ng;
    a.coef = dcoef;
    a.halo_q = t.halo_q;
    a.halo_a = t.halo_a;
    const int alen = TK + 2 * t.halo_a, qlen = TK + 2 * t.halo_q;
    const size_t smem = sizeof(float2) * ((size_t)modes * (alen + alen / 8 + 2) + qlen + qlen / 8 + 2);
    if (smem > 200 * 1024) return set_error(c, FOCSS_ERR_UNSUPPORTED, "triplet: term offsets too large for a tile");
    dim3 grid((samples + TK - 1) / TK, batch);
    if (modes == 1) {
        cudaFuncSetAttribute(triplet_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        triplet_kernel<1><<<grid, NT, smem, s>>>(a);
    } else {
        cudaFuncSetAttribute(triplet_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        triplet_kernel<2><<<grid, NT, smem, s>>>(a);
    }
    count_launch();
    e = cudaGetLastError();
    return cuda_check(c, e, "triplet");
}

namespace {
focss_status run_triplet(Ctx* c, const Field* in, const Field* rx, int radius, int n_terms, const int32_t* m,
                         const int32_t* n, const double* coef, float2 inv_lw, Field* out) {
    return run_triplet_rows(c, in->d, (size_t)in->modes * in->samples, in->modes, in->samples, in->batch,
                            rx ? rx->d : nullptr, radius, n_terms, m, n, coef, inv_lw, out->d);
}
}  // namespace
}  // namespace fg

extern "C" {

FOCSS_API focss_status focss_triplet_apply(focss_ctx* c, const focss_field* in, int radius, int n_terms,
                                           const int32_t* m, const int32_t* n, const double* coef,
                                           focss_field* out) {
    if (!c || !in || !out) return FOCSS_ERR_INVALID_ARG;
    if (in->modes != out->modes || in->samples != out->samples || in->batch != out->batch || in == out)
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "triplet_apply: out must be a distinct field of the same shape");
    return fg::run_triplet(c, in, nullptr, radius, n_terms, m, n, coef, make_float2(1.f, 0.f), out);
}

FOCSS_API focss_status focss_sino_equalize(focss_ctx* c, const focss_field* rx, const focss_field* tx, int radius,
                                           int n_terms, const int32_t* m, const int32_t* n, const double* coef,
                                           double lw_re, double lw_im, focss_field* out) {
    if (!c || !rx || !tx || !out) return FOCSS_ERR_INVALID_ARG;
    if (rx->modes != tx->modes || rx->samples != tx->samples || rx->batch != tx->batch ||
        out->modes != rx->modes || out->samples != rx->samples || out->batch != rx->batch || out == tx)
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "sino_equalize: shapes");
    const double den = lw_re * lw_re + lw_im * lw_im;
    if (!(den > 0)) return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "sino_equalize: linear weight is zero");
    const float2 inv = make_float2((float)(lw_re / den), (float)(-lw_im / den));
    return fg::run_triplet(c, tx, rx, radius, n_terms, m, n, coef, inv, out);
}

}  // extern "C"
