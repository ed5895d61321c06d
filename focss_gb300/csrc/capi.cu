// capi.cu -- the extern "C" boundary (include/focss_gpu.h) over the kernels.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "fft.cuh"
#include "internal.h"

using fg::Ctx;
using fg::Field;

namespace fg {

focss_status set_error(Ctx* ctx, focss_status st, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return st;
}

focss_status cuda_check(Ctx* ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return FOCSS_OK;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return set_error(ctx, FOCSS_ERR_OOM, std::string(what) + ": " + cudaGetErrorString(e));
    }
    return set_error(ctx, FOCSS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

focss_status get_plan(Ctx* ctx, int N, const Plan** out) {
    int lg = 0;
    while ((1 << lg) < N) ++lg;
    return get_plan_split(ctx, N, lg / 2, out);
}

int default_split(int N) {
    int lg = 0;
    while ((1 << lg) < N) ++lg;
    return lg / 2;
}

bool split_supported(int N, int log2N1) {
    int lg = 0;
    while ((1 << lg) < N) ++lg;
    return fft_size_supported(N) && log2N1 >= 4 && log2N1 <= 10 && lg - log2N1 >= 4 && lg - log2N1 <= 10;
}

focss_status get_plan_split(Ctx* ctx, int N, int log2N1, const Plan** out) {
    const long long key = ((long long)log2N1 << 32) | (unsigned)N;
    auto it = ctx->plans.find(key);
    if (it != ctx->plans.end()) {
        *out = &it->second;
        return FOCSS_OK;
    }
    if (!fft_size_supported(N))
        return set_error(ctx, FOCSS_ERR_UNSUPPORTED,
                         "field length " + std::to_string(N) + " is not a power of two in [2^8, 2^20]");
    if (!split_supported(N, log2N1))
        return set_error(ctx, FOCSS_ERR_UNSUPPORTED, "FFT split 2^" + std::to_string(log2N1) + " of length " +
                                                         std::to_string(N) + " is outside [2^4, 2^10] x [2^4, 2^10]");
    Plan p;
    int lg = 0;
    while ((1 << lg) < N) ++lg;
    p.N = N;
    p.log2N1 = log2N1;
    p.log2N2 = lg - log2N1;
    p.N1 = 1 << p.log2N1;
    p.N2 = 1 << p.log2N2;
    // Twiddle tables from FP64 as double-float pairs {re_hi, im_hi, re_lo, im_lo}
    // (layout documented in internal.h).
    std::vector<float4> h(2 * (size_t)p.N1 + 2 * (size_t)p.N2 + 512);
    const double two_pi = 2.0 * 3.14159265358979323846;
    auto df = [](double re, double im) {
        const float rh = (float)re, ih = (float)im;
        return make_float4(rh, ih, (float)(re - (double)rh), (float)(im - (double)ih));
    };
    // cos/sin of 2 pi e / L evaluated on an exactly reduced argument (e mod L).
    auto w = [&](long long e, long long L) { return df(std::cos(two_pi * e / L), -std::sin(two_pi * e / L)); };
    // Threads per group of a length-L sub-FFT (must match PQ<L>::P in fft.cuh).
    auto groupP = [](int L) { return L <= 32 ? 4 : L <= 128 ? 8 : L <= 512 ? 16 : 32; };
    auto fill_pq = [&](float4* dst, int L, int P) {
        const int Q = L / P;
        for (int u = 0; u < Q; ++u)
            for (int t = 0; t < P; ++t) dst[u * P + t] = w((long long)t * u % L, L);
    };
    fill_pq(h.data(), p.N1, col_group_p(p.N1));
    fill_pq(h.data() + p.N1, p.N2, groupP(p.N2));
    for (int j = 0; j < 512; ++j)
        h[2 * p.N1 + 2 * p.N2 + j] = df(std::cos(two_pi * j / 512), std::sin(two_pi * j / 512));
    cudaError_t e = cudaMalloc(&p.tw, sizeof(float4) * h.size());
    if (e != cudaSuccess) return cuda_check(ctx, e, "twiddle alloc");
    e = cudaMemcpy(p.tw, h.data(), sizeof(float4) * h.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(p.tw);
        return cuda_check(ctx, e, "twiddle upload");
    }
    p.staging = ctx->staging;
    auto res = ctx->plans.emplace(key, p);
    *out = &res.first->second;
    return FOCSS_OK;
}

focss_status ensure_state(Ctx* ctx, int batch) {
    if (batch <= ctx->state_cap) return FOCSS_OK;
    if (ctx->d_state) cudaFree(ctx->d_state);
    ctx->d_state = nullptr;
    ctx->state_cap = 0;
    cudaError_t e = cudaMalloc(&ctx->d_state, sizeof(SsfmState) * (size_t)batch);
    if (e != cudaSuccess) return cuda_check(ctx, e, "state alloc");
    ctx->state_cap = batch;
    return FOCSS_OK;
}

focss_status ensure_red(Ctx* ctx, size_t doubles) {
    if (doubles <= ctx->red_cap) return FOCSS_OK;
    if (ctx->d_red) cudaFree(ctx->d_red);
    ctx->d_red = nullptr;
    ctx->red_cap = 0;
    cudaError_t e = cudaMalloc(&ctx->d_red, sizeof(double) * doubles);
    if (e != cudaSuccess) return cuda_check(ctx, e, "reduction alloc");
    ctx->red_cap = doubles;
    return FOCSS_OK;
}

int sm_count() {
    static int cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!cached[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 152;
        cached[dev] = n;
    }
    return cached[dev];
}

void* scratch_buffer(Ctx* ctx, int slot, size_t bytes) {
    if ((int)ctx->scratch.size() <= slot) {
        ctx->scratch.resize(slot + 1, nullptr);
        ctx->scratch_cap.resize(slot + 1, 0);
    }
    if (ctx->scratch_cap[slot] >= bytes) return ctx->scratch[slot];
    if (ctx->scratch[slot]) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->scratch[slot]);
    }
    ctx->scratch[slot] = nullptr;
    ctx->scratch_cap[slot] = 0;
    if (cudaMalloc(&ctx->scratch[slot], bytes) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    ctx->scratch_cap[slot] = bytes;
    return ctx->scratch[slot];
}

static long long g_launches = 0;
// Launches recorded into a graph are counted when the graph runs, not here.
thread_local int g_capturing = 0;
void count_launch(long long n) {
    if (!g_capturing) __atomic_fetch_add(&g_launches, n, __ATOMIC_RELAXED);
}
void count_launch_graph(long long n) { __atomic_fetch_add(&g_launches, n, __ATOMIC_RELAXED); }
void set_capturing(bool on) { g_capturing += on ? 1 : -1; }

}  // namespace fg

namespace fg {
// Amplifier::amplify / add_noise / give_power / drop_power
// (src/focss/module/amplifier.cpp:15-42) as A <- scale*A + sigma*(z0 + i z1).
bool amplifier_coeffs(int op, double gain, double noise_factor, double f0, double dt, double* scale,
                      double* sigma) {
    const double kPlanck = 6.62607004081818181818181e-34;  // src/focss/definitions.h:14
    bool noise = false;
    switch (op) {
        case FOCSS_AMP_AMPLIFY: *scale = std::sqrt(gain); noise = noise_factor != 0; break;     // :15-18
        case FOCSS_AMP_ADD_NOISE: *scale = 1.0; noise = true; break;                            // :20-28
        case FOCSS_AMP_GIVE_POWER: *scale = gain > 1 ? std::sqrt(gain) : std::sqrt(1 / gain); break;  // :30-35
        case FOCSS_AMP_DROP_POWER: *scale = gain < 1 ? std::sqrt(gain) : std::sqrt(1 / gain); break;  // :37-42
        default: return false;
    }
    *sigma = 0.0;
    if (noise) {
        // amplifier.cpp:21-27: variance = h f0 NF (G-1)/2 * (1/dt); sigma per quadrature = sqrt(var/2)
        double variance = kPlanck * f0;
        variance *= noise_factor * (gain - 1) / 2;
        variance *= 1.0 / dt;
        *sigma = std::sqrt(variance / 2);
    }
    return true;
}
}  // namespace fg

namespace {

bool same_shape(const Field* a, const Field* b) {
    return a->modes == b->modes && a->samples == b->samples && a->batch == b->batch;
}
}  // namespace

extern "C" {

FOCSS_API int focss_abi_version(void) { return 1; }

FOCSS_API const char* focss_status_string(int s) {
    switch (s) {
        case FOCSS_OK: return "ok";
        case FOCSS_ERR_INVALID_ARG: return "invalid argument";
        case FOCSS_ERR_OOM: return "out of memory";
        case FOCSS_ERR_CUDA: return "CUDA error";
        case FOCSS_ERR_TIMEOUT: return "timeout";
        case FOCSS_ERR_NOT_CONVERGED: return "not converged";
        case FOCSS_ERR_UNSUPPORTED: return "unsupported";
        case FOCSS_ERR_NO_DEVICE: return "no CUDA device";
        default: return "unknown status";
    }
}

FOCSS_API focss_status focss_ctx_create(int device, focss_ctx** out) {
    if (!out) return FOCSS_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return FOCSS_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) return FOCSS_ERR_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return FOCSS_ERR_CUDA;
    focss_ctx* c = new (std::nothrow) focss_ctx();
    if (!c) return FOCSS_ERR_OOM;
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        e = cudaMemPoolCreate(&c->pool, &props);
    }
    if (e == cudaSuccess) {
        unsigned long long keep = ~0ull;  // released blocks stay in the pool
        e = cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) e = cudaMalloc(&c->d_counters, sizeof(int) * 16);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_pinned, sizeof(int) * 16);
    if (e != cudaSuccess) {
        focss_ctx_destroy(c);
        return e == cudaErrorMemoryAllocation ? FOCSS_ERR_OOM : FOCSS_ERR_CUDA;
    }
    *out = c;
    return FOCSS_OK;
}

FOCSS_API focss_status focss_ctx_destroy(focss_ctx* c) {
    if (!c) return FOCSS_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (fg::Field* f : c->fields) f->ctx = nullptr;  // still valid until destroyed; see focss_field_destroy
    for (auto& kv : c->plans) cudaFree(kv.second.tw);
    for (void* p : c->scratch) cudaFree(p);
    for (cudaEvent_t e : c->prof_events) cudaEventDestroy(e);
    for (auto& kv : c->tables) cudaFree(kv.second);
    fg::free_loop_graphs(c);
    cudaFree(c->d_state);
    cudaFree(c->d_counters);
    cudaFree(c->d_red);
    if (c->h_pinned) cudaFreeHost(c->h_pinned);
    if (c->stream) cudaStreamDestroy(c->stream);
    // fields still alive keep their blocks; the pool goes when they are freed
    if (c->pool) cudaMemPoolDestroy(c->pool);
    delete c;
    return FOCSS_OK;
}

FOCSS_API focss_status focss_ctx_sync(focss_ctx* c) {
    if (!c) return FOCSS_ERR_INVALID_ARG;
    return fg::cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
}

FOCSS_API void* focss_ctx_stream(focss_ctx* c) { return c ? (void*)c->stream : nullptr; }

FOCSS_API const char* focss_ctx_last_error(const focss_ctx* c) { return c ? c->last_error.c_str() : ""; }

FOCSS_API focss_status focss_field_create(focss_ctx* c, const focss_domain* d, int batch, focss_field** out) {
    if (!c || !d || !out) return FOCSS_ERR_INVALID_ARG;
    *out = nullptr;
    // src/focss/field.cpp:25 asserts modes > 0, samples > 0, time_step > 0.
    if (d->modes <= 0 || d->samples <= 0 || !(d->time_step > 0) || batch <= 0)
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "field_create: modes, samples, time_step, batch must be > 0");
    // the kernels put realizations (or realization x mode rows) on a grid's y dimension
    if ((long long)batch * d->modes > 65535)
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "field_create: batch x modes must be <= 65535");
    focss_field* f = new (std::nothrow) focss_field();
    if (!f) return FOCSS_ERR_OOM;
    f->ctx = c;
    f->modes = d->modes;
    f->samples = d->samples;
    f->dt = d->time_step;
    f->f0 = d->center_frequency;
    f->batch = batch;
    // stream-ordered: the block is usable by work queued on the context's
    // stream after this call (every library call on the field)
    cudaError_t e = cudaMallocFromPoolAsync((void**)&f->d, sizeof(float2) * f->n(), c->pool, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(f->d, 0, sizeof(float2) * f->n(), c->stream);
    if (e != cudaSuccess) {
        if (f->d) cudaFreeAsync(f->d, c->stream);
        delete f;
        return fg::cuda_check(c, e, "field alloc");
    }
    c->fields.insert(f);
    *out = f;
    return FOCSS_OK;
}

FOCSS_API focss_status focss_field_destroy(focss_field* f) {
    if (!f) return FOCSS_OK;
    if (f->ctx) {
        f->ctx->fields.erase(f);
        // released after the work already queued on the context's stream
        if (f->d) cudaFreeAsync(f->d, f->ctx->stream);
    } else if (f->d) {
        cudaFree(f->d);  // the context went first: a plain (synchronizing) release
    }
    delete f;
    return FOCSS_OK;
}

FOCSS_API focss_status focss_field_domain(const focss_field* f, focss_domain* d, int* batch) {
    if (!f) return FOCSS_ERR_INVALID_ARG;
    if (d) *d = focss_domain{f->modes, f->samples, f->dt, f->f0};
    if (batch) *batch = f->batch;
    return FOCSS_OK;
}

FOCSS_API void* focss_field_device_ptr(focss_field* f) { return f ? (void*)f->d : nullptr; }

FOCSS_API focss_status focss_field_upload_c64(focss_field* f, const float* h, size_t n) {
    if (!f || !h) return FOCSS_ERR_INVALID_ARG;
    if (n != f->n()) return fg::set_error(f->ctx, FOCSS_ERR_INVALID_ARG, "upload: size mismatch");
    return fg::cuda_check(f->ctx,
                          cudaMemcpyAsync(f->d, h, sizeof(float2) * n, cudaMemcpyHostToDevice, f->ctx->stream),
                          "upload");
}

FOCSS_API focss_status focss_field_download_c64(focss_field* f, float* h, size_t n) {
    if (!f || !h) return FOCSS_ERR_INVALID_ARG;
    if (n != f->n()) return fg::set_error(f->ctx, FOCSS_ERR_INVALID_ARG, "download: size mismatch");
    cudaError_t e = cudaMemcpyAsync(h, f->d, sizeof(float2) * n, cudaMemcpyDeviceToHost, f->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->ctx->stream);
    return fg::cuda_check(f->ctx, e, "download");
}

FOCSS_API focss_status focss_field_upload(focss_field* f, const double* h, size_t n) {
    if (!f || !h) return FOCSS_ERR_INVALID_ARG;
    if (n != f->n()) return fg::set_error(f->ctx, FOCSS_ERR_INVALID_ARG, "upload: size mismatch");
    std::vector<float> tmp(2 * n);
    for (size_t i = 0; i < 2 * n; ++i) tmp[i] = (float)h[i];
    cudaError_t e = cudaMemcpyAsync(f->d, tmp.data(), sizeof(float2) * n, cudaMemcpyHostToDevice, f->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->ctx->stream);
    return fg::cuda_check(f->ctx, e, "upload");
}

FOCSS_API focss_status focss_field_download(focss_field* f, double* h, size_t n) {
    if (!f || !h) return FOCSS_ERR_INVALID_ARG;
    if (n != f->n()) return fg::set_error(f->ctx, FOCSS_ERR_INVALID_ARG, "download: size mismatch");
    std::vector<float> tmp(2 * n);
    cudaError_t e = cudaMemcpyAsync(tmp.data(), f->d, sizeof(float2) * n, cudaMemcpyDeviceToHost, f->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->ctx->stream);
    if (e != cudaSuccess) return fg::cuda_check(f->ctx, e, "download");
    for (size_t i = 0; i < 2 * n; ++i) h[i] = (double)tmp[i];
    return FOCSS_OK;
}

FOCSS_API focss_status focss_field_copy(focss_field* dst, const focss_field* src) {
    if (!dst || !src) return FOCSS_ERR_INVALID_ARG;
    if (!same_shape(dst, src)) return fg::set_error(dst->ctx, FOCSS_ERR_INVALID_ARG, "copy: shape mismatch");
    return fg::cuda_check(dst->ctx,
                          cudaMemcpyAsync(dst->d, src->d, sizeof(float2) * dst->n(), cudaMemcpyDeviceToDevice,
                                          dst->ctx->stream),
                          "copy");
}

FOCSS_API focss_status focss_field_copy_realizations(focss_field* dst, int dst_first, const focss_field* src,
                                                     int src_first, int count) {
    if (!dst || !src || count < 0 || dst_first < 0 || src_first < 0) return FOCSS_ERR_INVALID_ARG;
    if (dst->modes != src->modes || dst->samples != src->samples || dst_first + count > dst->batch ||
        src_first + count > src->batch)
        return fg::set_error(dst->ctx, FOCSS_ERR_INVALID_ARG, "copy_realizations: shapes");
    const size_t per = (size_t)src->modes * src->samples;
    return fg::cuda_check(dst->ctx,
                          cudaMemcpyAsync(dst->d + per * dst_first, src->d + per * src_first,
                                          sizeof(float2) * per * count, cudaMemcpyDeviceToDevice, dst->ctx->stream),
                          "copy_realizations");
}

FOCSS_API focss_status focss_field_copy_modes(focss_field* dst, int dst_first, const focss_field* src, int src_first,
                                              int count) {
    if (!dst || !src || count < 0 || dst_first < 0 || src_first < 0) return FOCSS_ERR_INVALID_ARG;
    if (dst->batch != src->batch || dst->samples != src->samples || dst_first + count > dst->modes ||
        src_first + count > src->modes)
        return fg::set_error(dst->ctx, FOCSS_ERR_INVALID_ARG, "copy_modes: shapes");
    if (count == 0) return FOCSS_OK;
    // one row of count * samples values per realization
    const size_t row = sizeof(float2) * (size_t)count * src->samples;
    return fg::cuda_check(dst->ctx,
                          cudaMemcpy2DAsync(dst->d + (size_t)dst_first * dst->samples,
                                            sizeof(float2) * (size_t)dst->modes * dst->samples,
                                            src->d + (size_t)src_first * src->samples,
                                            sizeof(float2) * (size_t)src->modes * src->samples, row, src->batch,
                                            cudaMemcpyDeviceToDevice, dst->ctx->stream),
                          "copy_modes");
}

FOCSS_API focss_status focss_field_scale(focss_field* f, double re, double im) {
    if (!f) return FOCSS_ERR_INVALID_ARG;
    return fg::cuda_check(f->ctx, fg::launch_scale(f->d, f->n(), make_float2((float)re, (float)im), f->ctx->stream),
                          "scale");
}

FOCSS_API focss_status focss_field_power(focss_field* f, double* average, double* peak) {
    if (!f) return FOCSS_ERR_INVALID_ARG;
    Ctx* c = f->ctx;
    focss_status st = fg::ensure_red(c, 2 * (size_t)f->batch);
    if (st != FOCSS_OK) return st;
    double* avg = c->d_red;
    unsigned* pk = (unsigned*)(c->d_red + f->batch);
    cudaError_t e = cudaMemsetAsync(c->d_red, 0, sizeof(double) * 2 * f->batch, c->stream);
    if (e == cudaSuccess) e = fg::launch_power(f->d, f->modes, f->samples, f->batch, avg, pk, c->stream);
    std::vector<double> ha(f->batch);
    std::vector<unsigned> hp(f->batch);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ha.data(), avg, sizeof(double) * f->batch, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), pk, sizeof(unsigned) * f->batch, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fg::cuda_check(c, e, "power");
    for (int b = 0; b < f->batch; ++b) {
        if (average) average[b] = ha[b];
        if (peak) {
            float v;
            std::memcpy(&v, &hp[b], sizeof(v));
            peak[b] = v;
        }
    }
    return FOCSS_OK;
}

FOCSS_API focss_status focss_field_fft(focss_field* f) {
    if (!f) return FOCSS_ERR_INVALID_ARG;
    return fg::fft_forward(f->ctx, f->d, f->samples, f->batch * f->modes);
}

FOCSS_API focss_status focss_field_ifft(focss_field* f) {
    if (!f) return FOCSS_ERR_INVALID_ARG;
    return fg::fft_inverse(f->ctx, f->d, f->samples, f->batch * f->modes);
}

FOCSS_API focss_status focss_ssfm_run(focss_ctx* c, focss_field* f, const focss_fiber* fiber,
                                      const focss_ssfm_opts* opts, double direction, int* steps_out) {
    if (!c || !f || !fiber || !opts) return FOCSS_ERR_INVALID_ARG;
    if (f->ctx != c) return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "field belongs to another context");
    if (direction != 1.0 && direction != -1.0)
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "direction must be FOCSS_FORWARD or FOCSS_BACKWARD");
    return fg::ssfm_run(c, f, *fiber, *opts, direction, steps_out);
}

FOCSS_API focss_status focss_set_pass_staging(focss_ctx* c, int mode) {
    if (!c || (mode != FOCSS_STAGING_LOADS && mode != FOCSS_STAGING_BULK && mode != FOCSS_STAGING_TMA))
        return FOCSS_ERR_INVALID_ARG;
    c->staging = mode;
    for (auto& kv : c->plans) kv.second.staging = mode;
    return FOCSS_OK;
}

FOCSS_API focss_status focss_set_row_staging(focss_ctx* c, int mode) {
    if (mode != FOCSS_STAGING_LOADS && mode != FOCSS_STAGING_BULK) return FOCSS_ERR_INVALID_ARG;
    return focss_set_pass_staging(c, mode);
}

// Step-grid record / replay: device copies of the step lists live in scratch
// slot 9 (sizes) and 10 (counts).
FOCSS_API focss_status focss_ssfm_run_record(focss_ctx* c, focss_field* f, const focss_fiber* fiber,
                                             const focss_ssfm_opts* opts, double direction, int capacity,
                                             double* steps_h, int* steps_out) {
    if (!c || !f || !fiber || !opts || !steps_h || capacity <= 0) return FOCSS_ERR_INVALID_ARG;
    if (f->ctx != c) return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "field belongs to another context");
    if (direction != 1.0 && direction != -1.0)
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "direction must be FOCSS_FORWARD or FOCSS_BACKWARD");
    const size_t n = (size_t)f->batch * capacity;
    double* d_h = (double*)fg::scratch_buffer(c, 9, sizeof(double) * n);
    if (!d_h) return fg::set_error(c, FOCSS_ERR_OOM, "ssfm_run_record: step buffer");
    fg::StepGrid g;
    g.record = d_h;
    g.cap = capacity;
    std::vector<int> rec(f->batch);
    focss_status st = fg::ssfm_run(c, f, *fiber, *opts, direction, steps_out, &g, rec.data());
    if (st != FOCSS_OK) return st;
    for (int b = 0; b < f->batch; ++b)
        if (rec[b] > capacity)
            return fg::set_error(c, FOCSS_ERR_INVALID_ARG,
                                 "ssfm_run_record: realization " + std::to_string(b) + " took " +
                                     std::to_string(rec[b]) + " steps, more than the capacity " +
                                     std::to_string(capacity));
    st = fg::cuda_check(c, cudaMemcpyAsync(steps_h, d_h, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream),
                        "ssfm_run_record: readback");
    if (st != FOCSS_OK) return st;
    return fg::cuda_check(c, cudaStreamSynchronize(c->stream), "ssfm_run_record: sync");
}

FOCSS_API focss_status focss_ssfm_run_steps(focss_ctx* c, focss_field* f, const focss_fiber* fiber,
                                            const double* steps_h, const int* n_steps, int capacity,
                                            double direction) {
    if (!c || !f || !fiber || !steps_h || !n_steps || capacity <= 0) return FOCSS_ERR_INVALID_ARG;
    if (f->ctx != c) return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "field belongs to another context");
    if (direction != 1.0 && direction != -1.0)
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "direction must be FOCSS_FORWARD or FOCSS_BACKWARD");
    int max_steps = 0;
    for (int b = 0; b < f->batch; ++b) {
        if (n_steps[b] < 1 || n_steps[b] > capacity)
            return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "ssfm_run_steps: step counts must be in [1, capacity]");
        for (int i = 0; i < n_steps[b]; ++i) {
            const double h = steps_h[(size_t)b * capacity + i];
            if (!(h > 0) || !(h < 1e300))
                return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "ssfm_run_steps: step sizes must be finite and > 0");
        }
        max_steps = std::max(max_steps, n_steps[b]);
    }
    const size_t n = (size_t)f->batch * capacity;
    double* d_h = (double*)fg::scratch_buffer(c, 9, sizeof(double) * n);
    int* d_n = (int*)fg::scratch_buffer(c, 10, sizeof(int) * (size_t)f->batch);
    if (!d_h || !d_n) return fg::set_error(c, FOCSS_ERR_OOM, "ssfm_run_steps: step buffer");
    focss_status st = fg::cuda_check(
        c, cudaMemcpyAsync(d_h, steps_h, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream), "steps upload");
    if (st != FOCSS_OK) return st;
    st = fg::cuda_check(c, cudaMemcpyAsync(d_n, n_steps, sizeof(int) * f->batch, cudaMemcpyHostToDevice, c->stream),
                        "step counts upload");
    if (st != FOCSS_OK) return st;
    fg::StepGrid g;
    g.replay = d_h;
    g.count = d_n;
    g.cap = capacity;
    g.max_steps = max_steps;
    // the grid rule is replaced; ADAPTIVE bookkeeping reports the counts
    focss_ssfm_opts o{FOCSS_ADAPTIVE, 0, 1.0, 1.0};
    return fg::ssfm_run(c, f, *fiber, o, direction, nullptr, &g, nullptr);
}

FOCSS_API focss_status focss_amplifier_apply(focss_ctx* c, focss_field* f, double gain, double noise_factor,
                                             uint64_t seed, uint64_t counter, int op) {
    if (!c || !f) return FOCSS_ERR_INVALID_ARG;
    if (!(gain > 0)) return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "amplifier: gain must be > 0");
    double scale = 1.0, sigma = 0.0;
    if (!fg::amplifier_coeffs(op, gain, noise_factor, f->f0, f->dt, &scale, &sigma))
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "amplifier: unknown op");
    return fg::cuda_check(c,
                          fg::launch_amplifier(f->d, f->modes, f->samples, f->batch, scale, (float)sigma,
                                               seed, counter, c->stream),
                          "amplifier");
}

FOCSS_API focss_status focss_forward_propagation(focss_ctx* c, focss_field* f, const focss_fiber* fiber,
                                                 const focss_ssfm_opts* opts, double gain, double noise_factor,
                                                 uint64_t seed, uint64_t counter0, int spans) {
    if (!c || !f || !fiber || !opts || spans < 0) return FOCSS_ERR_INVALID_ARG;
    for (int i = 0; i < spans; ++i) {
        focss_status st = focss_ssfm_run(c, f, fiber, opts, FOCSS_FORWARD, nullptr);
        if (st != FOCSS_OK) return st;
        st = focss_amplifier_apply(c, f, gain, noise_factor, seed, counter0 + (uint64_t)i, FOCSS_AMP_AMPLIFY);
        if (st != FOCSS_OK) return st;
    }
    return FOCSS_OK;
}

FOCSS_API focss_status focss_backward_propagation(focss_ctx* c, focss_field* f, const focss_fiber* fiber,
                                                  const focss_ssfm_opts* opts, double gain, int spans) {
    if (!c || !f || !fiber || !opts || spans < 0) return FOCSS_ERR_INVALID_ARG;
    for (int i = 0; i < spans; ++i) {
        focss_status st = focss_amplifier_apply(c, f, gain, 0.0, 0, 0, FOCSS_AMP_DROP_POWER);
        if (st != FOCSS_OK) return st;
        st = focss_ssfm_run(c, f, fiber, opts, FOCSS_BACKWARD, nullptr);
        if (st != FOCSS_OK) return st;
    }
    return FOCSS_OK;
}

FOCSS_API focss_status focss_cd_compensation(focss_ctx* c, focss_field* f, const focss_fiber* fiber, int spans) {
    if (!c || !f || !fiber || spans < 0) return FOCSS_ERR_INVALID_ARG;
    // fiber.dispersive() * spans (src/focss/module/fiber.cpp:17-22, 32-45), then UNIFORM 1 step BACKWARD.
    focss_fiber d = *fiber;
    d.alpha = 0;
    d.gamma = 0;
    d.length *= spans;
    if (spans == 0) return FOCSS_OK;
    focss_ssfm_opts o{FOCSS_UNIFORM, 1, 0.0, 0.0};
    return focss_ssfm_run(c, f, &d, &o, FOCSS_BACKWARD, nullptr);
}

FOCSS_API focss_status focss_profile_enable(focss_ctx* c, int enable) {
    if (!c) return FOCSS_ERR_INVALID_ARG;
    c->profiling = enable != 0;
    return FOCSS_OK;
}

FOCSS_API focss_status focss_profile_read(focss_ctx* c, double* col_ms, long long* col_launches, double* row_ms,
                                          long long* row_launches, int reset) {
    if (!c) return FOCSS_ERR_INVALID_ARG;
    if (col_ms) *col_ms = c->prof_ms[0];
    if (row_ms) *row_ms = c->prof_ms[1];
    if (col_launches) *col_launches = c->prof_launches[0];
    if (row_launches) *row_launches = c->prof_launches[1];
    if (reset) {
        c->prof_ms[0] = c->prof_ms[1] = 0;
        c->prof_launches[0] = c->prof_launches[1] = 0;
    }
    return FOCSS_OK;
}

FOCSS_API long long focss_launch_count(void) { return __atomic_load_n(&fg::g_launches, __ATOMIC_RELAXED); }

}  // extern "C"
