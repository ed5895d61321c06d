// ssfm.cu -- two-pass (six-step) split-step Fourier kernels for sm_103a.
//
// A field of N = N1*N2 complex64 samples is viewed as an N1 x N2 row-major
// matrix (sample n = N2*n1 + n2).  One split step costs exactly two passes over
// HBM, each one read and one write of the field (16 B per sample per pass):
//
//   column pass  [inverse six-step twiddle, inverse length-N1 FFT over n1]
//                -> time domain: Kerr phase exp(i*kappa*gamma*h*|A|^2),
//                   peak-power reduction (adaptive step estimate)
//                -> [forward length-N1 FFT, forward six-step twiddle]
//   row pass     [forward length-N2 FFT] -> exp(-alpha*hl/2)/N *
//                exp(i*beta2/2*hl*w_k^2) -> [inverse length-N2 FFT]
//
// The spectrum never leaves the transposed layout (row k1, column k2 holds
// bin k = k1 + N1*k2), so no transposes are needed.  The merged half steps of
// the reference's Strang splitting (src/focss/solver/ssfm.cpp:62-118) appear
// as one row pass with hl = (h_i + h_{i+1})/2.
//
// The dispersion phase is formed from an FP64 per-step scalar
// a = beta2/2*hl*dw^2/(2*pi) (turns per k'^2) held as a 64-bit fixed-point
// turn fraction; a*k'^2 mod 1 is then an exact wrapping 64-bit integer
// product, so the FP32 sincospi argument is already range-reduced to [-1, 1).
#include <algorithm>
#include <cmath>
#include <mutex>

#include "ssfm_kernels.cuh"
#include "tma_map.h"

namespace fg {

// ---------------------------------------------------------------- dispatch
namespace {
int ilog2i(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return (1 << l) == n ? l : -1;
}
}  // namespace

Launch col_launch_4();
Launch col_launch_5();
Launch col_launch_6();
Launch col_launch_7();
Launch col_launch_8();
Launch col_launch_9();
Launch col_launch_10();
Launch row_launch_4();
Launch row_launch_5();
Launch row_launch_6();
Launch row_launch_7();
Launch row_launch_8();
Launch row_launch_9();
Launch row_launch_10();

Launch col_launch_for(int lg) {
    switch (lg) {
        case 4: return col_launch_4();
        case 5: return col_launch_5();
        case 6: return col_launch_6();
        case 7: return col_launch_7();
        case 8: return col_launch_8();
        case 9: return col_launch_9();
        case 10: return col_launch_10();
        default: return Launch{};
    }
}

Launch row_launch_for(int lg) {
    switch (lg) {
        case 4: return row_launch_4();
        case 5: return row_launch_5();
        case 6: return row_launch_6();
        case 7: return row_launch_7();
        case 8: return row_launch_8();
        case 9: return row_launch_9();
        case 10: return row_launch_10();
        default: return Launch{};
    }
}

bool fft_size_supported(int N) {
    const int lg = ilog2i(N);
    return lg >= 8 && lg <= 20;
}

// Launch descriptions per device and FFT length: the dynamic shared-memory
// opt-in (cudaFuncSetAttribute) applies to the current device only, so each
// device keeps its own record of it.
constexpr int kMaxDevices = 64;
std::mutex g_launch_mutex;

// The cached launch of pass kind `kind` (0 column, 1 row, 2 row with
// bulk-copy staging, 3 row in 64-thread CTAs, 4 column in 64-thread CTAs, 5
// column with TMA tensor staging) for log2 length lg on the current device,
// opted in to `smem` bytes of dynamic shared memory.
cudaError_t cached_launch(int kind, int lg, size_t smem, Launch* out) {
    static Launch cache[kMaxDevices][6][16];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices || lg < 0 || lg >= 16) return cudaErrorInvalidValue;
    std::lock_guard<std::mutex> lock(g_launch_mutex);
    Launch& l = cache[dev][kind][lg];
    if (!l.fn) {
        l = kind == 0 || kind == 4 || kind == 5 ? col_launch_for(lg) : row_launch_for(lg);
        if (kind == 2) l.fn = l.fn_bulk;
        if (kind == 3 || kind == 4) {
            l.fn = l.fn_narrow;
            l.threads = l.per_block_narrow * (l.threads / l.per_block);
            l.per_block = l.per_block_narrow;
        }
    }
    if (!l.fn) return cudaErrorInvalidValue;
    if (!l.attr_set || smem > l.smem) {
        const void* fn = kind == 5 ? (const void*)l.fn_tma : (const void*)l.fn;
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        l.attr_set = true;
        l.smem = smem;
    }
    *out = l;
    return cudaSuccess;
}

// Launches a pass kernel.  Launched directly into a stream, it carries
// programmatic stream serialization: when the previous operation in the
// stream is a kernel, this one may be scheduled as soon as that kernel's CTAs
// have all started, and runs up to its pdl_wait (the column pass computes its
// six-step factors there) while the other finishes, instead of paying the
// launch latency after it (one 2^17 field, 100 steps through focss_ssfm_run:
// 2.31 -> 2.13 ms).  Captured into a graph it is a plain kernel node: graph
// launches already hide that latency, and programmatic edges there measured
// slower (800 steps of one 2^17 field: 17.8 -> 19.9 us per step).
cudaError_t launch_pass(const Launch& l, dim3 grid, int threads, size_t smem, cudaStream_t s, const PassArgs& a) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const cudaError_t ce = cudaStreamIsCapturing(s, &cs);
    if (ce != cudaSuccess) return ce;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = cs == cudaStreamCaptureStatusNone ? 1 : 0;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, l.fn, a);
    count_launch();
    const cudaError_t last = cudaGetLastError();  // consumed, as after a <<<>>> launch
    return e != cudaSuccess ? e : last;
}

// The column pass with TMA tensor staging (FOCSS_STAGING_TMA): a tensor map
// over the launch's fields (batch x modes x N1 rows of N2 8-byte elements,
// boxes of C columns x min(N1, 256) rows) passed as a kernel parameter.
cudaError_t launch_col_tma(const Plan& p, const PassArgs& a, int batch, int modes, size_t smem, cudaStream_t s) {
    Launch l;
    cudaError_t e = cached_launch(5, p.log2N1, smem, &l);
    if (e != cudaSuccess) return e;
    PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    e = tensor_map_encoder(&encode);
    if (e != cudaSuccess) return e;
    CUtensorMap map;
    const cuuint64_t dims[2] = {(cuuint64_t)p.N2, (cuuint64_t)batch * modes * p.N1};
    const cuuint64_t strides[1] = {(cuuint64_t)p.N2 * sizeof(float2)};
    const cuuint32_t box[2] = {(cuuint32_t)l.per_block, (cuuint32_t)(p.N1 < 256 ? p.N1 : 256)}, estr[2] = {1, 1};
    if (encode(&map, CU_TENSOR_MAP_DATA_TYPE_INT64, 2, a.data, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(p.N2 / l.per_block, batch);
    cfg.blockDim = dim3(l.threads * modes);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(s, &cs);
    if (e != cudaSuccess) return e;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = cs == cudaStreamCaptureStatusNone ? 1 : 0;
    e = cudaLaunchKernelEx(&cfg, l.fn_tma, map, a);
    count_launch();
    const cudaError_t last = cudaGetLastError();
    return e != cudaSuccess ? e : last;
}

cudaError_t launch_col(const Plan& p, PassArgs a, int batch, cudaStream_t s) {
    Launch l = col_launch_for(p.log2N1);
    if (!l.fn) return cudaErrorInvalidValue;
    const int modes = a.modes > 1 ? a.modes : 1;
    // few column blocks in the whole launch: 64-thread CTAs spread them over more SMs
    const bool narrow = p.staging != FOCSS_STAGING_TMA && l.per_block_narrow < l.per_block &&
                        (long long)(p.N2 / l.per_block) * batch < sm_count() && p.N2 % l.per_block_narrow == 0;
    const int C = narrow ? l.per_block_narrow : l.per_block;
    // s_fc (N1) + six-step table (Q x C, Q = N1/P) + exchange (N1 x C per mode)
    const int P = l.threads / l.per_block;
    const size_t smem = sizeof(float4) * ((size_t)p.N1 + (size_t)(p.N1 / P) * C) +
                        sizeof(float2) * (size_t)p.N1 * C * modes;
    a.N = p.N;
    a.N1 = p.N1;
    a.N2 = p.N2;
    a.log2N2 = p.log2N2;
    a.tw = p.tw;
    a.batch = batch;
    if (p.staging == FOCSS_STAGING_TMA) return launch_col_tma(p, a, batch, modes, smem + 128, s);
    cudaError_t e = cached_launch(narrow ? 4 : 0, p.log2N1, smem, &l);
    if (e != cudaSuccess) return e;
    return launch_pass(l, dim3(p.N2 / l.per_block, batch), l.threads * modes, smem, s, a);
}

cudaError_t launch_row(const Plan& p, PassArgs a, int batch, cudaStream_t s) {
    Launch l = row_launch_for(p.log2N2);
    if (!l.fn) return cudaErrorInvalidValue;
    const int P = l.threads / l.per_block;
    const int Q = p.N2 / P;
    const int rows = batch * (a.modes > 1 ? a.modes : 1);
    // few row blocks in the whole launch: 64-thread CTAs spread them over more SMs
    const bool narrow = p.staging == FOCSS_STAGING_LOADS && (long long)(p.N1 / l.per_block) * rows < sm_count() &&
                        p.N1 % l.per_block_narrow == 0;
    const int kind = p.staging != FOCSS_STAGING_LOADS ? 2 : narrow ? 3 : 1;
    int R = narrow ? l.per_block_narrow : l.per_block;
    const size_t smem = sizeof(float4) * ((size_t)p.N2 + 512) + sizeof(float2) * (size_t)R * Q * (P + 1);
    cudaError_t e = cached_launch(kind, p.log2N2, smem, &l);
    if (e != cudaSuccess) return e;
    a.N = p.N;
    a.N1 = p.N1;
    a.N2 = p.N2;
    a.log2N2 = p.log2N2;
    a.tw = p.tw;
    a.batch = batch;
    if (p.N1 % R != 0) return cudaErrorInvalidValue;
    return launch_pass(l, dim3(p.N1 / R, batch * (a.modes > 1 ? a.modes : 1)), l.threads, smem, s, a);
}

// ---------------------------------------------------------------- SSFM driver
namespace {
// Event triples (before column pass, between, after row pass) for the
// instrumentation mode; consumed by prof_collect after the run synchronizes.
size_t prof_used = 0;
cudaEvent_t* prof_events(Ctx* ctx, int n) {
    while (ctx->prof_events.size() < prof_used + n) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        ctx->prof_events.push_back(e);
    }
    cudaEvent_t* r = ctx->prof_events.data() + prof_used;
    prof_used += n;
    return r;
}
void prof_collect(Ctx* ctx) {
    for (size_t i = 0; i + 2 < prof_used; i += 3) {
        float a = 0, b = 0;
        cudaEventElapsedTime(&a, ctx->prof_events[i], ctx->prof_events[i + 1]);
        cudaEventElapsedTime(&b, ctx->prof_events[i + 1], ctx->prof_events[i + 2]);
        ctx->prof_ms[0] += a;
        ctx->prof_ms[1] += b;
        ctx->prof_launches[0] += 1;
        ctx->prof_launches[1] += 1;
    }
    prof_used = 0;
}
}  // namespace

focss_status ssfm_validate(Ctx* ctx, const Field* f, const focss_fiber& fib, const focss_ssfm_opts& o) {
    if (f->modes != 1 && f->modes != 2)
        return set_error(ctx, FOCSS_ERR_UNSUPPORTED, "ssfm_run: fields of 1 or 2 modes are implemented");
    if (!fft_size_supported(f->samples))
        return set_error(ctx, FOCSS_ERR_UNSUPPORTED,
                         "field length " + std::to_string(f->samples) + " is not a power of two in [2^8, 2^20]");
    if (o.grid == FOCSS_UNIFORM && o.total_steps <= 0)
        return set_error(ctx, FOCSS_ERR_INVALID_ARG, "ssfm_run: total_steps must be > 0 for UNIFORM");
    if (o.grid != FOCSS_UNIFORM && (!(o.maximum_step_size > 0) || !(o.maximum_phase_shift > 0)))
        return set_error(ctx, FOCSS_ERR_INVALID_ARG,
                         "ssfm_run: maximum_step_size and maximum_phase_shift must be > 0");
    if (o.grid == FOCSS_LOGARITHMIC && !(fib.alpha != 0))
        return set_error(ctx, FOCSS_ERR_INVALID_ARG, "ssfm_run: LOGARITHMIC grid needs alpha != 0");
    if (!(fib.length > 0)) return set_error(ctx, FOCSS_ERR_INVALID_ARG, "ssfm_run: fiber length must be > 0");
    if (o.grid < 0 || o.grid > 2) return set_error(ctx, FOCSS_ERR_INVALID_ARG, "ssfm_run: unknown grid");
    return FOCSS_OK;
}

PassArgs ssfm_args(const Field* f, const focss_fiber& fib, const focss_ssfm_opts& o, double dir, SsfmState* state,
                   int* n_done) {
    const int N = f->samples;
    PassArgs a{};
    a.data = f->d;
    a.state = state;
    a.prm.alpha = fib.alpha;
    a.prm.beta2 = fib.beta2;
    a.prm.gamma = fib.gamma;
    a.prm.kappa = fib.kappa;
    a.prm.length = fib.length;
    a.prm.direction = dir;
    a.prm.max_phase = o.maximum_phase_shift;
    a.prm.max_step = o.maximum_step_size;
    a.prm.dw = 2.0 * 3.14159265358979323846 / (f->dt * N);  // Field::dw (field.cpp:220)
    a.prm.grid = o.grid;
    a.prm.total_steps = o.total_steps;
    a.prm.samples = N;
    a.prm.n_done = n_done;
    ssfm_derive(a.prm);
    a.modes = f->modes;
    return a;
}

focss_status ssfm_plan(Ctx* ctx, int N, const Plan** out) {
    auto it = ctx->ssfm_split.find(N);
    int l1 = it != ctx->ssfm_split.end() ? it->second : default_split(N);
    if (l1 == kSingleCta) l1 = block_split(N);
    return get_plan_split(ctx, N, l1, out);
}

bool ssfm_single_cta(const Ctx* ctx, const Field* f) {
    auto it = ctx->ssfm_split.find(f->samples);
    return it != ctx->ssfm_split.end() && it->second == kSingleCta && f->modes == 1 && block_split(f->samples) != 0;
}

focss_status ssfm_finish(Ctx* ctx, Field* f, const focss_ssfm_opts& o, int* steps_out, int* recorded_out);

focss_status ssfm_run(Ctx* ctx, Field* f, const focss_fiber& fib, const focss_ssfm_opts& o, double dir,
                      int* steps_out, const StepGrid* grid, int* recorded_out) {
    focss_status st = ssfm_validate(ctx, f, fib, o);
    if (st != FOCSS_OK) return st;
    const Plan* p = nullptr;
    st = ssfm_plan(ctx, f->samples, &p);
    if (st != FOCSS_OK) return st;
    st = ensure_state(ctx, f->batch);
    if (st != FOCSS_OK) return st;
    cudaStream_t s = ctx->stream;
    st = cuda_check(ctx, cudaMemsetAsync(ctx->d_state, 0, sizeof(SsfmState) * f->batch, s), "memset state");
    if (st != FOCSS_OK) return st;
    st = cuda_check(ctx, cudaMemsetAsync(ctx->d_counters, 0, sizeof(int) * 4, s), "memset counters");
    if (st != FOCSS_OK) return st;
    PassArgs a = ssfm_args(f, fib, o, dir, ctx->d_state, ctx->d_counters);
    a.fault = ctx->d_counters + 2;
    if (grid) {
        a.prm.h_record = grid->record;
        a.prm.h_replay = grid->replay;
        a.prm.h_count = grid->count;
        a.prm.h_cap = grid->cap;
    }
    const bool replay = grid && grid->replay;

    // Upper bound on column passes: UNIFORM and replayed grids are exact; the
    // others are polled.
    long long cap;
    if (replay) {
        cap = (long long)grid->max_steps + 2;
    } else if (o.grid == FOCSS_UNIFORM) {
        cap = (long long)o.total_steps + 2;
    } else {
        cap = 1ll << 17;  // ~100x the step count of a 0.005 rad/step span at +11 dBm
    }
    if (ssfm_single_cta(ctx, f)) {
        st = cuda_check(ctx, launch_block(*p, a, f->batch, (int)std::min<long long>(cap, 1 << 30), s), "ssfm block");
        if (st != FOCSS_OK) return st;
        st = ssfm_finish(ctx, f, o, steps_out, recorded_out);
        // the kernel stops a realization at the cap, leaving it unfinished
        return st == FOCSS_ERR_TIMEOUT ? set_error(ctx, FOCSS_ERR_NOT_CONVERGED, "ssfm_run: step cap reached") : st;
    }
    const bool fixed = replay || o.grid == FOCSS_UNIFORM;  // pass count known up front
    const int chunk = 16;
    long long launched = 0;
    bool done = false;
    cudaEvent_t ev = nullptr;
    if (!fixed) {
        st = cuda_check(ctx, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
        if (st != FOCSS_OK) return st;
    }
    bool pending = false;
    while (!done) {
        const long long n = fixed ? cap : chunk;
        for (long long i = 0; i < n; ++i) {
            cudaError_t e = cudaSuccess;
            if (ctx->profiling) {
                cudaEvent_t* pe = prof_events(ctx, 3);
                if (!pe) e = cudaErrorMemoryAllocation;
                if (e == cudaSuccess) e = cudaEventRecord(pe[0], s);
                if (e == cudaSuccess) e = launch_col(*p, a, f->batch, s);
                if (e == cudaSuccess) e = cudaEventRecord(pe[1], s);
                if (e == cudaSuccess) e = launch_row(*p, a, f->batch, s);
                if (e == cudaSuccess) e = cudaEventRecord(pe[2], s);
            } else {
                e = launch_col(*p, a, f->batch, s);
                if (e == cudaSuccess) e = launch_row(*p, a, f->batch, s);
            }
            if (e != cudaSuccess) {
                if (ev) cudaEventDestroy(ev);
                return cuda_check(ctx, e, "ssfm pass launch");
            }
        }
        launched += n;
        if (fixed) break;
        // Double-buffered poll: queue the next chunk before waiting on this one.
        if (pending) {
            cudaError_t e = cudaEventSynchronize(ev);
            if (e != cudaSuccess) {
                cudaEventDestroy(ev);
                return cuda_check(ctx, e, "ssfm poll");
            }
            if (*(volatile int*)ctx->h_pinned >= f->batch) done = true;
        }
        if (!done) {
            cudaMemcpyAsync(ctx->h_pinned, ctx->d_counters, sizeof(int), cudaMemcpyDeviceToHost, s);
            cudaEventRecord(ev, s);
            pending = true;
        }
        if (launched > cap) {
            cudaEventDestroy(ev);
            return set_error(ctx, FOCSS_ERR_NOT_CONVERGED, "ssfm_run: step cap reached");
        }
    }
    if (ev) cudaEventDestroy(ev);
    return ssfm_finish(ctx, f, o, steps_out, recorded_out);
}

// Reads the step states back after a run: every realization must be idle;
// steps_out gets the step counts, recorded_out the recorded step-size counts.
focss_status ssfm_finish(Ctx* ctx, Field* f, const focss_ssfm_opts& o, int* steps_out, int* recorded_out) {
    cudaStream_t s = ctx->stream;
    focss_status st;
    std::vector<SsfmState> hs(f->batch);
    int fault = 0;
    st = cuda_check(ctx,
                    cudaMemcpyAsync(hs.data(), ctx->d_state, sizeof(SsfmState) * f->batch,
                                    cudaMemcpyDeviceToHost, s),
                    "state readback");
    if (st != FOCSS_OK) return st;
    st = cuda_check(ctx, cudaMemcpyAsync(&fault, ctx->d_counters + 2, sizeof(int), cudaMemcpyDeviceToHost, s),
                    "fault readback");
    if (st != FOCSS_OK) return st;
    st = cuda_check(ctx, cudaStreamSynchronize(s), "ssfm sync");
    if (st != FOCSS_OK) return st;
    if (fault) return set_error(ctx, FOCSS_ERR_TIMEOUT, "ssfm_run: a bulk-copy wait ran out");
    if (ctx->profiling) prof_collect(ctx);
    for (int b = 0; b < f->batch; ++b) {
        if (hs[b].action != COL_IDLE)
            return set_error(ctx, FOCSS_ERR_TIMEOUT, "ssfm_run: a realization did not finish");
        if (steps_out) steps_out[b] = (o.grid == FOCSS_ADAPTIVE) ? hs[b].steps : hs[b].n_steps;
        if (recorded_out) recorded_out[b] = hs[b].recorded;
    }
    return FOCSS_OK;
}

// ---------------------------------------------------------------- plain FFTs
focss_status fft_forward_transposed(Ctx* ctx, float2* data, int N, int batch, float scale) {
    const Plan* p = nullptr;
    focss_status st = get_plan(ctx, N, &p);
    if (st != FOCSS_OK) return st;
    PassArgs a{};
    a.data = data;
    a.op = COL_FWD;
    cudaError_t e = launch_col(*p, a, batch, ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, "fft col");
    a.op = ROW_FWD;
    a.scale = scale;
    return cuda_check(ctx, launch_row(*p, a, batch, ctx->stream), "fft row");
}

focss_status fft_inverse_transposed(Ctx* ctx, float2* data, int N, int batch) {
    const Plan* p = nullptr;
    focss_status st = get_plan(ctx, N, &p);
    if (st != FOCSS_OK) return st;
    PassArgs a{};
    a.data = data;
    a.op = ROW_INV;
    cudaError_t e = launch_row(*p, a, batch, ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, "ifft row");
    a.op = COL_INV;
    return cuda_check(ctx, launch_col(*p, a, batch, ctx->stream), "ifft col");
}

focss_status spectral_apply(Ctx* ctx, float2* data, int N, int batch, int row_op, const float2* table,
                            float scale, int bp_cut) {
    const Plan* p = nullptr;
    focss_status st = get_plan(ctx, N, &p);
    if (st != FOCSS_OK) return st;
    PassArgs a{};
    a.data = data;
    a.op = COL_FWD;
    cudaError_t e = launch_col(*p, a, batch, ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, "spectral col");
    a.op = row_op;
    a.table = table;
    a.scale = scale;
    a.bp_cut = bp_cut;
    e = launch_row(*p, a, batch, ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, "spectral row");
    a.op = COL_INV;
    return cuda_check(ctx, launch_col(*p, a, batch, ctx->stream), "spectral col inv");
}

focss_status fft_forward(Ctx* ctx, float2* data, int N, int batch) {
    const Plan* p = nullptr;
    focss_status st = get_plan(ctx, N, &p);
    if (st != FOCSS_OK) return st;
    st = fft_forward_transposed(ctx, data, N, batch, 1.0f / (float)N);
    if (st != FOCSS_OK) return st;
    float2* tmp = (float2*)scratch_buffer(ctx, 0, sizeof(float2) * (size_t)N * batch);
    if (!tmp) return set_error(ctx, FOCSS_ERR_OOM, "fft scratch");
    cudaError_t e = launch_transpose_to_natural(data, tmp, p->N1, p->N2, batch, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(data, tmp, sizeof(float2) * (size_t)N * batch, cudaMemcpyDeviceToDevice, ctx->stream);
    return cuda_check(ctx, e, "fft transpose");
}

focss_status fft_inverse(Ctx* ctx, float2* data, int N, int batch) {
    const Plan* p = nullptr;
    focss_status st = get_plan(ctx, N, &p);
    if (st != FOCSS_OK) return st;
    float2* tmp = (float2*)scratch_buffer(ctx, 0, sizeof(float2) * (size_t)N * batch);
    if (!tmp) return set_error(ctx, FOCSS_ERR_OOM, "ifft scratch");
    cudaError_t e = launch_transpose_from_natural(data, tmp, p->N1, p->N2, batch, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(data, tmp, sizeof(float2) * (size_t)N * batch, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, "ifft transpose");
    return fft_inverse_transposed(ctx, data, N, batch);
}

}  // namespace fg
