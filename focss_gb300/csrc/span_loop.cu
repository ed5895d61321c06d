// span_loop.cu -- span loops recorded as CUDA graphs, over several fields at
// once, and the split-step FFT autotuner.
//
// A span loop (forward_propagation / backward_propagation,
// src/tasks/systems.cpp:26-91) is a long, fixed chain of small launches:
// per span an optional amplifier, one SSFM run (K+2 column/row pass pairs for
// a UNIFORM grid, a data-dependent number for ADAPTIVE / LOGARITHMIC) and
// another optional amplifier.  Here the whole chain, for every field of the
// call, is captured once into one graph:
//   * each field is one branch (fields of different lengths and batches run
//     concurrently and fill the GPU together);
//   * UNIFORM spans are plain pass sequences;
//   * ADAPTIVE / LOGARITHMIC spans are a conditional WHILE node whose body is
//     kChunk pass pairs plus a one-thread check kernel; the check ends the loop
//     once the SSFM state machines of all realizations report the span done
//     (the counter they increment on completion), or after kMaxPairs passes,
//     so the loop is bounded whatever the data;
//   * amplifier noise reads its seed and counter from device memory, so a
//     replay with new noise needs no re-capture.
// Passes of a realization that already finished are no-ops (the kernels
// return on its idle state), so the chunked loop gives the same result as the
// host-polled ssfm_run.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace fg {

struct LoopGraph {
    cudaGraphExec_t exec = nullptr;
    SsfmState* d_state = nullptr;         // every field's realizations
    int* d_ctr = nullptr;                 // kCtr counters per field
    int* d_steps = nullptr;               // steps per realization, summed over spans
    unsigned long long* d_amp = nullptr;  // {seed, counter0} per field
    std::vector<int> offset, batch;       // first realization and batch of each field
    int total = 0;
    long long static_kernels = 0;         // kernel nodes outside loop bodies
    std::vector<int> body_kernels;        // kernels per loop-body iteration, per field
};

namespace {
// Per-field counters: [0] realizations that finished the current span (the
// SSFM state machine's n_done), [1] loop iterations in the current span,
// [2] step cap hit, [3] a realization did not finish, [4] loop iterations
// over all spans.
constexpr int kCtr = 8;
constexpr int kChunk = 8;                // pass pairs per loop-body iteration
constexpr long long kMaxPairs = 1ll << 17;
constexpr int kMaxIter = (int)(kMaxPairs / kChunk);
constexpr size_t kMaxCachedGraphs = 64;

__global__ void loop_check_kernel(int* ctr, int batch, cudaGraphConditionalHandle h) {
    if (threadIdx.x != 0) return;
    const int it = ++ctr[1];
    ++ctr[4];
    const bool pending = *(volatile int*)&ctr[0] < batch;
    if (pending && it >= kMaxIter) ctr[2] = 1;
    cudaGraphSetConditional(h, (pending && it < kMaxIter) ? 1u : 0u);
}

__global__ void span_end_kernel(const SsfmState* __restrict__ st, int batch, int adaptive, int* ctr, int* steps) {
    for (int b = threadIdx.x; b < batch; b += blockDim.x) {
        if (st[b].action != COL_IDLE) atomicOr(&ctr[3], 1);
        steps[b] += adaptive ? st[b].steps : st[b].n_steps;
    }
}

__global__ void amp_graph_kernel(float2* __restrict__ d, int samples, size_t n, float2 scale, float sigma,
                                 const unsigned long long* __restrict__ sc, int span) {
    const unsigned long long seed = sc[0], counter = sc[1] + (unsigned long long)span;
    const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        d[i] = amplifier_sample(d[i], i, samples, scale, sigma, key, (uint32_t)counter, (uint32_t)(counter >> 32));
}

int amp_grid(size_t n) {
    size_t g = (n + 255) / 256;
    if (g > (size_t)sm_count() * 32) g = (size_t)sm_count() * 32;
    return (int)(g ? g : 1);
}

std::string loop_key(int nf, Field* const* fs, const focss_fiber& fib, const focss_ssfm_opts* opts,
                     const focss_amp& amp, int spans, double dir, const Ctx* ctx) {
    std::string k;
    char buf[256];
    std::snprintf(buf, sizeof buf, "%a %a %a %a %a %a|%a %a %d %d|%d %a|", fib.alpha, fib.beta2, fib.gamma,
                  fib.length, fib.wavelength, fib.kappa, amp.gain, amp.noise_factor, amp.before, amp.after, spans,
                  dir);
    k += buf;
    for (int i = 0; i < nf; ++i) {
        const Field* f = fs[i];
        auto it = ctx->ssfm_split.find(f->samples);
        std::snprintf(buf, sizeof buf, "%p %d %d %d %a %a %d %d %a %a %d;", (void*)f->d, f->modes, f->samples,
                      f->batch, f->dt, f->f0, opts[i].grid, opts[i].total_steps, opts[i].maximum_phase_shift,
                      opts[i].maximum_step_size, it == ctx->ssfm_split.end() ? -99 : it->second);
        k += buf;
    }
    return k;
}

void destroy_graph(LoopGraph* g) {
    if (!g) return;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    cudaFree(g->d_state);
    cudaFree(g->d_ctr);
    cudaFree(g->d_steps);
    cudaFree(g->d_amp);
    delete g;
}

cudaError_t ensure_side(Ctx* ctx, size_t streams, size_t events) {
    while (ctx->side_streams.size() < streams) {
        cudaStream_t s;
        cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e != cudaSuccess) return e;
        ctx->side_streams.push_back(s);
    }
    while (ctx->side_events.size() < events) {
        cudaEvent_t e;
        cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        if (r != cudaSuccess) return r;
        ctx->side_events.push_back(e);
    }
    return cudaSuccess;
}

// Records field i's branch (all spans) on stream `s`; `body_stream` captures
// loop bodies.  Returns the first error.
cudaError_t record_branch(Ctx* ctx, LoopGraph* g, int i, Field* f, const Plan& p, const focss_fiber& fib,
                          const focss_ssfm_opts& o, const focss_amp& amp, int spans, double dir, cudaStream_t s,
                          cudaStream_t body_stream) {
    const int B = f->batch;
    SsfmState* state = g->d_state + g->offset[i];
    int* ctr = g->d_ctr + kCtr * i;
    int* steps = g->d_steps + g->offset[i];
    const size_t n = f->n();
    double sc_b = 1, sg_b = 0, sc_a = 1, sg_a = 0;
    if (amp.before != FOCSS_AMP_NONE) amplifier_coeffs(amp.before, amp.gain, amp.noise_factor, f->f0, f->dt, &sc_b, &sg_b);
    if (amp.after != FOCSS_AMP_NONE) amplifier_coeffs(amp.after, amp.gain, amp.noise_factor, f->f0, f->dt, &sc_a, &sg_a);
    const PassArgs a = ssfm_args(f, fib, o, dir, state, ctr);
    cudaError_t e = cudaMemsetAsync(steps, 0, sizeof(int) * B, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctr, 0, sizeof(int) * kCtr, s);
    for (int span = 0; span < spans && e == cudaSuccess; ++span) {
        if (amp.before != FOCSS_AMP_NONE) {
            amp_graph_kernel<<<amp_grid(n), 256, 0, s>>>(f->d, f->samples, n, split_df(sc_b), (float)sg_b,
                                                         g->d_amp + 2 * i, span);
            e = cudaGetLastError();
            g->static_kernels += 1;
        }
        if (e == cudaSuccess) e = cudaMemsetAsync(state, 0, sizeof(SsfmState) * B, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(ctr, 0, sizeof(int) * 2, s);  // [0], [1]: per span
        if (e != cudaSuccess) break;
        if (ssfm_single_cta(ctx, f)) {
            // the whole span in one launch (single-CTA kernel), bounded like the loop below
            e = launch_block(p, a, B, o.grid == FOCSS_UNIFORM ? o.total_steps + 2 : (int)kMaxPairs, s);
            g->static_kernels += 1;
        } else if (o.grid == FOCSS_UNIFORM) {
            for (int k = 0; k < o.total_steps + 2 && e == cudaSuccess; ++k) {
                e = launch_col(p, a, B, s);
                if (e == cudaSuccess) e = launch_row(p, a, B, s);
            }
            g->static_kernels += 2ll * (o.total_steps + 2);
        } else {
            // Conditional WHILE node appended to the branch's capture.
            cudaStreamCaptureStatus cs;
            cudaGraph_t graph = nullptr;
            const cudaGraphNode_t* deps = nullptr;
            const cudaGraphEdgeData* edges = nullptr;
            size_t ndeps = 0;
            e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, &deps, &edges, &ndeps);
            if (e != cudaSuccess) break;
            if (cs != cudaStreamCaptureStatusActive) {
                e = cudaErrorStreamCaptureInvalidated;
                break;
            }
            cudaGraphConditionalHandle h;
            e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
            if (e != cudaSuccess) break;
            cudaGraphNodeParams cp{};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = h;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t node;
            e = cudaGraphAddNode(&node, graph, deps, edges, ndeps, &cp);
            if (e != cudaSuccess) break;
            e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
            if (e != cudaSuccess) break;
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            e = cudaStreamBeginCaptureToGraph(body_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
            if (e != cudaSuccess) break;
            for (int c = 0; c < kChunk && e == cudaSuccess; ++c) {
                e = launch_col(p, a, B, body_stream);
                if (e == cudaSuccess) e = launch_row(p, a, B, body_stream);
            }
            if (e == cudaSuccess) {
                loop_check_kernel<<<1, 32, 0, body_stream>>>(ctr, B, h);
                e = cudaGetLastError();
            }
            cudaGraph_t done = nullptr;
            const cudaError_t e2 = cudaStreamEndCapture(body_stream, &done);
            if (e == cudaSuccess) e = e2;
            g->body_kernels[i] = 2 * kChunk + 1;
            if (e != cudaSuccess) break;
        }
        span_end_kernel<<<1, 256, 0, s>>>(state, B, o.grid == FOCSS_ADAPTIVE, ctr, steps);
        e = cudaGetLastError();
        g->static_kernels += 1;
        if (e == cudaSuccess && amp.after != FOCSS_AMP_NONE) {
            amp_graph_kernel<<<amp_grid(n), 256, 0, s>>>(f->d, f->samples, n, split_df(sc_a), (float)sg_a,
                                                         g->d_amp + 2 * i, span);
            e = cudaGetLastError();
            g->static_kernels += 1;
        }
    }
    return e;
}

focss_status build_graph(Ctx* ctx, LoopGraph* g, int nf, Field* const* fs, const std::vector<const Plan*>& plans,
                         const focss_fiber& fib, const focss_ssfm_opts* opts, const focss_amp& amp, int spans,
                         double dir) {
    g->offset.resize(nf);
    g->batch.resize(nf);
    g->body_kernels.assign(nf, 0);
    for (int i = 0; i < nf; ++i) {
        g->offset[i] = g->total;
        g->batch[i] = fs[i]->batch;
        g->total += fs[i]->batch;
    }
    cudaError_t e = cudaMalloc(&g->d_state, sizeof(SsfmState) * g->total);
    if (e == cudaSuccess) e = cudaMalloc(&g->d_ctr, sizeof(int) * kCtr * nf);
    if (e == cudaSuccess) e = cudaMalloc(&g->d_steps, sizeof(int) * g->total);
    if (e == cudaSuccess) e = cudaMalloc(&g->d_amp, sizeof(unsigned long long) * 2 * nf);
    if (e == cudaSuccess) e = ensure_side(ctx, (size_t)nf + 1, (size_t)nf + 1);
    if (e != cudaSuccess) return cuda_check(ctx, e, "span loop set-up");

    cudaStream_t s = ctx->stream;
    cudaStream_t body_stream = ctx->side_streams[nf];
    set_capturing(true);
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
        set_capturing(false);
        return cuda_check(ctx, e, "span loop capture");
    }
    cudaEvent_t fork = ctx->side_events[nf];
    e = cudaEventRecord(fork, s);
    for (int i = 0; i < nf && e == cudaSuccess; ++i) {
        cudaStream_t b = ctx->side_streams[i];
        e = cudaStreamWaitEvent(b, fork, 0);
        if (e == cudaSuccess) e = record_branch(ctx, g, i, fs[i], *plans[i], fib, opts[i], amp, spans, dir, b, body_stream);
        // always join, so that the capture can be ended cleanly
        const cudaError_t e1 = cudaEventRecord(ctx->side_events[i], b);
        const cudaError_t e2 = cudaStreamWaitEvent(s, ctx->side_events[i], 0);
        if (e == cudaSuccess) e = e1 != cudaSuccess ? e1 : e2;
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(s, &graph);
    set_capturing(false);
    if (e == cudaSuccess) e = ee;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return cuda_check(ctx, e, "span loop graph");
}
}  // namespace

void free_loop_graphs(Ctx* ctx) {
    for (auto& kv : ctx->loops) destroy_graph(kv.second);
    ctx->loops.clear();
    for (cudaStream_t s : ctx->side_streams) cudaStreamDestroy(s);
    ctx->side_streams.clear();
    for (cudaEvent_t e : ctx->side_events) cudaEventDestroy(e);
    ctx->side_events.clear();
}

}  // namespace fg

using fg::Ctx;
using fg::Field;

extern "C" {

FOCSS_API focss_status focss_span_loop(focss_ctx* c, int n_fields, focss_field* const* fields,
                                       const focss_fiber* fiber, const focss_ssfm_opts* opts, const focss_amp* amp,
                                       int spans, double direction, int* steps_out) {
    if (!c || n_fields <= 0 || !fields || !fiber || !opts || !amp || spans < 0) return FOCSS_ERR_INVALID_ARG;
    if (n_fields > 256) return fg::set_error(c, FOCSS_ERR_UNSUPPORTED, "span_loop: at most 256 fields per call");
    for (int i = 0; i < n_fields; ++i)
        if (!fields[i]) return FOCSS_ERR_INVALID_ARG;
    for (int op : {amp->before, amp->after})
        if (op != FOCSS_AMP_NONE && (op < FOCSS_AMP_AMPLIFY || op > FOCSS_AMP_DROP_POWER))
            return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "span_loop: unknown amplifier op");
    if ((amp->before != FOCSS_AMP_NONE || amp->after != FOCSS_AMP_NONE) && !(amp->gain > 0))
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "span_loop: amplifier gain must be > 0");
    if (spans == 0) return FOCSS_OK;
    Field* const* fs = reinterpret_cast<Field* const*>(fields);
    std::vector<const fg::Plan*> plans(n_fields);
    for (int i = 0; i < n_fields; ++i) {
        if (fs[i]->ctx != c) return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "span_loop: field of another context");
        for (int j = 0; j < i; ++j)
            if (fs[j]->d == fs[i]->d) return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "span_loop: a field is listed twice");
        focss_status st = fg::ssfm_validate(c, fs[i], *fiber, opts[i]);
        if (st != FOCSS_OK) return st;
        st = fg::ssfm_plan(c, fs[i]->samples, &plans[i]);
        if (st != FOCSS_OK) return st;
    }
    const std::string key = fg::loop_key(n_fields, fs, *fiber, opts, *amp, spans, direction, c);
    fg::LoopGraph* g = nullptr;
    auto it = c->loops.find(key);
    if (it != c->loops.end()) {
        g = it->second;
    } else {
        if (c->loops.size() >= fg::kMaxCachedGraphs) {
            cudaStreamSynchronize(c->stream);
            for (auto& kv : c->loops) fg::destroy_graph(kv.second);
            c->loops.clear();
        }
        g = new fg::LoopGraph();
        focss_status st = fg::build_graph(c, g, n_fields, fs, plans, *fiber, opts, *amp, spans, direction);
        if (st != FOCSS_OK) {
            fg::destroy_graph(g);
            return st;
        }
        c->loops[key] = g;
    }
    std::vector<unsigned long long> sc(2 * (size_t)n_fields);
    for (int i = 0; i < n_fields; ++i) {
        sc[2 * i] = amp->seed + (unsigned long long)i;
        sc[2 * i + 1] = amp->counter0;
    }
    cudaStream_t s = c->stream;
    cudaError_t e = cudaMemcpyAsync(g->d_amp, sc.data(), sizeof(unsigned long long) * sc.size(),
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaGraphLaunch(g->exec, s);
    std::vector<int> ctr(fg::kCtr * (size_t)n_fields), steps(g->total);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctr.data(), g->d_ctr, sizeof(int) * ctr.size(), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(steps.data(), g->d_steps, sizeof(int) * steps.size(), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fg::cuda_check(c, e, "span loop run");
    long long kernels = g->static_kernels;
    for (int i = 0; i < n_fields; ++i) kernels += (long long)ctr[fg::kCtr * i + 4] * g->body_kernels[i];
    fg::count_launch_graph(kernels);
    for (int i = 0; i < n_fields; ++i) {
        if (ctr[fg::kCtr * i + 2])
            return fg::set_error(c, FOCSS_ERR_NOT_CONVERGED, "span_loop: step cap reached (field " + std::to_string(i) + ")");
        if (ctr[fg::kCtr * i + 3]) {
            // a single-CTA run stops a realization at the step cap, unfinished
            if (fg::ssfm_single_cta(c, fs[i]))
                return fg::set_error(c, FOCSS_ERR_NOT_CONVERGED, "span_loop: step cap reached (field " + std::to_string(i) + ")");
            return fg::set_error(c, FOCSS_ERR_TIMEOUT, "span_loop: a realization did not finish (field " + std::to_string(i) + ")");
        }
    }
    if (steps_out) std::copy(steps.begin(), steps.end(), steps_out);
    return FOCSS_OK;
}

FOCSS_API focss_status focss_set_fft_split(focss_ctx* c, int samples, int log2_n1) {
    if (!c) return FOCSS_ERR_INVALID_ARG;
    if (log2_n1 == 0) {
        c->ssfm_split.erase(samples);
        return FOCSS_OK;
    }
    if (log2_n1 == fg::kSingleCta) {
        if (!fg::block_split(samples))
            return fg::set_error(c, FOCSS_ERR_UNSUPPORTED, "set_fft_split: the single-CTA kernel covers 2^12..2^14");
        c->ssfm_split[samples] = log2_n1;
        return FOCSS_OK;
    }
    if (!fg::split_supported(samples, log2_n1))
        return fg::set_error(c, FOCSS_ERR_UNSUPPORTED, "set_fft_split: split outside [2^4, 2^10] x [2^4, 2^10]");
    c->ssfm_split[samples] = log2_n1;
    return FOCSS_OK;
}

FOCSS_API focss_status focss_autotune(focss_ctx* c, int samples, int batch, int* log2_n1, double* ms_per_step) {
    if (!c || batch <= 0) return FOCSS_ERR_INVALID_ARG;
    if (!fg::fft_size_supported(samples))
        return fg::set_error(c, FOCSS_ERR_UNSUPPORTED, "autotune: length is not a power of two in [2^8, 2^20]");
    int lg = 0;
    while ((1 << lg) < samples) ++lg;
    Field f;
    f.ctx = c;
    f.modes = 1;
    f.samples = samples;
    f.batch = batch;
    f.dt = 1.0 / 512e9;
    f.f0 = 299792458.0 / 1.55e-6;
    cudaStream_t s = c->stream;
    cudaError_t e = cudaMalloc(&f.d, sizeof(float2) * f.n());
    if (e != cudaSuccess) return fg::cuda_check(c, e, "autotune scratch");
    // Gaussian field of ~1 mW per sample: a representative nonlinear phase.
    e = cudaMemsetAsync(f.d, 0, sizeof(float2) * f.n(), s);
    if (e == cudaSuccess) e = fg::launch_amplifier(f.d, 1, samples, batch, 0.0, std::sqrt(0.5e-3f), 17, 0, s);
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    const focss_fiber fib{0.2e-3 * std::log(10.0) / 10, -2.168e-26, 1.3e-3, 8e3, 1.55e-6, 1.0};
    const focss_ssfm_opts o{FOCSS_UNIFORM, 8, 0.0, 0.0};
    const auto saved = c->ssfm_split;
    // candidates: every two-pass split, and the single-CTA kernel where it exists
    std::vector<int> cands;
    for (int l1 = 4; l1 <= 10; ++l1)
        if (fg::split_supported(samples, l1)) cands.push_back(l1);
    if (fg::block_split(samples)) cands.push_back(fg::kSingleCta);
    constexpr int kNone = -100;
    int best = kNone;
    double best_ms = 1e300;
    focss_status st = fg::cuda_check(c, e, "autotune set-up");
    for (size_t ci = 0; ci < cands.size() && st == FOCSS_OK; ++ci) {
        const int l1 = cands[ci];
        c->ssfm_split[samples] = l1;
        st = fg::ssfm_run(c, &f, fib, o, FOCSS_FORWARD, nullptr);  // warm-up (plan, attributes)
        if (st != FOCSS_OK) break;
        double ms = 1e300;
        for (int rep = 0; rep < 3 && st == FOCSS_OK; ++rep) {
            e = cudaEventRecord(t0, s);
            if (e == cudaSuccess) st = fg::ssfm_run(c, &f, fib, o, FOCSS_FORWARD, nullptr);
            if (e == cudaSuccess && st == FOCSS_OK) e = cudaEventRecord(t1, s);
            if (e == cudaSuccess && st == FOCSS_OK) e = cudaEventSynchronize(t1);
            float t = 0;
            if (e == cudaSuccess && st == FOCSS_OK) e = cudaEventElapsedTime(&t, t0, t1);
            if (e != cudaSuccess) st = fg::cuda_check(c, e, "autotune timing");
            if (st == FOCSS_OK) ms = std::min(ms, (double)t / o.total_steps);
        }
        if (st == FOCSS_OK && ms < best_ms) {
            best_ms = ms;
            best = l1;
        }
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    cudaStreamSynchronize(s);
    cudaFree(f.d);
    c->ssfm_split = saved;
    if (st != FOCSS_OK) return st;
    if (best == kNone) return fg::set_error(c, FOCSS_ERR_UNSUPPORTED, "autotune: no admissible split");
    c->ssfm_split[samples] = best;
    if (log2_n1) *log2_n1 = best;
    if (ms_per_step) *ms_per_step = best_ms;
    return FOCSS_OK;
}

}  // extern "C"
