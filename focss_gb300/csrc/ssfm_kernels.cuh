// ssfm_kernels.cuh -- device code of the two-pass split-step kernels (see ssfm.cu
// for the algorithm).  Each FFT length is instantiated in its own translation
// unit (ssfm_len_*.cu) so the build compiles them in parallel.
#pragma once
#include <cmath>

#include <cuda.h>  // CUtensorMap

#include "fft.cuh"
#include "internal.h"

namespace fg {

// ---------------------------------------------------------------- state update
// The state update runs on one thread between the passes of every split step,
// so its FP64 dependency chain is on the critical path of small launches
// (FP64 instructions have long latency on this GPU: the library exp() alone
// takes ~1600 cycles).  The per-run constants come precomputed in SsfmParams
// (ssfm_derive) and the per-step exponential is the short-chain one below.

// exp(x), |x| < 700, to ~2 ulp: Cody & Waite's reduction x = k ln2 + r with a
// two-part ln 2 (the 42-bit head makes k ln2_hi exact for |k| < 2^11),
// |r| <= ln2/2, then the Taylor series of exp(r) to degree 13 (remainder below
// 2^-55 relative) evaluated by Estrin's scheme (depth 4 instead of Horner's
// 13), and 2^k put into the exponent field.
__device__ __forceinline__ double exp_short(double x) {
    constexpr double kLog2e = 1.4426950408889634;
    constexpr double kLn2Hi = 0x1.62e42fefa38p-1, kLn2Lo = 0x1.ef35793c7673p-45;
    constexpr double c2 = 1.0 / 2, c3 = 1.0 / 6, c4 = 1.0 / 24, c5 = 1.0 / 120, c6 = 1.0 / 720,
                     c7 = 1.0 / 5040, c8 = 1.0 / 40320, c9 = 1.0 / 362880, c10 = 1.0 / 3628800,
                     c11 = 1.0 / 39916800, c12 = 1.0 / 479001600, c13 = 1.0 / 6227020800.0;
    const double k = rint(x * kLog2e);
    const double r = fma(-k, kLn2Lo, fma(-k, kLn2Hi, x));
    const double r2 = r * r, r4 = r2 * r2, r8 = r4 * r4;
    const double q0 = fma(r2, fma(r, c3, c2), 1.0 + r);
    const double q1 = fma(r2, fma(r, c7, c6), fma(r, c5, c4));
    const double q2 = fma(r2, fma(r, c11, c10), fma(r, c9, c8));
    const double q3 = fma(r, c13, c12);
    const double e = fma(r8, fma(r4, q3, q2), fma(r4, q1, q0));
    return e * __longlong_as_double((long long)(1023 + (int)k) << 52);
}

__device__ __forceinline__ double adaptive_estimate(const SsfmParams& p, float peak) {
    // src/focss/solver/ssfm.cpp:136-140 (argument = |kappa gamma|, kg_abs)
    const double argument = p.kg_abs;
    const double phase_shift = argument * (double)peak;
    const double h = p.max_phase / phase_shift;
    return p.max_step < h ? p.max_step : h;
}

__device__ __forceinline__ double log_step(const SsfmParams& p, int K, int i) {
    // src/focss/solver/ssfm.cpp:76-84
    const double inv_alpha = -1.0 / p.alpha * p.direction;
    double inv_gain = exp(-p.alpha * p.length) - 1;
    inv_gain /= K;
    return inv_alpha * log(1 + inv_gain / (1 + inv_gain * i));
}

// a (turns, any sign) -> 96-bit two's-complement turn fraction hi*2^-64 + lo*2^-96.
__device__ __forceinline__ void turns_fix96(double a, unsigned long long& hi, unsigned long long& lo) {
    const double ab = fabs(a);
    const double fr = ab - floor(ab);             // exact
    const double s64 = fr * 0x1p64;               // exact, < 2^64
    const double h = floor(s64);
    hi = __double2ull_rz(h);
    lo = __double2ull_rz((s64 - h) * 0x1p32);     // < 2^32
    if (a < 0) {
        if (lo == 0) {
            hi = 0ull - hi;
        } else {
            lo = (1ull << 32) - lo;
            hi = ~hi;
        }
    }
}

// Step i (0-based) of realization b on a replayed grid, signed by the direction.
__device__ __forceinline__ double replay_step(const SsfmParams& p, int b, int i) {
    return p.direction * p.h_replay[(size_t)b * p.h_cap + i];
}

__device__ __noinline__ static void ssfm_advance(SsfmState& s, const SsfmParams& p, int b, int op_done, float peak,
                                                double sum) {
    if (op_done == COL_INV) {
        s.action = COL_IDLE;
        s.row_active = 0;
        atomicAdd(p.n_done, 1);
        return;
    }
    double hl;
    if (op_done == COL_FWD) {
        s.distance = 0;
        s.index = 0;
        s.steps = 1;
        s.gain_ratio = 1.0;
        s.recorded = 0;
        if (p.h_replay) {
            const int n = p.h_count[b];
            s.n_steps = n;
            s.steps = n;
            s.h = replay_step(p, b, 0);
            s.final_step = n == 1;
        } else if (p.grid == FOCSS_UNIFORM) {
            s.n_steps = p.total_steps;
            s.h = p.direction * (p.length / p.total_steps);
            s.final_step = p.total_steps == 1;
        } else if (p.grid == FOCSS_LOGARITHMIC) {
            // src/focss/solver/ssfm.cpp:120-134
            const double avg = sum / p.samples;
            const double L_nl = 1.0 / p.gamma / avg;
            const double CL = p.max_phase * L_nl / p.kappa;
            const double L_eff = (1.0 - exp(-p.alpha * p.length)) / p.alpha;
            const double L_nl_eff = (1.0 - exp(-p.alpha * CL)) / p.alpha;
            const int est = (int)(L_eff / L_nl_eff);
            const int mn = (int)(p.length / p.max_step);
            const int K = mn > est ? mn : est;
            s.n_steps = K;
            s.h = log_step(p, K, 0);
            s.final_step = K == 1;
        } else {
            const double h0 = adaptive_estimate(p, peak);
            if (h0 < p.length) {
                s.h = p.direction * h0;
                s.final_step = 0;
            } else {
                s.h = p.direction * p.length;
                s.final_step = 1;
            }
        }
        hl = 0.5 * s.h;
        s.action = COL_KERR;
    } else {  // COL_KERR finished with step s.h
        if (s.final_step) {
            hl = 0.5 * s.h;
            s.action = COL_INV;
        } else {
            double next;
            int fin;
            if (p.h_replay) {
                const int i = ++s.index;
                next = replay_step(p, b, i);
                fin = (i == s.n_steps - 1);
            } else if (p.grid == FOCSS_UNIFORM) {
                const int i = ++s.index;
                next = s.h;
                fin = (i == s.n_steps - 1);
            } else if (p.grid == FOCSS_LOGARITHMIC) {
                const int i = ++s.index;
                next = log_step(p, s.n_steps, i);
                fin = (i == s.n_steps - 1);
            } else {
                s.distance += fabs(s.h);
                s.steps++;
                const double nm = adaptive_estimate(p, peak);
                if (s.distance + nm < p.length) {
                    next = p.direction * nm;
                    fin = 0;
                } else {
                    next = p.direction * (p.length - s.distance);
                    fin = 1;
                }
            }
            hl = 0.5 * (s.h + next);
            s.h = next;
            s.final_step = fin;
        }
    }
    if (p.h_record && s.action == COL_KERR) {
        // the nonlinear step about to be taken (s.h) is step s.recorded
        if (s.recorded < p.h_cap) p.h_record[(size_t)b * p.h_cap + s.recorded] = fabs(s.h);
        s.recorded++;
    }
    // A linear step equal to the previous one (UNIFORM grids, ADAPTIVE steps
    // at the maximum step size) keeps its dispersion phase and loss factor:
    // the same values a recomputation would give, without its FP64 chain.
    double g;
    if (op_done == COL_KERR && hl == s.hl) {
        g = s.g_exact;
    } else {
        turns_fix96(p.disp_c * hl, s.disp_hi, s.disp_lo);  // beta2/2 hl dw^2 in turns
        g = exp_short(p.loss_c * hl) * p.inv_samples;
        s.g_exact = g;
    }
    s.hl = hl;
    // FP32 gain with error feedback: the running product of applied gains
    // tracks the exact FP64 product to one rounding instead of drifting.
    // ratio' = t / g32 = 1 + (t - g32) / g32 with t - g32 exact (Sterbenz) and
    // ~2^-24 relative, so the FP32 reciprocal of g32 carries it to ~2^-48.
    const double t = g * s.gain_ratio;
    const float g32 = (float)t;
    s.gain_ratio = fma(t - (double)g32, (double)__frcp_rn(g32), 1.0);
    s.lin_gain = g32;
    s.row_active = 1;
    s.kerr_coef = (float)(p.kg * s.h);
}

// Column-pass tile width: 16 columns (128-byte rows) below N1 = 512, 8 from
// there (N1 = 1024: keeps 256 threads and its per-thread register budget;
// N1 = 512: 256-thread CTAs, four per SM instead of two of 512 at the same
// 64 registers, so one CTA's barriers stall fewer warps -- 126 x 2^19
// column pass 0.414 -> 0.400 ms; 4 columns, with 32-byte row segments,
// measured 0.525 ms).  MINB is the CTAs per SM of (up to) two
// mode groups the launch bound sizes the register budget for.
template <int N1>
struct ColShape {
    static constexpr int C = N1 >= 512 ? 8 : 16;
    static constexpr int MINB = N1 == 512 ? 2 : 1;
    // 64-thread CTAs (2 columns at N1 = 512, 4 at 256) when a launch has fewer
    // column blocks than the GPU has SMs: a single 2^17 field at a 512 x 256
    // split has 16 blocks of 16 columns, which leaves 136 SMs idle while each
    // of the 16 runs 16 warps through the whole transform pair.
    static constexpr int CN = 64 / ColFFT<N1>::P < C ? 64 / ColFFT<N1>::P : C;
};

// ---------------------------------------------------------------- column pass
// The work of one thread group (C columns x P threads, `gt` its thread index)
// on columns [n2_0, n2_0 + C) of one mode of one realization; `data` points
// at that mode's first sample and rows are `ld` samples apart (N2 in global
// memory for the two-pass kernels; padded in the single-CTA kernel's shared
// memory).  `sB` holds the six-step
// factors W_N^{n2 a1 j} of these columns at sB[j * sB_stride + c].  Adds the
// time-domain field's peak and sum of |A|^2 to pk / sm.
template <int N1, int C>
__device__ __forceinline__ void col_work(const PassArgs& a, int op, const SsfmState* st, float2* data, int n2_0,
                                         const float4* s_fc, const float4* sB, int sB_stride, float2* sx,
                                         float2* s_x0, int mo, int modes, int gt, int ld, float& pk, float& sm,
                                         const float2* src = nullptr, int src_ld = 0) {
    constexpr int P = ColFFT<N1>::P, Q = ColFFT<N1>::Q;
    constexpr bool PAIR = ColFFT<N1>::PAIR;
    // Element j of a thread is time-domain row t + P j; in the spectral
    // layout it is row a0 + a1 j (a0 = t, a1 = P for the PQ form; lane-pair
    // form: a0 = (t>>1) + Q^2 (t&1), a1 = Q).  Six-step twiddle of column n2:
    // W_N^{n2 (a0 + a1 j)} = W_N^{n2 a0} (per thread) x W_N^{n2 a1 j} (per
    // column table over j), each a quarter turn times a lifting rotation whose
    // inverse mirrors it exactly.
    constexpr int a1 = PAIR ? Q : P;
    const int log2N = a.log2N2 + ilog2c(N1);
    const int c = gt % C, t = (gt / C) % P;
    const int a0 = PAIR ? (t >> 1) + Q * Q * (t & 1) : t;
    const int n2 = n2_0 + c;
    const float4 fa = sixstep_factor(n2 * a0, log2N);
    const float2 tsA = make_float2(fa.x, fa.y);
    const int qA = __float_as_int(fa.z);
    float2* base = data + n2;
    // the columns come from `src` (a tile of C columns, rows src_ld apart,
    // staged in shared memory) when given, else from data
    const float2* lb = src ? src + c : base;
    const size_t lld = src ? (size_t)src_ld : (size_t)ld;
    float2 v[Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) v[j] = lb[(size_t)(op == COL_FWD ? t + P * j : a0 + a1 * j) * lld];
    __syncthreads();

    const ColLayout<P, C> lay{c};
    if (op != COL_FWD) {
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            const float4 fb = sB[j * sB_stride + c];
            v[j] = lift_rot_inv(lift_rot_inv(quarter_turns(v[j], -(qA + __float_as_int(fb.z)) & 3),
                                             make_float2(fb.x, fb.y)),
                                tsA);
        }
        if constexpr (PAIR)
            fft_p2q_lift_inv<Q, true>(v, sx, lay, t, s_fc, C);
        else
            fft_pq_lift_inv<P, Q, true>(v, sx, lay, t, s_fc);
    }
    if (op == COL_KERR) {
        // src/focss/solver/ssfm.cpp:160-164: A *= exp(i kappa gamma h |A|^2); the
        // peak is taken from |A|^2 before the rotation (which preserves it).
        const float coef = st->kerr_coef;
        if (modes == 1) {
#pragma unroll
            for (int j = 0; j < Q; ++j) {
                const float p = cnorm(v[j]);
                v[j] = kerr_rotate(v[j], coef * p);
                pk = fmaxf(pk, p);
            }
        } else {
            // |A_0|^2 + |A_1|^2 through the (now free) exchange buffers
            float* pw = reinterpret_cast<float*>(s_x0);
            const int stride = N1 * C;
#pragma unroll
            for (int j = 0; j < Q; ++j) pw[mo * stride + (t + P * j) * C + c] = cnorm(v[j]);
            __syncthreads();
#pragma unroll
            for (int j = 0; j < Q; ++j) {
                const int i = (t + P * j) * C + c;
                const float p = pw[i] + pw[stride + i];
                v[j] = kerr_rotate(v[j], coef * p);
                pk = fmaxf(pk, p);
            }
            __syncthreads();  // the forward transform reuses the buffers
        }
    } else if (op == COL_FWD && st) {
        if (modes == 1) {
#pragma unroll
            for (int j = 0; j < Q; ++j) {
                const float p = cnorm(v[j]);
                pk = fmaxf(pk, p);
                sm += p;
            }
        } else {
            float* pw = reinterpret_cast<float*>(s_x0);
            const int stride = N1 * C;
#pragma unroll
            for (int j = 0; j < Q; ++j) {
                const float p = cnorm(v[j]);
                pw[mo * stride + (t + P * j) * C + c] = p;
                sm += p;
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < Q; ++j) {
                const int i = (t + P * j) * C + c;
                pk = fmaxf(pk, pw[i] + pw[stride + i]);
            }
            __syncthreads();
        }
    }
    if (op == COL_FWD || op == COL_KERR) {
        if constexpr (PAIR)
            fft_p2q_lift<Q, true>(v, sx, lay, t, s_fc, C);
        else
            fft_pq_lift<P, Q, true>(v, sx, lay, t, s_fc);
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            const float4 fb = sB[j * sB_stride + c];
            v[j] = quarter_turns(lift_rot(lift_rot(v[j], tsA), make_float2(fb.x, fb.y)), qA + __float_as_int(fb.z));
        }
    }
#pragma unroll
    for (int j = 0; j < Q; ++j) base[(size_t)(op == COL_INV ? t + P * j : a0 + a1 * j) * ld] = v[j];
}

// The column-pass CTAs of realization b add their peak and energy to its
// state; the last one to finish advances the step state (ssfm_advance).
__device__ __forceinline__ void col_advance(const PassArgs& a, SsfmState* st, int b, int op, float pk, float sm,
                                            float* red) {
    block_max_sum(pk, sm, red);
    if (threadIdx.x == 0) {
        if (op != COL_INV) atomicMax(&st->peak_bits, __float_as_uint(pk));
        if (op == COL_FWD) atomicAdd(&st->sum, (double)sm);  // the energy is read at the first step only
        __threadfence();
        const unsigned prev = atomicAdd(&st->blocks_done, 1u);
        if (prev == gridDim.x - 1) {
            __threadfence();
            const float peak = __uint_as_float(atomicOr(&st->peak_bits, 0u));
            const double sum = op == COL_FWD ? atomicAdd(&st->sum, 0.0) : 0.0;
            ssfm_advance(*st, a.prm, b, op, peak, sum);
            st->peak_bits = 0u;
            st->sum = 0.0;
            st->blocks_done = 0u;
            __threadfence();
        }
    }
}

// A CTA holds the same C columns of every mode of one realization (a.modes
// groups of C*P threads; 1 or 2 modes), so the Kerr phase can use the power
// summed over modes (Field::power, src/focss/field.cpp:164-171).  The launch
// bound of 2 groups x MINB CTAs fixes the register budget at
// 65536 / (2 C P MINB) per thread (64 for N1 = 512: 2 x 2 x 256 threads),
// exactly what 2 MINB single-mode CTAs (1 group each) need to share an SM, so
// that residency cannot be lost to a register heuristic; a bound of
// (C P, 2 MINB) would express the same budget but reject the two-mode
// launches of 2 C P threads.
template <int N1, int C>
__global__ void __launch_bounds__(2 * C * ColFFT<N1>::P, ColShape<N1>::MINB) col_kernel(const PassArgs a) {
    constexpr int P = ColFFT<N1>::P, Q = ColFFT<N1>::Q;
    constexpr int a1 = ColFFT<N1>::PAIR ? Q : P;
    extern __shared__ float4 smem4[];
    float4* s_fc = smem4;                                  // column sub-FFT twiddles, (u,t) order
    float4* s_B = s_fc + N1;                               // six-step factors W_N^{n2 a1 j}, [j][c]
    float2* s_x0 = reinterpret_cast<float2*>(s_B + Q * C); // exchange buffers, N1*C per mode
    const int mo = threadIdx.x / (C * P);                  // mode of this thread group
    float2* sx = s_x0 + (size_t)mo * N1 * C;
    __shared__ float red[64];

    // The six-step factors depend on nothing in memory: computed while the
    // previous pass finishes (programmatic dependent launch).
    pdl_trigger();
    const int log2N = a.log2N2 + ilog2c(N1);
    for (int i = threadIdx.x; i < Q * C; i += blockDim.x)
        s_B[i] = sixstep_factor((blockIdx.x * C + i % C) * a1 * (i / C), log2N);
    pdl_wait();
    const int b = blockIdx.y;
    SsfmState* st = a.state ? a.state + b : nullptr;
    int op = a.op;
    if (st) {
        op = *(volatile int*)&st->action;
        if (op == COL_IDLE) return;
    }
    for (int i = threadIdx.x; i < N1; i += blockDim.x) s_fc[i] = a.tw[i];
    const int modes = a.modes > 1 ? a.modes : 1;
    float pk = 0.0f, sm = 0.0f;
    col_work<N1, C>(a, op, st, a.data + ((size_t)b * modes + mo) * a.N, blockIdx.x * C, s_fc, s_B, C, sx, s_x0, mo,
                    modes, threadIdx.x % (C * P), a.N2, pk, sm);
    if (st) col_advance(a, st, b, op, pk, sm, red);
}

// ---------------------------------------------------------------- row pass
// The work of the P threads of row k1 (`rl` the row's slot in the exchange
// buffer, t the thread in the row) of one mode; `data` points at that mode's
// first sample (global or shared memory), rows `ld` samples apart.  ROW_SSFM
// applies exp(-alpha hl/2)/N (FP32 gain g) times the dispersion phase from the
// 96-bit fraction dhi/dlo.
// a k'^2 in turns as the 96-bit fixed-point product of the step's fraction
// a (a96 = dhi 2^32 + the low 32 bits) and k'^2, carried exactly (mod 2^128)
// along an arithmetic progression k' = k0 + delta i by second differences:
// P_i = a k_i'^2, P_{i+1} = P_i + dP_i, dP_{i+1} = dP_i + 2 a delta^2.  next()
// returns bits 32..95 of P_i, which equal dhi k'^2 + umulhi(dlo 2^32, k'^2)
// mod 2^64.  |k0|, |delta| <= 2^19, so the integer factors fit in 64 bits.
struct PhaseRun {
    unsigned __int128 P, dP, C2;
    __device__ __forceinline__ PhaseRun(unsigned __int128 a, long long k0, long long delta) {
        P = a * (unsigned __int128)(unsigned long long)(k0 * k0);
        dP = a * (unsigned __int128)(__int128)(2 * delta * k0 + delta * delta);
        C2 = a * (unsigned __int128)(unsigned long long)(2 * delta * delta);
    }
    __device__ __forceinline__ unsigned long long next() {
        const unsigned long long X = (unsigned long long)(P >> 32);
        P += dP;
        dP += C2;
        return X;
    }
};

// The row work on the thread's elements v[j] = x[t + P j] of row k1, in
// registers from load to store.
template <int N2>
__device__ __forceinline__ void row_core(const PassArgs& a, int op, float2 (&v)[PQ<N2>::Q], int k1, int rl, int t,
                                         const float4* s_tw, const float4* s_T, float2* sx, float g,
                                         unsigned long long dhi, unsigned long long dlo) {
    constexpr int P = PQ<N2>::P, Q = PQ<N2>::Q;
    const RowLayout<P> lay{rl * Q * (P + 1)};
    // Lifting sub-FFTs with a mirrored inverse, as in the column pass: the
    // forward transform's constant roundings are undone exactly by the
    // inverse, so between the two they act only through their commutator
    // with the (near-identity) Kerr step of the next column pass.
    if (op != ROW_INV) fft_pq_lift<P, Q, false>(v, sx, lay, t, s_tw);
    const int N = a.N, N1 = a.N1;
    if (op == ROW_SSFM) {
        // exp(-alpha hl/2)/N * exp(i beta2/2 hl w_k^2) (ssfm.cpp:142-158), w_k = k' dw,
        // phase in turns = a k'^2 mod 1 formed exactly from the 96-bit fraction.
        // The thread's own bins go through its column of the exchange buffer
        // so that this long per-bin body is emitted once (a rolled loop), not
        // Q times: the unrolled kernel overflowed the instruction cache.
        //
        // The thread's bins k = s0 + D j (s0 = k1 + N1 t, D = N1 P) fold to
        // k' = s0 + D j for j < Q/2 and k' = N - s0 - D j above: two
        // arithmetic progressions, along which a k'^2 is carried exactly by
        // second differences (PhaseRun) instead of a 64 x 64-bit product per
        // bin -- the same bits, so the same rotation.
        float2* mine = sx + lay(0, t);
#pragma unroll
        for (int j = 0; j < Q; ++j) mine[j * (P + 1)] = v[j];
        const unsigned __int128 a96 = ((unsigned __int128)dhi << 32) | (unsigned __int128)(dlo >> 32);
        const long long s0 = (long long)k1 + (long long)N1 * t, D = (long long)N1 * P;
        {
            PhaseRun run(a96, s0, D);
#pragma unroll 1
            for (int j = 0; j < Q / 2; ++j)
                mine[j * (P + 1)] = turns_rotate(cscale(mine[j * (P + 1)], g), run.next(), s_T);
        }
        {
            PhaseRun run(a96, (long long)(N >> 1) - s0, -D);
#pragma unroll 1
            for (int j = Q / 2; j < Q; ++j)
                mine[j * (P + 1)] = turns_rotate(cscale(mine[j * (P + 1)], g), run.next(), s_T);
        }
#pragma unroll
        for (int j = 0; j < Q; ++j) v[j] = mine[j * (P + 1)];
    } else if (op == ROW_TABLE) {
        const float2* tb = a.table + (size_t)k1 * N2 + t;
#pragma unroll
        for (int j = 0; j < Q; ++j) v[j] = cscale(cmul(v[j], tb[P * j]), g);
    } else if (op == ROW_BANDPASS) {
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            const int k = k1 + N1 * (t + P * j);
            v[j] = (k >= a.bp_cut && k <= N - a.bp_cut) ? make_float2(0.f, 0.f) : cscale(v[j], g);
        }
    } else if (op != ROW_INV) {  // ROW_SCALE, ROW_FWD
#pragma unroll
        for (int j = 0; j < Q; ++j) v[j] = cscale(v[j], g);
    }
    if (op != ROW_FWD) fft_pq_lift_inv<P, Q, false>(v, sx, lay, t, s_tw);
}

template <int N2>
__device__ __forceinline__ void row_work(const PassArgs& a, int op, float2* data, int k1, int rl, int t,
                                         const float4* s_tw, const float4* s_T, float2* sx, float g,
                                         unsigned long long dhi, unsigned long long dlo, int ld) {
    constexpr int P = PQ<N2>::P, Q = PQ<N2>::Q;
    float2* base = data + (size_t)k1 * ld + t;
    float2 v[Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) v[j] = base[P * j];
    __syncthreads();
    row_core<N2>(a, op, v, k1, rl, t, s_tw, s_T, sx, g, dhi, dlo);
#pragma unroll
    for (int j = 0; j < Q; ++j) base[P * j] = v[j];
}

template <int N2, int R>
__global__ void __launch_bounds__(R* PQ<N2>::P, 2) row_kernel(const PassArgs a) {
    constexpr int P = PQ<N2>::P;
    extern __shared__ float4 smem4[];
    float4* s_tw = smem4;                                    // W_N2^e (double-float)
    float4* s_T = s_tw + N2;                                 // exp(2 pi i j/512)
    float2* sx = reinterpret_cast<float2*>(s_T + 512);       // R * Q * (P+1)

    pdl_trigger();
    pdl_wait();
    const int b = blockIdx.y;  // realization * modes + mode
    const SsfmState* st = a.state ? a.state + b / (a.modes > 1 ? a.modes : 1) : nullptr;
    unsigned long long dhi = 0ull, dlo = 0ull;
    float g = a.scale;
    if (st) {
        if (!*(volatile const int*)&st->row_active) return;
        dhi = st->disp_hi;
        dlo = st->disp_lo << 32;
        g = st->lin_gain;
    }
    for (int i = threadIdx.x; i < N2; i += blockDim.x) s_tw[i] = a.tw[a.N1 + i];
    if (st)
        for (int i = threadIdx.x; i < 512; i += blockDim.x) s_T[i] = a.tw[2 * a.N1 + 2 * N2 + i];
    const int rl = threadIdx.x / P, t = threadIdx.x % P;
    row_work<N2>(a, st ? (int)ROW_SSFM : a.op, a.data + (size_t)b * a.N, blockIdx.x * R + rl, rl, t, s_tw, s_T, sx,
                 g, dhi, dlo, N2);
}

// ---------------------------------------------------------------- row pass, bulk-copy staging
// The same row pass with its rows moved by the TMA bulk-copy engine
// (cp.async.bulk): one thread queues the CTA's R rows (N2 x 8 B each,
// contiguous in HBM) into the rows' exchange-buffer slots behind one
// mbarrier while the CTA loads its tables, the threads read their elements
// from shared memory, and each row goes back to HBM as one bulk store.  The
// wait is bounded: past kBulkWaitCap polls the CTA records a fault (a.fault)
// and skips its rows.
constexpr int kBulkWaitCap = 1 << 22;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
    for (int i = 0; i < kBulkWaitCap; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

template <int N2, int R>
__global__ void __launch_bounds__(R* PQ<N2>::P, 2) row_kernel_bulk(const PassArgs a) {
    constexpr int P = PQ<N2>::P, Q = PQ<N2>::Q;
    constexpr uint32_t kRowBytes = N2 * sizeof(float2);
    static_assert(kRowBytes % 16 == 0 && (Q * (P + 1) * sizeof(float2)) % 16 == 0, "bulk copies move 16-byte units");
    extern __shared__ float4 smem4[];
    float4* s_tw = smem4;                                    // W_N2^e (double-float)
    float4* s_T = s_tw + N2;                                 // exp(2 pi i j/512)
    float2* sx = reinterpret_cast<float2*>(s_T + 512);       // R * Q * (P+1): landing zone and exchange
    __shared__ __align__(8) unsigned long long bar;

    pdl_trigger();
    pdl_wait();
    const int b = blockIdx.y;  // realization * modes + mode
    const SsfmState* st = a.state ? a.state + b / (a.modes > 1 ? a.modes : 1) : nullptr;
    unsigned long long dhi = 0ull, dlo = 0ull;
    float g = a.scale;
    if (st) {
        if (!*(volatile const int*)&st->row_active) return;  // before any copy is queued
        dhi = st->disp_hi;
        dlo = st->disp_lo << 32;
        g = st->lin_gain;
    }
    const int k1_0 = blockIdx.x * R;
    float2* rows = a.data + (size_t)b * a.N + (size_t)k1_0 * N2;
    const uint32_t ub = smem_addr(&bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ub) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ub), "r"(R * kRowBytes)
                     : "memory");
        for (int r = 0; r < R; ++r)
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                             smem_addr(sx + (size_t)r * Q * (P + 1))),
                         "l"(rows + (size_t)r * N2), "r"(kRowBytes), "r"(ub)
                         : "memory");
    }
    for (int i = threadIdx.x; i < N2; i += blockDim.x) s_tw[i] = a.tw[a.N1 + i];
    if (st)
        for (int i = threadIdx.x; i < 512; i += blockDim.x) s_T[i] = a.tw[2 * a.N1 + 2 * N2 + i];
    __syncthreads();  // barrier initialised, tables in place
    // every thread polls; the CTA leaves together if any of them gave up
    if (__syncthreads_or(!mbar_wait_bounded(ub, 0))) {
        if (a.fault) atomicExch(a.fault, 1);
        if (threadIdx.x == 0) mbar_wait_bounded(ub, 0);  // the copies must land before the CTA exits
        return;
    }
    const int rl = threadIdx.x / P, t = threadIdx.x % P;
    float2* row_s = sx + (size_t)rl * Q * (P + 1);
    float2 v[Q];
#pragma unroll
    for (int j = 0; j < Q; ++j) v[j] = row_s[t + P * j];
    __syncwarp();  // the row's lanes (one warp holds whole rows) have read before the exchange writes
    row_core<N2>(a, st ? (int)ROW_SSFM : a.op, v, k1_0 + rl, rl, t, s_tw, s_T, sx, g, dhi, dlo);
#pragma unroll
    for (int j = 0; j < Q; ++j) row_s[t + P * j] = v[j];
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the writes, visible to the copy engine
    __syncwarp();
    if (t == 0) {
        asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(rows + (size_t)rl * N2),
                     "r"(smem_addr(row_s)), "r"(kRowBytes)
                     : "memory");
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // shared memory read before exit
    }
}

// ---------------------------------------------------------------- column pass, TMA tensor staging
// The same column pass with the CTA's tile (C columns x N1 rows of each mode,
// a strided block of the field) moved by the TMA engine as 2-D tensor boxes
// (cp.async.bulk.tensor.2d, at most 256 rows per box) into the modes'
// exchange buffers, behind one mbarrier whose wait is bounded; the threads
// read their elements from there and the results go back with ordinary
// stores.  `fmap` views the launch's fields as one row-major matrix of
// batch x modes x N1 rows of N2 8-byte elements, boxes of C x min(N1, 256).
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

template <int N1, int C>
__global__ void __launch_bounds__(2 * C * ColFFT<N1>::P, ColShape<N1>::MINB)
    col_kernel_tma(const __grid_constant__ CUtensorMap fmap, const PassArgs a) {
    constexpr int P = ColFFT<N1>::P, Q = ColFFT<N1>::Q;
    constexpr int a1 = ColFFT<N1>::PAIR ? Q : P;
    constexpr int BOX = N1 < 256 ? N1 : 256;
    extern __shared__ float4 smem4[];
    float4* s_fc = smem4;                                  // column sub-FFT twiddles, (u,t) order
    float4* s_B = s_fc + N1;                               // six-step factors W_N^{n2 a1 j}, [j][c]
    // exchange buffers (the TMA landing tiles), N1*C per mode, from a
    // 128-byte boundary (the launch adds 128 bytes for it)
    const uint32_t xb = smem_addr(s_B + Q * C), xpad = (128u - (xb & 127u)) & 127u;
    float2* s_x0 = reinterpret_cast<float2*>(reinterpret_cast<char*>(s_B + Q * C) + xpad);
    const int mo = threadIdx.x / (C * P);
    float2* sx = s_x0 + (size_t)mo * N1 * C;
    __shared__ float red[64];
    __shared__ __align__(8) unsigned long long bar;

    pdl_trigger();
    const int log2N = a.log2N2 + ilog2c(N1);
    for (int i = threadIdx.x; i < Q * C; i += blockDim.x)
        s_B[i] = sixstep_factor((blockIdx.x * C + i % C) * a1 * (i / C), log2N);
    pdl_wait();
    const int b = blockIdx.y;
    SsfmState* st = a.state ? a.state + b : nullptr;
    int op = a.op;
    if (st) {
        op = *(volatile int*)&st->action;
        if (op == COL_IDLE) return;  // before any copy is queued
    }
    const int modes = a.modes > 1 ? a.modes : 1;
    const uint32_t ub = smem_addr(&bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ub) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ub),
                     "r"((uint32_t)(modes * N1 * C * sizeof(float2)))
                     : "memory");
        for (int m = 0; m < modes; ++m)
            for (int h = 0; h < N1 / BOX; ++h)
                tma_load_2d(smem_addr(s_x0 + (size_t)m * N1 * C + (size_t)h * BOX * C), &fmap, blockIdx.x * C,
                            (b * modes + m) * N1 + h * BOX, ub);
    }
    for (int i = threadIdx.x; i < N1; i += blockDim.x) s_fc[i] = a.tw[i];
    __syncthreads();  // barrier initialised, tables in place
    if (__syncthreads_or(!mbar_wait_bounded(ub, 0))) {
        if (a.fault) atomicExch(a.fault, 1);
        if (threadIdx.x == 0) mbar_wait_bounded(ub, 0);  // the copies must land before the CTA exits
        return;
    }
    float pk = 0.0f, sm = 0.0f;
    col_work<N1, C>(a, op, st, a.data + ((size_t)b * modes + mo) * a.N, blockIdx.x * C, s_fc, s_B, C, sx, s_x0, mo,
                    modes, threadIdx.x % (C * P), a.N2, pk, sm, sx, C);
    if (st) col_advance(a, st, b, op, pk, sm, red);
}

// ---------------------------------------------------------------- single CTA
// For N = N1 N2 <= 2^14 one CTA of kBlockThreads runs a realization's whole
// split-step loop with the field resident in shared memory: the column and
// row work of the two-pass kernels (the same arithmetic, so the same
// results), over all columns and then all rows of the field, with thread 0
// advancing the step state between the phases.  HBM is read once and written
// once per SSFM run instead of twice per step, and a run is one launch.
constexpr int kBlockThreads = 256;

template <int N1, int N2>
struct BlockShape {
    // rows of the resident field are LD = N2 + 8 samples apart: the row
    // phase's warps read 4 rows x 64 bytes, which then fall on both halves of
    // the banks (two wavefronts instead of four)
    static constexpr int LD = N2 + 8;
    static constexpr int C = 16;
    static constexpr int G = kBlockThreads / (C * ColFFT<N1>::P);  // column groups
    static constexpr int RPI = kBlockThreads / PQ<N2>::P;          // rows per row phase step
    static constexpr size_t XCH = (size_t)G * N1 * C > (size_t)RPI * PQ<N2>::Q * (PQ<N2>::P + 1)
                                      ? (size_t)G * N1 * C
                                      : (size_t)RPI * PQ<N2>::Q * (PQ<N2>::P + 1);
    static constexpr size_t SMEM = sizeof(float4) * ((size_t)N1 + (size_t)ColFFT<N1>::Q * N2 + N2 + 512) +
                                   sizeof(float2) * ((size_t)N1 * LD + XCH);
    static_assert(G >= 1 && N2 % (G * C) == 0 && N1 % RPI == 0, "single-CTA split");
};

template <int N1, int N2>
__global__ void __launch_bounds__(kBlockThreads, BlockShape<N1, N2>::SMEM <= 113 * 1024 ? 2 : 1)
    block_kernel(const PassArgs a, int cap) {
    using S = BlockShape<N1, N2>;
    constexpr int C = S::C, G = S::G, RPI = S::RPI;
    constexpr int Pc = ColFFT<N1>::P, Qc = ColFFT<N1>::Q, Pr = PQ<N2>::P;
    constexpr int a1 = ColFFT<N1>::PAIR ? Qc : Pc;
    constexpr int N = N1 * N2, LD = S::LD;
    extern __shared__ float4 smem4[];
    float4* s_fc = smem4;                                 // column sub-FFT twiddles
    float4* s_B = s_fc + N1;                              // six-step factors, [j][n2]
    float4* s_tw = s_B + Qc * N2;                         // row sub-FFT twiddles
    float4* s_T = s_tw + N2;                              // exp(2 pi i j/512)
    float2* s_f = reinterpret_cast<float2*>(s_T + 512);   // the field, N1 rows of LD
    float2* s_x = s_f + (size_t)N1 * LD;                  // exchange buffers
    __shared__ float red[64];

    SsfmState* st = a.state + blockIdx.x;
    const int log2N = a.log2N2 + ilog2c(N1);
    for (int i = threadIdx.x; i < N1; i += kBlockThreads) s_fc[i] = a.tw[i];
    for (int i = threadIdx.x; i < N2; i += kBlockThreads) s_tw[i] = a.tw[N1 + i];
    for (int i = threadIdx.x; i < 512; i += kBlockThreads) s_T[i] = a.tw[2 * N1 + 2 * N2 + i];
    for (int i = threadIdx.x; i < Qc * N2; i += kBlockThreads)
        s_B[i] = sixstep_factor((i % N2) * a1 * (i / N2), log2N);
    float4* g4 = reinterpret_cast<float4*>(a.data + (size_t)blockIdx.x * N);
    float4* f4 = reinterpret_cast<float4*>(s_f);
    for (int i = threadIdx.x; i < N / 2; i += kBlockThreads) f4[(i / (N2 / 2)) * (LD / 2) + i % (N2 / 2)] = g4[i];
    __syncthreads();

    const int grp = threadIdx.x / (C * Pc), gt = threadIdx.x % (C * Pc);
    const int rl = threadIdx.x / Pr, t = threadIdx.x % Pr;
    for (int it = 0; it < cap; ++it) {
        const int op = *(volatile const int*)&st->action;
        if (op == COL_IDLE) break;
        float pk = 0.0f, sm = 0.0f;
        for (int cb = 0; cb < N2 / (G * C); ++cb) {
            const int n2_0 = (cb * G + grp) * C;
            col_work<N1, C>(a, op, st, s_f, n2_0, s_fc, s_B + n2_0, N2, s_x + (size_t)grp * N1 * C, s_x, grp, 1, gt,
                            LD, pk, sm);
            __syncthreads();
        }
        block_max_sum(pk, sm, red);
        if (threadIdx.x == 0) ssfm_advance(*st, a.prm, blockIdx.x, op, pk, (double)sm);
        __syncthreads();
        if (*(volatile const int*)&st->row_active) {
            const float g = *(volatile const float*)&st->lin_gain;
            const unsigned long long dhi = *(volatile const unsigned long long*)&st->disp_hi;
            const unsigned long long dlo = *(volatile const unsigned long long*)&st->disp_lo << 32;
            for (int rb = 0; rb < N1 / RPI; ++rb) {
                row_work<N2>(a, ROW_SSFM, s_f, rb * RPI + rl, rl, t, s_tw, s_T, s_x, g, dhi, dlo, LD);
                __syncthreads();
            }
        }
    }
    for (int i = threadIdx.x; i < N / 2; i += kBlockThreads) g4[i] = f4[(i / (N2 / 2)) * (LD / 2) + i % (N2 / 2)];
}

typedef void (*PassFn)(PassArgs);
typedef void (*ColTmaFn)(CUtensorMap, PassArgs);
struct Launch {
    PassFn fn = nullptr;
    PassFn fn_bulk = nullptr;  // row pass with bulk-copy staging
    PassFn fn_narrow = nullptr;  // the pass in 64-thread CTAs (few blocks in the whole launch)
    ColTmaFn fn_tma = nullptr;   // column pass with TMA tensor staging
    int per_block_narrow = 0;
    int threads = 0, per_block = 0;
    size_t smem = 0;
    bool attr_set = false;
};

// Row-pass rows per block: must divide N1 (N1 >= max(16, N2/2) for every plan).
template <int N2>
struct RowShape {
    static constexpr int P = PQ<N2>::P;
    static constexpr int R0 = 256 / P;
    static constexpr int RH = (N2 / 2 > 16 ? N2 / 2 : 16);
    static constexpr int R = R0 < RH ? R0 : RH;
    // 64-thread CTAs: when a launch has fewer row blocks than the GPU has SMs
    // (a single field of 2^17 samples at a 128 x 1024 split has 16), four
    // times as many SMs take part.
    static constexpr int RN = 64 / P;
};

Launch col_launch_for(int log2N1);
Launch row_launch_for(int log2N2);

}  // namespace fg

#define FG_INSTANTIATE_COL(L, LG)                                              \
    namespace fg {                                                             \
    Launch col_launch_##LG() {                                                 \
        Launch l;                                                              \
        l.fn = col_kernel<L, ColShape<L>::C>;                                  \
        l.fn_narrow = col_kernel<L, ColShape<L>::CN>;                          \
        l.fn_tma = col_kernel_tma<L, ColShape<L>::C>;                          \
        l.per_block_narrow = ColShape<L>::CN;                                  \
        l.threads = ColShape<L>::C * ColFFT<L>::P;                             \
        l.per_block = ColShape<L>::C;                                          \
        return l;                                                              \
    }                                                                          \
    }
#define FG_INSTANTIATE_ROW(L, LG)                                              \
    namespace fg {                                                             \
    Launch row_launch_##LG() {                                                 \
        Launch l;                                                              \
        l.fn = row_kernel<L, RowShape<L>::R>;                                  \
        l.fn_bulk = row_kernel_bulk<L, RowShape<L>::R>;                        \
        l.fn_narrow = row_kernel<L, RowShape<L>::RN>;                          \
        l.per_block_narrow = RowShape<L>::RN;                                  \
        l.threads = RowShape<L>::R * PQ<L>::P;                                 \
        l.per_block = RowShape<L>::R;                                          \
        return l;                                                              \
    }                                                                          \
    }
