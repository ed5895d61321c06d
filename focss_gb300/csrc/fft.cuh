// fft.cuh -- FFT building blocks for the SSFM kernels.
//
// Layout convention used throughout: a length-L sub-FFT (L = P*Q, Q a multiple
// of P) is computed by a group of P threads; thread t holds the Q elements
// x[t + P*j], j = 0..Q-1, in registers.  fft_pq() returns the transform in the
// same layout (v[j] = X[t + P*j]), so a forward transform, a pointwise
// operator and an inverse transform chain without any extra data movement.
// One exchange through shared memory per transform:
//   1. Q-point DFT in registers over j          (radix-2 DIF, constant twiddles)
//   2. twiddle W_L^{t*u}                        (table in shared memory)
//   3. write (u, t), read (u = t + P*i, s)      (caller-chosen conflict-free layout)
//   4. P-point DFT in registers over s.
// Sign convention: forward = exp(-2 pi i nk/L), unnormalized (FFTW_FORWARD).
//
// Precision.  The split-step loop applies the same transforms thousands of
// times, so a rounding error that depends only on a constant (a twiddle
// factor) repeats identically every step and grows linearly with the step
// count, while roundings that depend on the data decorrelate and grow like
// sqrt(steps).  Every twiddle is therefore held as an unevaluated sum
// hi + lo of two floats (about 48 significant bits) and applied with a
// compensated product: the only roundings left are data-dependent.
#pragma once

#include "common.cuh"

namespace fg {

// (hi, lo) with hi + lo = cos(pi*j/32) to ~2^-48, j = 0..16
__host__ __device__ __forceinline__ constexpr float2 cos_pi32_df(int j) {
    constexpr float2 t[17] = {
        {1.0f, 0.0f},
        {0.9951847195625305f, 7.109666189109021e-09f},
        {0.9807852506637573f, 2.9739473106360492e-08f},
        {0.9569403529167175f, -1.7184508038781132e-08f},
        {0.9238795042037964f, 2.830748968563057e-08f},
        {0.8819212913513184f, -2.7002963420841297e-08f},
        {0.8314695954322815f, 1.687026340846387e-08f},
        {0.7730104327201843f, 2.0642552556182636e-08f},
        {0.7071067690849304f, 1.2101617485882343e-08f},
        {0.6343932747840881f, 9.37955757507325e-09f},
        {0.5555702447891235f, -1.1769521357507529e-08f},
        {0.4713967442512512f, -7.425253745196869e-09f},
        {0.3826834261417389f, 6.2233507236442165e-09f},
        {0.290284663438797f, 1.3815665056426951e-08f},
        {0.19509032368659973f, -1.670471427850373e-09f},
        {0.0980171412229538f, -8.933931927579408e-10f},
        {0.0f, 0.0f}};
    return t[j];
}

// (cos, sin) of pi*idx/32 for idx in [0, 64) as double-float: {c_hi, c_lo, s_hi, s_lo}
__host__ __device__ __forceinline__ constexpr float4 cs64_df(int idx) {
    return idx <= 16   ? float4{cos_pi32_df(idx).x, cos_pi32_df(idx).y, cos_pi32_df(16 - idx).x,
                              cos_pi32_df(16 - idx).y}
           : idx <= 32 ? float4{-cos_pi32_df(32 - idx).x, -cos_pi32_df(32 - idx).y, cos_pi32_df(idx - 16).x,
                                cos_pi32_df(idx - 16).y}
           : idx <= 48 ? float4{-cos_pi32_df(idx - 32).x, -cos_pi32_df(idx - 32).y, -cos_pi32_df(48 - idx).x,
                                -cos_pi32_df(48 - idx).y}
                       : float4{cos_pi32_df(64 - idx).x, cos_pi32_df(64 - idx).y, -cos_pi32_df(idx - 48).x,
                                -cos_pi32_df(idx - 48).y};
}

// a * (w_hi + w_lo) with w = {re_hi, im_hi, re_lo, im_lo}: compensated complex
// product; the representation error of w drops out, data roundings remain.
__device__ __forceinline__ float2 cmul_df(float2 a, float4 w) {
    const float re = fmaf(a.x, w.x, fmaf(-a.y, w.y, fmaf(a.x, w.z, -a.y * w.w)));
    const float im = fmaf(a.x, w.y, fmaf(a.y, w.x, fmaf(a.x, w.w, a.y * w.z)));
    return make_float2(re, im);
}
// a * conj(w_hi + w_lo)
__device__ __forceinline__ float2 cmulc_df(float2 a, float4 w) {
    const float re = fmaf(a.x, w.x, fmaf(a.y, w.y, fmaf(a.x, w.z, a.y * w.w)));
    const float im = fmaf(a.y, w.x, fmaf(-a.x, w.y, fmaf(a.y, w.z, -a.x * w.w)));
    return make_float2(re, im);
}

// a * exp(-+ i*pi*idx/32): forward uses the minus sign.
template <bool INV>
__device__ __forceinline__ float2 twmul64(float2 a, int idx) {
    idx &= 63;
    if (idx == 0) return a;
    if (idx == 32) return make_float2(-a.x, -a.y);
    if (idx == 16) return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
    if (idx == 48) return INV ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
    const float4 w = cs64_df(idx);  // (c_hi, c_lo, s_hi, s_lo)
    // forward multiplies by (c - i s), inverse by (c + i s)
    return INV ? cmul_df(a, make_float4(w.x, w.z, w.y, w.w)) : cmul_df(a, make_float4(w.x, -w.z, w.y, -w.w));
}

__host__ __device__ __forceinline__ constexpr int bitrev(int i, int bits) {
    int r = 0;
    for (int b = 0; b < bits; ++b) r |= ((i >> b) & 1) << (bits - 1 - b);
    return r;
}

__host__ __device__ __forceinline__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n >> 1); }

// In-register DFT of size R (power of two <= 64), natural order in and out.
template <int R, bool INV>
__device__ __forceinline__ void dft(float2 (&v)[R]) {
#pragma unroll
    for (int half = R / 2; half >= 1; half >>= 1) {
#pragma unroll
        for (int base = 0; base < R; base += 2 * half) {
#pragma unroll
            for (int j = 0; j < half; ++j) {
                const float2 a = v[base + j], b = v[base + j + half];
                v[base + j] = cadd(a, b);
                v[base + j + half] = twmul64<INV>(csub(a, b), j * (32 / half));
            }
        }
    }
    constexpr int bits = ilog2c(R);
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int r = bitrev(i, bits);
        if (i < r) {
            const float2 tmp = v[i];
            v[i] = v[r];
            v[r] = tmp;
        }
    }
}

// Thread-group shape for a sub-FFT of length L.
template <int L>
struct PQ;
template <> struct PQ<16> { static constexpr int P = 4, Q = 4; };
template <> struct PQ<32> { static constexpr int P = 4, Q = 8; };
template <> struct PQ<64> { static constexpr int P = 8, Q = 8; };
template <> struct PQ<128> { static constexpr int P = 8, Q = 16; };
template <> struct PQ<256> { static constexpr int P = 16, Q = 16; };
template <> struct PQ<512> { static constexpr int P = 16, Q = 32; };
template <> struct PQ<1024> { static constexpr int P = 32, Q = 32; };

// Shared-memory layouts for the exchange (element (u, s), u < Q, s < P).
// Row kernels: one group per row, padded rows of P+1 (conflict-free reads).
template <int P>
struct RowLayout {
    int base;
    __device__ __forceinline__ int operator()(int u, int s) const { return base + u * (P + 1) + s; }
};
// Column kernels: C columns interleaved, column index fastest.
template <int P, int C>
struct ColLayout {
    int c;
    __device__ __forceinline__ int operator()(int u, int s) const { return (u * P + s) * C + c; }
};

// XOR swizzle of a table index inside groups of 8 entries (16-byte entries:
// 8 per 128-byte shared-memory wavefront), so strided reads spread over banks.
__host__ __device__ __forceinline__ int swz8(int e) { return e ^ (((e >> 3) ^ (e >> 6)) & 7); }
// The same for 8-byte entries (16 per wavefront).
__host__ __device__ __forceinline__ int swz16(int e) { return e ^ ((e >> 4) & 15); }

// ---------------------------------------------------------------------------
// Rotations by lifting (three shears, A. W. Paeth, "A fast algorithm for
// general raster rotation", Graphics Interface 1986): with ts = {tan(theta/2),
// sin(theta)} in FP32,
//     x -= t y;  y += s x;  x -= t y
// rotates (x, y) by theta in three FMAs, and the same shears undone in reverse
// order invert it exactly up to the data's own roundings, whatever the
// rounding of t and s.  A forward transform whose inverse is its exact mirror
// therefore adds no error that repeats identically from step to step (the
// rounding of a plain FP32 twiddle does), which is what the column pass needs:
// it applies the inverse transform, a Kerr phase close to identity and the
// forward transform.  |theta| <= pi/2 keeps |t| <= 1.
__device__ __forceinline__ float2 lift_rot(float2 v, float2 ts) {
    float x = fmaf(-ts.x, v.y, v.x);
    const float y = fmaf(ts.y, x, v.y);
    x = fmaf(-ts.x, y, x);
    return make_float2(x, y);
}
__device__ __forceinline__ float2 lift_rot_inv(float2 v, float2 ts) {
    float x = fmaf(ts.x, v.y, v.x);
    const float y = fmaf(-ts.y, x, v.y);
    x = fmaf(ts.x, y, x);
    return make_float2(x, y);
}
// W_N^e = exp(-2 pi i e/N) = (-i)^q rot(theta), q = round(4e/N), |theta| <= pi/4,
// for 0 <= e < N = 2^log2N: {tan(theta/2), sin(theta), q (int bits), 0}.  The
// residual turn fraction is exact, so the pair is a deterministic function of
// (e, N): a rotation applied in one launch is undone exactly in another.
__device__ __forceinline__ float4 sixstep_factor(int e, int log2N) {
    const int q = ((e << 2) + (1 << (log2N - 1))) >> log2N;
    const float r = (float)(e - (q << (log2N - 2))) * __int_as_float((127 - log2N) << 23);
    float sp, cp;
    sincospif(r, &sp, &cp);  // sin, cos of pi*r;  theta = -2 pi r
    return make_float4(-sp / cp, -2.0f * sp * cp, __int_as_float(q & 3), 0.0f);
}

// v * (-i)^q (exact).
__device__ __forceinline__ float2 quarter_turns(float2 v, int q) {
    const float2 r = (q & 1) ? make_float2(v.y, -v.x) : v;
    return (q & 2) ? make_float2(-r.x, -r.y) : r;
}

// Group-wide sub-FFT (see file comment).  twPQ[u*P + t] = exp(-2 pi i t u / L)
// as double-float {re_hi, im_hi, re_lo, im_lo}: the P threads of a group read
// P consecutive entries (conflict-free).
// BLOCK_SYNC selects __syncthreads (group spans warps) or __syncwarp.
template <int P, int Q, bool INV, bool BLOCK_SYNC, class Lay>
__device__ __forceinline__ void fft_pq(float2 (&v)[Q], float2* __restrict__ sm, const Lay lay, int t,
                                       const float4* __restrict__ twPQ) {
    static_assert(Q % P == 0, "Q must be a multiple of P");
    constexpr int M = Q / P;
    dft<Q, INV>(v);
#pragma unroll
    for (int u = 1; u < Q; ++u)
        v[u] = INV ? cmulc_df(v[u], twPQ[u * P + t]) : cmul_df(v[u], twPQ[u * P + t]);
#pragma unroll
    for (int u = 0; u < Q; ++u) sm[lay(u, t)] = v[u];
    if (BLOCK_SYNC) __syncthreads(); else __syncwarp();
#pragma unroll
    for (int i = 0; i < M; ++i) {
        float2 w[P];
        const int u = t + P * i;
#pragma unroll
        for (int s = 0; s < P; ++s) w[s] = sm[lay(u, s)];
        dft<P, INV>(w);
#pragma unroll
        for (int s = 0; s < P; ++s) v[i + M * s] = w[s];
    }
    if (BLOCK_SYNC) __syncthreads(); else __syncwarp();
}

// ---------------------------------------------------------------------------
// Mirrored sub-FFTs for the column pass: in-register DFT twiddles as lifting
// rotations (quarter turns exact, residual |angle| <= pi/4 in three FMAs), and
// an inverse that undoes the forward operation by operation in reverse order
// (see lift_rot).  The inter-stage table twiddles stay double-float.

// {tan(theta/2), sin(theta)} for theta = -pi*r/32, r = 0..8 (forward sign).
__host__ __device__ __forceinline__ constexpr float2 lift_pi32(int r) {
    constexpr float2 t[9] = {{0.0f, 0.0f},
                             {-0.049126848578453064f, -0.0980171412229538f},
                             {-0.09849140048027039f, -0.19509032368659973f},
                             {-0.1483359932899475f, -0.290284663438797f},
                             {-0.1989123672246933f, -0.3826834261417389f},
                             {-0.25048696994781494f, -0.4713967442512512f},
                             {-0.3033466935157776f, -0.5555702447891235f},
                             {-0.3578057289123535f, -0.6343932747840881f},
                             {-0.4142135679721832f, -0.7071067690849304f}};
    return r >= 0 ? t[r] : float2{-t[-r].x, -t[-r].y};
}

// a * exp(-i pi idx/32) = (-i)^q * rot(-pi r/32), idx = 16 q + r, |r| <= 8.
__device__ __forceinline__ float2 twlift(float2 a, int idx) {
    idx &= 63;
    const int q = (idx + 8) >> 4, r = idx - 16 * q;
    if (r != 0) a = lift_rot(a, lift_pi32(r));
    return quarter_turns(a, q & 3);
}
// Exact inverse of twlift.
__device__ __forceinline__ float2 twlift_inv(float2 a, int idx) {
    idx &= 63;
    const int q = (idx + 8) >> 4, r = idx - 16 * q;
    a = quarter_turns(a, -q & 3);
    return r != 0 ? lift_rot_inv(a, lift_pi32(r)) : a;
}

template <int R>
__device__ __forceinline__ void bitrev_swap(float2 (&v)[R]) {
    constexpr int bits = ilog2c(R);
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int r = bitrev(i, bits);
        if (i < r) {
            const float2 tmp = v[i];
            v[i] = v[r];
            v[r] = tmp;
        }
    }
}

// Forward in-register DFT (radix-2 DIF, natural order in and out).
template <int R>
__device__ __forceinline__ void dft_lift(float2 (&v)[R]) {
#pragma unroll
    for (int half = R / 2; half >= 1; half >>= 1) {
#pragma unroll
        for (int base = 0; base < R; base += 2 * half) {
#pragma unroll
            for (int j = 0; j < half; ++j) {
                const float2 a = v[base + j], b = v[base + j + half];
                v[base + j] = cadd(a, b);
                v[base + j + half] = twlift(csub(a, b), j * (32 / half));
            }
        }
    }
    bitrev_swap<R>(v);
}
// Its mirror: R times the inverse DFT.
template <int R>
__device__ __forceinline__ void dft_lift_inv(float2 (&v)[R]) {
    bitrev_swap<R>(v);
#pragma unroll
    for (int half = 1; half < R; half <<= 1) {
#pragma unroll
        for (int base = 0; base < R; base += 2 * half) {
#pragma unroll
            for (int j = 0; j < half; ++j) {
                const float2 s = v[base + j], d = twlift_inv(v[base + j + half], j * (32 / half));
                v[base + j] = cadd(s, d);
                v[base + j + half] = csub(s, d);
            }
        }
    }
}

// fft_pq with the mirrored pieces (same layouts; forward and L times inverse).
template <int P, int Q, bool BLOCK_SYNC, class Lay>
__device__ __forceinline__ void fft_pq_lift(float2 (&v)[Q], float2* __restrict__ sm, const Lay lay, int t,
                                            const float4* __restrict__ twPQ) {
    static_assert(Q % P == 0, "Q must be a multiple of P");
    constexpr int M = Q / P;
    dft_lift<Q>(v);
#pragma unroll
    for (int u = 1; u < Q; ++u) v[u] = cmul_df(v[u], twPQ[u * P + t]);
#pragma unroll
    for (int u = 0; u < Q; ++u) sm[lay(u, t)] = v[u];
    if (BLOCK_SYNC) __syncthreads(); else __syncwarp();
#pragma unroll
    for (int i = 0; i < M; ++i) {
        float2 w[P];
        const int u = t + P * i;
#pragma unroll
        for (int s = 0; s < P; ++s) w[s] = sm[lay(u, s)];
        dft_lift<P>(w);
#pragma unroll
        for (int s = 0; s < P; ++s) v[i + M * s] = w[s];
    }
    if (BLOCK_SYNC) __syncthreads(); else __syncwarp();
}
template <int P, int Q, bool BLOCK_SYNC, class Lay>
__device__ __forceinline__ void fft_pq_lift_inv(float2 (&v)[Q], float2* __restrict__ sm, const Lay lay, int t,
                                                const float4* __restrict__ twPQ) {
    static_assert(Q % P == 0, "Q must be a multiple of P");
    constexpr int M = Q / P;
#pragma unroll
    for (int i = 0; i < M; ++i) {
        float2 w[P];
#pragma unroll
        for (int s = 0; s < P; ++s) w[s] = v[i + M * s];
        dft_lift_inv<P>(w);
        const int u = t + P * i;
#pragma unroll
        for (int s = 0; s < P; ++s) sm[lay(u, s)] = w[s];
    }
    if (BLOCK_SYNC) __syncthreads(); else __syncwarp();
#pragma unroll
    for (int u = 0; u < Q; ++u) v[u] = sm[lay(u, t)];
    if (BLOCK_SYNC) __syncthreads(); else __syncwarp();
#pragma unroll
    for (int u = 1; u < Q; ++u) v[u] = cmulc_df(v[u], twPQ[u * P + t]);
    dft_lift_inv<Q>(v);
}

// ---------------------------------------------------------------------------
// Column sub-FFT with half the registers: L = 2 Q^2 on P = 2Q threads of Q
// elements (L = 32, 128, 512).  Thread t holds x[t + P j]; after an in-register
// Q-point DFT over j, the twiddle W_L^{t u} and one exchange, lane pair
// (u = t >> 1, h = t & 1) holds the even (h = 0) or odd (h = 1) half of the
// P-point DFT over t for row u, transforms it in registers and finishes with
// one radix-2 butterfly across the pair (__shfl_xor, the partner lane differs
// by `pair_xor`).  Output: thread t holds X[k1], k1 = (t>>1) + Q k + Q^2 (t&1).
// The inverse mirrors the forward operation by operation (lifting rotations).
template <int Q, bool BLOCK_SYNC, class Lay>
__device__ __forceinline__ void fft_p2q_lift(float2 (&v)[Q], float2* __restrict__ sm, const Lay lay, int t,
                                             const float4* __restrict__ twPQ, int pair_xor) {
    constexpr int P = 2 * Q;
    dft_lift<Q>(v);
#pragma unroll
    for (int u = 1; u < Q; ++u) v[u] = cmul_df(v[u], twPQ[u * P + t]);
#pragma unroll
    for (int u = 0; u < Q; ++u) sm[lay(u, t)] = v[u];
    if (BLOCK_SYNC) __syncthreads(); else __syncwarp();
    const int u = t >> 1, h = t & 1;
#pragma unroll
    for (int s = 0; s < Q; ++s) v[s] = sm[lay(u, h + 2 * s)];
    if (BLOCK_SYNC) __syncthreads(); else __syncwarp();
    dft_lift<Q>(v);
    const float sg = h ? -1.0f : 1.0f;
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        // h = 0: Z = Y0 + W Y1;  h = 1: Z = Y0 - W Y1, W = W_P^k
        const float2 tw = twlift(v[k], k * (32 / Q));
        const float2 mine = h ? tw : v[k];
        const float ox = __shfl_xor_sync(0xffffffffu, mine.x, pair_xor);
        const float oy = __shfl_xor_sync(0xffffffffu, mine.y, pair_xor);
        v[k] = make_float2(fmaf(sg, mine.x, ox), fmaf(sg, mine.y, oy));
    }
}
template <int Q, bool BLOCK_SYNC, class Lay>
__device__ __forceinline__ void fft_p2q_lift_inv(float2 (&v)[Q], float2* __restrict__ sm, const Lay lay, int t,
                                                 const float4* __restrict__ twPQ, int pair_xor) {
    constexpr int P = 2 * Q;
    const int u = t >> 1, h = t & 1;
    const float sg = h ? -1.0f : 1.0f;
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        // h = 0: 2 Y0 = Z0 + Z1;  h = 1: 2 Y1 = W^-1 (Z0 - Z1)
        const float ox = __shfl_xor_sync(0xffffffffu, v[k].x, pair_xor);
        const float oy = __shfl_xor_sync(0xffffffffu, v[k].y, pair_xor);
        const float2 sd = make_float2(fmaf(sg, v[k].x, ox), fmaf(sg, v[k].y, oy));
        const float2 tw = twlift_inv(sd, k * (32 / Q));
        v[k] = h ? tw : sd;
    }
    dft_lift_inv<Q>(v);
#pragma unroll
    for (int s = 0; s < Q; ++s) sm[lay(u, h + 2 * s)] = v[s];
    if (BLOCK_SYNC) __syncthreads(); else __syncwarp();
#pragma unroll
    for (int w = 0; w < Q; ++w) v[w] = sm[lay(w, t)];
    if (BLOCK_SYNC) __syncthreads(); else __syncwarp();
#pragma unroll
    for (int w = 1; w < Q; ++w) v[w] = cmulc_df(v[w], twPQ[w * P + t]);
    dft_lift_inv<Q>(v);
}

// Column-pass sub-FFT shape: lane-pair form (P = 2Q) where L = 2 Q^2, else PQ.
template <int L>
struct ColFFT {
    static constexpr bool PAIR = (L == 32 || L == 128 || L == 512);
    static constexpr int Q = PAIR ? (L == 32 ? 4 : L == 128 ? 8 : 16) : PQ<L>::Q;
    static constexpr int P = L / Q;
};
// Threads per group of the column pass for length L (host side of ColFFT).
__host__ __device__ __forceinline__ int col_group_p(int L) {
    return L == 32 ? 8 : L == 128 ? 16 : L == 512 ? 32 : (L <= 32 ? 4 : L <= 128 ? 8 : L <= 512 ? 16 : 32);
}

// ---------------------------------------------------------------------------
// exp(2 pi i x) for a 64-bit fixed-point turn fraction x = X / 2^64, returned
// as a double-float rotation {re_hi, im_hi, re_lo, im_lo} accurate to ~1e-12.
// x = j/512 + r with |r| <= 1/1024: T[j] = exp(2 pi i j/512) from a
// double-float table, exp(i theta) (theta = 2 pi r, |theta| <= pi/512) from
// its Taylor series, combined with error-free products and sums
// (Dekker / Knuth two-product and two-sum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bv = s - a;
    e = (a - (s - bv)) + (b - bv);
}

// Exact float of a 23-bit unsigned integer (exponent trick, no conversion unit).
__device__ __forceinline__ float u23_to_float(unsigned u) { return __int_as_float(0x4B000000u | u) - 8388608.0f; }

__device__ __forceinline__ float4 turns_rotation_df(unsigned long long X, const float4* __restrict__ T512) {
    // Y = X + 2^54: j = Y >> 55 is the nearest multiple of 1/512 turn, and the
    // remainder r = X - j 2^55 in [-2^54, 2^54) is (Y mod 2^55) - 2^54.
    const unsigned long long Y = X + (1ull << 54);
    const unsigned yh = (unsigned)(Y >> 32);
    const int j = (int)((yh >> 23) & 511u);
    // r + 2^54 = A 2^32 + B 2^9 + (9 dropped bits, < 2e-16 rad), A, B < 2^23.
    const unsigned A = yh & 0x7FFFFFu;
    const unsigned B = (unsigned)(Y >> 9) & 0x7FFFFFu;
    const float fA = u23_to_float(A) - 4194304.0f;  // exact, in [-2^22, 2^22)
    const float fB = u23_to_float(B);
    // theta = 2 pi r / 2^64 = fA * 2pi/2^32 + fB * 2pi/2^55, as th + tl
    const float c32_hi = 1.462918119976564e-09f, c32_lo = -4.070940267922164e-17f;
    const float c9 = 1.7439342975337076e-16f;
    const float th = fA * c32_hi;
    const float tl = fmaf(fA, c32_hi, -th) + fmaf(fA, c32_lo, fB * c9);
    const float th2 = th * th;
    // sin(theta) = th + (tl - th^3/6),  cos(theta) - 1 = -th^2/2 - th*tl + th^4/24
    const float s_hi = th;
    const float s_lo = fmaf(-th2 * th, 1.0f / 6.0f, tl);
    const float cm1 = fmaf(th2 * th2, 1.0f / 24.0f, fmaf(-0.5f, th2, -th * tl));
    const float4 t = T512[j];  // {c_hi, s_hi, c_lo, s_lo}
    // re = Tc (1 + cm1) - Ts s ;  im = Ts (1 + cm1) + Tc s
    const float p = t.y * s_hi, pe = fmaf(t.y, s_hi, -p);
    const float q = t.x * s_hi, qe = fmaf(t.x, s_hi, -q);
    float re_hi, re_e, im_hi, im_e;
    two_sum(t.x, -p, re_hi, re_e);
    two_sum(t.y, q, im_hi, im_e);
    const float re_lo = re_e + t.z + fmaf(t.x, cm1, -pe) - fmaf(t.y, s_lo, t.w * s_hi);
    const float im_lo = im_e + t.w + fmaf(t.y, cm1, qe) + fmaf(t.x, s_lo, t.z * s_hi);
    return make_float4(re_hi, im_hi, re_lo, im_lo);
}

// v * exp(2 pi i x), x = X / 2^64 as in turns_rotation_df, applied to the data
// in two steps: w = v * T[j] (double-float table entry, compensated product),
// then w + w * (cos(theta) - 1 + i sin(theta)) for the residual |theta| <=
// pi/512, whose angle is carried as the exact split th + tl.  Every constant
// stays at ~48 bits; the intermediate w adds one data rounding.
__device__ __forceinline__ float2 turns_rotate(float2 v, unsigned long long X, const float4* __restrict__ T512) {
    const unsigned long long Y = X + (1ull << 54);
    const unsigned yh = (unsigned)(Y >> 32);
    const int j = (int)((yh >> 23) & 511u);
    const unsigned A = yh & 0x7FFFFFu;
    const unsigned B = (unsigned)(Y >> 9) & 0x7FFFFFu;
    const float fA = u23_to_float(A) - 4194304.0f;
    const float fB = u23_to_float(B);
    const float c32_hi = 1.462918119976564e-09f, c32_lo = -4.070940267922164e-17f;
    const float c9 = 1.7439342975337076e-16f;
    const float th = fA * c32_hi;
    const float tl = fmaf(fA, c32_hi, -th) + fmaf(fA, c32_lo, fB * c9);
    const float th2 = th * th;
    const float sl = fmaf(-th2 * th, 1.0f / 6.0f, tl);                             // sin = th + sl
    const float cm1 = fmaf(th2 * th2, 1.0f / 24.0f, fmaf(-0.5f, th2, -th * tl));  // cos - 1
    const float2 w = cmul_df(v, T512[j]);
    const float re = w.x + fmaf(-w.y, th, fmaf(w.x, cm1, -(w.y * sl)));
    const float im = w.y + fmaf(w.x, th, fmaf(w.y, cm1, w.x * sl));
    return make_float2(re, im);
}

}  // namespace fg
