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
#pragma once

#include "common.cuh"

namespace fg {

// cos(pi*j/32), j = 0..16
__host__ __device__ __forceinline__ constexpr float cos_pi32(int j) {
    constexpr float t[17] = {
        1.0f,
        0.99518472667219688624f,
        0.98078528040323044913f,
        0.95694033573220886494f,
        0.92387953251128675613f,
        0.88192126434835502971f,
        0.83146961230254523708f,
        0.77301045336273696081f,
        0.7071067811865475244f,
        0.63439328416364549822f,
        0.55557023301960222474f,
        0.47139673682599764856f,
        0.38268343236508977173f,
        0.29028467725446236764f,
        0.19509032201612826785f,
        0.098017140329560601994f,
        0.0f};
    return t[j];
}

// (cos, sin) of pi*idx/32 for idx in [0, 64)
__host__ __device__ __forceinline__ constexpr float2 cs64(int idx) {
    return idx <= 16   ? float2{cos_pi32(idx), cos_pi32(16 - idx)}
           : idx <= 32 ? float2{-cos_pi32(32 - idx), cos_pi32(idx - 16)}
           : idx <= 48 ? float2{-cos_pi32(idx - 32), -cos_pi32(48 - idx)}
                       : float2{cos_pi32(64 - idx), -cos_pi32(idx - 48)};
}

// a * exp(-+ i*pi*idx/32): forward uses the minus sign.
template <bool INV>
__device__ __forceinline__ float2 twmul64(float2 a, int idx) {
    idx &= 63;
    if (idx == 0) return a;
    if (idx == 32) return make_float2(-a.x, -a.y);
    if (idx == 16) return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
    if (idx == 48) return INV ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
    const float2 w = cs64(idx);
    const float s = INV ? w.y : -w.y;
    return make_float2(fmaf(a.x, w.x, -a.y * s), fmaf(a.x, s, a.y * w.x));
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
template <> struct PQ<2048> { static constexpr int P = 32, Q = 64; };

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

// Group-wide sub-FFT (see file comment).  twL[e] = exp(-2 pi i e / L), e < L.
// BLOCK_SYNC selects __syncthreads (group spans warps) or __syncwarp.
template <int P, int Q, bool INV, bool BLOCK_SYNC, class Lay>
__device__ __forceinline__ void fft_pq(float2 (&v)[Q], float2* __restrict__ sm, const Lay lay, int t,
                                       const float2* __restrict__ twL) {
    static_assert(Q % P == 0, "Q must be a multiple of P");
    constexpr int M = Q / P;
    dft<Q, INV>(v);
#pragma unroll
    for (int u = 1; u < Q; ++u) {
        float2 w = twL[t * u];
        if (INV) w.y = -w.y;
        v[u] = cmul(v[u], w);
    }
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

}  // namespace fg
