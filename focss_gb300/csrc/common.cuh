// common.cuh -- shared device helpers for the focss GB300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fg {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float cnorm(float2 a) { return fmaf(a.x, a.x, a.y * a.y); }

// (cos phi, sin phi).  |phi| <= 1/4 (every step of an adaptive grid, whose
// nonlinear phase is bounded by construction): Taylor polynomials to degree
// 8/9 (truncation < 3e-13), about one FP32 rounding; larger phases take the
// reduced path below.
__device__ __forceinline__ float2 phase_rotation(float phi) {
    if (fabsf(phi) <= 0.25f) {
        const float p2 = phi * phi;
        const float s = phi * fmaf(p2, fmaf(p2, fmaf(p2, -1.0f / 5040.0f, 1.0f / 120.0f), -1.0f / 6.0f), 1.0f);
        const float c = fmaf(p2, fmaf(p2, fmaf(p2, fmaf(p2, 1.0f / 40320.0f, -1.0f / 720.0f), 1.0f / 24.0f), -0.5f),
                             1.0f);
        return make_float2(c, s);
    }
    // Larger phases: Cody-Waite reduction by q quarter turns (pi/2 as a
    // two-float constant), Taylor series on |r| <= pi/4 (truncation below
    // 3e-9), exact quarter-turn placement.  Straight-line code with no local
    // memory, so it stays cheap to inline in unrolled loops.
    const float q = rintf(phi * 0.63661977236758134f);
    float r = fmaf(-q, 1.57079637050628662f, phi);
    r = fmaf(q, 4.37113900018624284e-8f, r);
    const float r2 = r * r;
    const float sr = r * fmaf(r2, fmaf(r2, fmaf(r2, fmaf(r2, 1.0f / 362880.0f, -1.0f / 5040.0f), 1.0f / 120.0f),
                                        -1.0f / 6.0f), 1.0f);
    const float cr = fmaf(r2, fmaf(r2, fmaf(r2, fmaf(r2, fmaf(r2, -1.0f / 3628800.0f, 1.0f / 40320.0f),
                                                         -1.0f / 720.0f), 1.0f / 24.0f), -0.5f), 1.0f);
    const int k = (int)q & 3;
    const float c = (k & 1) ? -sr : cr, s = (k & 1) ? cr : sr;
    return (k & 2) ? make_float2(-c, -s) : make_float2(c, s);
}

// v * exp(i phi) applied as v + v * (cos(phi) - 1 + i sin(phi)) with cos(phi) - 1
// formed directly.  Rounding cos(phi) itself to FP32 makes |exp(i phi)| miss 1
// by up to 2^-25, and for |phi| < 2^-12 always upwards (cos rounds to exactly
// 1): a gain that repeats at every split step and grows the field error
// quadratically along a link.  The increment form leaves one unbiased rounding
// (the final additions).
__device__ __forceinline__ float2 kerr_rotate(float2 v, float phi) {
    float cm1, s;
    if (fabsf(phi) <= 0.25f) {
        // The increment multiplies v, so sin and cos - 1 need FP32 accuracy
        // relative to themselves: Taylor to phi^5 and phi^6 (truncation below
        // 5e-8 and 1.3e-8 relative at |phi| = 1/4).
        const float p2 = phi * phi;
        s = phi * fmaf(p2, fmaf(p2, 1.0f / 120.0f, -1.0f / 6.0f), 1.0f);
        cm1 = p2 * fmaf(p2, fmaf(p2, -1.0f / 720.0f, 1.0f / 24.0f), -0.5f);
    } else {
        const float2 r = phase_rotation(phi);  // cos(phi) <= 0.97: cos - 1 is exact
        cm1 = r.x - 1.0f;
        s = r.y;
    }
    const float dx = fmaf(v.x, cm1, -v.y * s);
    const float dy = fmaf(v.y, cm1, v.x * s);
    return make_float2(v.x + dx, v.y + dy);
}

// Block-wide reductions (blockDim.x multiple of 32, <= 1024).
// Programmatic dependent launch (kernels launched with the programmatic
// stream-serialization attribute): pdl_trigger lets the next such kernel in
// the stream be scheduled now; pdl_wait blocks until the grids this one
// depends on have completed and their memory is visible (a no-op in a kernel
// launched without the attribute).  A kernel reads or writes no global memory
// that its predecessors touch before pdl_wait.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Reduce (max, sum) over the block; result valid in thread 0.  `scratch` holds
// 2*32 floats.  Must be called by every thread of the block.
__device__ __forceinline__ void block_max_sum(float& mx, float& sm, float* scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    mx = warp_max(mx);
    sm = warp_sum(sm);
    __syncthreads();
    if (lane == 0) {
        scratch[warp] = mx;
        scratch[32 + warp] = sm;
    }
    __syncthreads();
    if (warp == 0) {
        mx = lane < nw ? scratch[lane] : 0.0f;
        sm = lane < nw ? scratch[32 + lane] : 0.0f;
        mx = warp_max(mx);
        sm = warp_sum(sm);
    }
}

__device__ __forceinline__ double block_sum_d(double v, double* scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum_d(v);
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < nw ? scratch[lane] : 0.0;
        v = warp_sum_d(v);
    }
    return v;
}

// A double as the unevaluated sum of two floats.
__host__ __device__ __forceinline__ float2 split_df(double v) {
    const float hi = (float)v;
    return make_float2(hi, (float)(v - (double)hi));
}

// Counter-based generator: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

// Box-Muller on two 24-bit uniforms (identical grid in the FP64 oracle).
__device__ __forceinline__ float2 gaussian_pair(uint32_t x0, uint32_t x1) {
    const float u1 = ((float)(x0 >> 8) + 0.5f) * (1.0f / 16777216.0f);
    const float u2 = (float)(x1 >> 8) * (1.0f / 16777216.0f);
    const float r = sqrtf(-2.0f * logf(u1));
    float s, c;
    sincospif(2.0f * u2, &s, &c);
    return make_float2(r * c, r * s);
}

// One sample of Amplifier::amplify / add_noise (src/focss/module/amplifier.cpp:15-28):
// scale*a + sigma*(z0 + i z1), (z0, z1) Box-Muller on Philox4x32-10 with
// counter {sample, mode + modes*realization, c_lo, c_hi} (element i of a
// realization-major, mode-major buffer of `samples` per mode).  The scale is a
// two-float sum hi + lo applied with a compensated product, so the span gain
// carries no FP32 rounding of its own that would repeat at every span.
__device__ __forceinline__ float2 amplifier_sample(float2 a, size_t i, int samples, float2 scale, float sigma,
                                                   uint2 key, uint32_t c_lo, uint32_t c_hi) {
    a.x = fmaf(a.x, scale.x, a.x * scale.y);
    a.y = fmaf(a.y, scale.x, a.y * scale.y);
    if (sigma != 0.0f) {
        const uint32_t sample = (uint32_t)(i % (size_t)samples);
        const uint32_t stream = (uint32_t)(i / (size_t)samples);
        const uint4 r = philox4x32_10(make_uint4(sample, stream, c_lo, c_hi), key);
        const float2 z = gaussian_pair(r.x, r.y);
        a.x = fmaf(sigma, z.x, a.x);
        a.y = fmaf(sigma, z.y, a.y);
    }
    return a;
}

}  // namespace fg
