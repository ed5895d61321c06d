// dsp_chain.cu -- transmitter / receiver DSP around the split-step path:
// 16QAM mapping, resampling, RRC shaping and matched filtering, spectral
// decimation, WDM multiplexing and channel selection, hard decisions, BER/SER,
// EVM/Q and the linear equalizers (reference: src/focss/processing/
// modulation.cpp, src/focss/field.cpp, src/focss/functions.cpp,
// src/focss/equalizer/*_equalizer.cpp).
//
// Filters reuse the two-pass FFT passes: the filter spectrum is computed once
// on the device, cached per (length, parameters) in the two-pass transposed
// layout, and applied by the row pass (ROW_TABLE) between the column passes.
// Decisions and metric sums run in FP64 (O(N), off the split-step hot loop)
// so that symbol decisions reproduce the reference's FP64 comparisons.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace fg {
namespace {

inline int grid_for(size_t n, int threads) {
    size_t g = (n + threads - 1) / threads;
    if (g > (size_t)sm_count() * 32) g = (size_t)sm_count() * 32;
    return (int)(g ? g : 1);
}

// Per-realization grid (x: samples of one realization, y: realization) with
// about 8 CTAs of 256 threads per SM over the whole launch (each CTA forms
// its realization's FP64 scale once, so fewer, longer CTAs amortize it).
inline dim3 grid_per_realization(size_t per, int batch) {
    const size_t by_work = (per + 255) / 256, by_fill = ((size_t)sm_count() * 8 + batch - 1) / (size_t)batch;
    size_t gx = by_work < by_fill ? by_work : by_fill;
    return dim3((unsigned)(gx ? gx : 1), (unsigned)batch);
}

#define FG_LAUNCH(...)       \
    do {                     \
        __VA_ARGS__;         \
        ::fg::count_launch(); \
    } while (0)

// Gray 16QAM constellation (src/focss/processing/modulation.cpp:9-17), FP64.
__constant__ double c_gray_re[16] = {-3, -1, 3, 1, -3, -1, 3, 1, -3, -1, 3, 1, -3, -1, 3, 1};
__constant__ double c_gray_im[16] = {-3, -3, -3, -3, -1, -1, -1, -1, 3, 3, 3, 3, 1, 1, 1, 1};

// demodulate_16qam (modulation.cpp:98-110): argmin over the 16 points, ties
// to the lowest code, FP64 distances.  The 16 points are the products of 4
// in-phase and 4 quadrature levels, so the 4 + 4 coordinate differences (the
// same values the point-by-point form computes) and the 4 quadrature squares
// are formed once and each distance is one fused multiply-add.
__device__ __forceinline__ unsigned demod16(double re, double im) {
    const double s = 1.0 / sqrt(10.0);
    double dr[4], qi[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        dr[l] = re - c_gray_re[l] * s;            // levels of codes l, l + 4, l + 8, l + 12
        const double di = im - c_gray_im[4 * l] * s;  // level of codes 4l .. 4l + 3
        qi[l] = di * di;
    }
    unsigned arg = 0;
    double mn = fma(dr[0], dr[0], qi[0]);
#pragma unroll
    for (unsigned code = 1; code < 16; ++code) {
        const double d = fma(dr[code & 3], dr[code & 3], qi[code >> 2]);
        if (mn > d) {
            mn = d;
            arg = code;
        }
    }
    return arg;
}

// The same decision from FP32 coordinates, where that is provably the same:
// the nearest point of the square grid is the nearest level on each axis,
// and a coordinate farther than kNear (1e-5 (1 + |v|)) from every level
// boundary (0, +-2/sqrt 10) has that level under the FP64 argmin above as
// well -- the FP32 coordinate is within 2e-7 |v| of the FP64 one, and the
// FP64 distances of the two nearest points then differ by ~1e-5, far above
// their rounding.  `near` is set when a coordinate is closer than that (or
// NaN); the caller then decides with demod16 on its FP64 coordinates, so
// the codes are those of the FP64 argmin for every input.
__device__ __forceinline__ bool near_value(float v, float t) {
    return !(fabsf(v - t) > 1e-5f * (1.0f + fabsf(v)));
}
__device__ __forceinline__ unsigned level4(float v, bool& near) {
    constexpr float kB = 0.632455532f;  // 2/sqrt(10)
    const float a = fabsf(v);
    near = near || near_value(a, 0.0f) || near_value(a, kB);
    // levels -3, -1, 1, 3 (/sqrt 10) are table indices 0, 1, 3, 2 on both axes
    return v < 0.0f ? (v < -kB ? 0u : 1u) : (v < kB ? 3u : 2u);
}
__device__ __forceinline__ unsigned demod16_f32(float re, float im, bool& near) {
    near = false;
    const unsigned lr = level4(re, near);
    const unsigned li = level4(im, near);
    return lr | (li << 2);
}

// FP64 fallbacks as calls: kept out of line so that the compiler does not
// if-convert them into every sample's path (GB300's FP64 pipe is narrow).
__device__ __noinline__ unsigned demod16_div(float x, float y, double sp) {
    return demod16((double)x / sp, (double)y / sp);
}
__device__ __noinline__ unsigned demod16_mul(float x, float y, double sc) { return demod16(sc * x, sc * y); }

__global__ void qam_map_kernel(const int32_t* __restrict__ codes, float2* __restrict__ out, size_t n) {
    const double s = 1.0 / sqrt(10.0);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int c = codes[i] & 15;
        out[i] = make_float2((float)(c_gray_re[c] * s), (float)(c_gray_im[c] * s));
    }
}

__global__ void upsample_kernel(const float2* __restrict__ in, float2* __restrict__ out, size_t n_in, int factor) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n_in; i += (size_t)gridDim.x * blockDim.x)
        out[i * factor] = in[i];
}

__global__ void downsample_kernel(const float2* __restrict__ in, float2* __restrict__ out, size_t n_out, int factor,
                                  float scale) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n_out; i += (size_t)gridDim.x * blockDim.x)
        out[i] = cscale(in[i * factor], scale);
}

// pulse::rrc taps in FP64 (modulation.cpp:47-74), before power normalization.
__global__ void rrc_taps_kernel(int n_symbols, int osf, double roll_off, double* __restrict__ taps, int len,
                                double* __restrict__ power) {
    const double pi = 3.14159265358979323846264338;
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
        const double t = (double)i / osf - n_symbols / 2.0;
        double v = 0.0;
        if (t == 0) {
            v = 1 - roll_off + 4 * roll_off / pi;
        } else if (fabs(t) == 1 / roll_off / 4) {
            v += (1 + 2 / pi) * sin(pi / roll_off / 4);
            v += (1 - 2 / pi) * cos(pi / roll_off / 4);
            v *= roll_off / sqrt(2.0);
        } else {
            v += cos(pi * t * (1 + roll_off));
            v *= 4 * roll_off * t;
            v += sin(pi * t * (1 - roll_off));
            v /= 1 - 16 * roll_off * roll_off * t * t;
            v /= pi * t;
        }
        taps[i] = v;
        acc += v * v;
    }
    __shared__ double sd[32];
    acc = block_sum_d(acc, sd);
    if (threadIdx.x == 0) atomicAdd(power, acc);
}

// Field::filter_inplace's ifftshifted, zero-padded response (field.cpp:359-365):
// zp[i] = h[i + half], zp[shift + i] = h[i] (i < h_len/2), times `scale`.
__global__ void zero_pad_kernel(const double* __restrict__ h_re, const double* __restrict__ h_im, int h_len,
                                int samples, const double* __restrict__ power, double len_for_norm,
                                float2* __restrict__ zp) {
    const double s = power ? len_for_norm / *power : 1.0;
    const int half = h_len / 2, shift = samples - half;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < samples; i += gridDim.x * blockDim.x) {
        double re = 0, im = 0;
        if (i < half) {
            re = h_re[i + half];
            im = h_im ? h_im[i + half] : 0.0;
        } else if (i >= shift && i - shift < half) {
            re = h_re[i - shift];
            im = h_im ? h_im[i - shift] : 0.0;
        }
        zp[i] = make_float2((float)(re * s), (float)(im * s));
    }
}

__global__ void scale_taps_kernel(double* __restrict__ taps, int len, const double* __restrict__ power,
                                  double* __restrict__ out_interleaved) {
    const double s = (double)len / *power;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
        out_interleaved[2 * i] = taps[i] * s;
        out_interleaved[2 * i + 1] = 0.0;
    }
}

// Decimation gather: out (M samples, transposed layout M1 x M2) takes bin
// k_out of the N-point spectrum `in` (transposed layout N1 x N2), with the
// reference's bin map (field.cpp:309-317).
__global__ void decimate_gather_kernel(const float2* __restrict__ in, float2* __restrict__ out, int N, int N1,
                                       int N2, int M, int M1, int M2, int rows) {
    const int cutoff = M / 2, shift = N - M;
    const size_t total = (size_t)rows * M;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t r = i / M;
        const int p = (int)(i % M);
        const int k1 = p / M2, k2 = p % M2;
        const int kout = k1 + M1 * k2;
        const int kin = kout < cutoff ? kout : kout + shift;
        out[i] = in[r * N + (size_t)(kin % N1) * N2 + kin / N1];
    }
}

// A *= exp(2 pi i x n), x = X / 2^64 turns per sample (two's complement),
// X n formed exactly modulo 2^64 (modulation.cpp:255-264).
__global__ void freq_shift_kernel(float2* __restrict__ d, int samples, size_t n, unsigned long long X) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const unsigned long long s = (unsigned long long)(i % (size_t)samples);
        const float x = (float)(long long)(X * s) * 1.0842021724855044e-19f;
        float sn, cs;
        sincospif(x, &sn, &cs);
        d[i] = cmul(d[i], make_float2(cs, sn));
    }
}

// wdm_mux: out[m,s] = sum_c ch_c[m,s] exp(2 pi i f_c dt s)
__global__ void wdm_mux_kernel(const float2* __restrict__ ch, int n_ch, int modes, int samples,
                               const unsigned long long* __restrict__ X, float2* __restrict__ out) {
    const size_t per = (size_t)modes * samples;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < per; i += (size_t)gridDim.x * blockDim.x) {
        const unsigned long long s = (unsigned long long)(i % (size_t)samples);
        float2 acc = make_float2(0.f, 0.f);
        for (int c = 0; c < n_ch; ++c) {
            const float x = (float)(long long)(X[c] * s) * 1.0842021724855044e-19f;
            float sn, cs;
            sincospif(x, &sn, &cs);
            acc = cadd(acc, cmul(ch[c * per + i], make_float2(cs, sn)));
        }
        out[i] = acc;
    }
}

// Per-realization FP64 power sum over all modes and samples (for decision scales).
__global__ void power_sum_kernel(const float2* __restrict__ d, size_t per, double* __restrict__ out) {
    const int b = blockIdx.y;
    const float2* base = d + (size_t)b * per;
    double acc = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < per; i += (size_t)gridDim.x * blockDim.x) {
        const double x = base[i].x, y = base[i].y;
        acc += x * x + y * y;
    }
    __shared__ double sd[32];
    acc = block_sum_d(acc, sd);
    if (threadIdx.x == 0) atomicAdd(out + b, acc);
}

// hard_decision_16qam (modulation.cpp:112-120): power = avg/modes,
// out = sqrt(power) * gray[demod(in / sqrt(power))].
// Grid (samples, realization): the realization's scale is formed once per thread.
__global__ void hard_decision_kernel(const float2* __restrict__ in, float2* __restrict__ out, int modes, int samples,
                                     size_t per, const double* __restrict__ psum) {
    const double s10 = 1.0 / sqrt(10.0);
    const int b = blockIdx.y;
    const double power = psum[b] / samples / modes;
    const double sp = sqrt(power);
    in += (size_t)b * per;
    out += (size_t)b * per;
    // the 16 outputs, formed once per CTA (a per-sample lookup with divergent
    // codes would serialize in the constant cache)
    __shared__ float2 s_out[16];
    if (threadIdx.x < 16)
        s_out[threadIdx.x] = make_float2((float)(sp * (c_gray_re[threadIdx.x] * s10)),
                                         (float)(sp * (c_gray_im[threadIdx.x] * s10)));
    __syncthreads();
    const float inv = (float)(1.0 / sp);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < per; i += (size_t)gridDim.x * blockDim.x) {
        const float2 z = in[i];
        bool near;
        unsigned c = demod16_f32(z.x * inv, z.y * inv, near);
        if (near) c = demod16_div(z.x, z.y, sp);
        out[i] = s_out[c];
    }
}

// The FP64 forms of one soft decision (modulation.cpp:122-146) and one
// certainty decision (src/tasks/wdm_scoring.cpp:128-144), out of line.
__device__ __noinline__ float2 soft_decision_fp64(float2 z, double sp, double thr) {
    const double s10 = 1.0 / sqrt(10.0), pivot = 2.0 / sqrt(10.0);
    const double re = (double)z.x / sp, im = (double)z.y / sp;
    const unsigned c = demod16(re, im);
    double gr = c_gray_re[c] * s10, gi = c_gray_im[c] * s10;
    if (fabs(re) < thr || fabs(re - pivot) < thr || fabs(re + pivot) < thr) gr = re;
    if (fabs(im) < thr || fabs(im - pivot) < thr || fabs(im + pivot) < thr) gi = im;
    return make_float2((float)(sp * gr), (float)(sp * gi));
}
__device__ __noinline__ float2 certainty_decision_fp64(float2 z, double amp, double thr) {
    const double s10 = 1.0 / sqrt(10.0);
    double re = (double)z.x / amp, im = (double)z.y / amp;
    const unsigned c = demod16(re, im);
    const double gr = c_gray_re[c] * s10, gi = c_gray_im[c] * s10;
    if (hypot(gr - re, gi - im) < thr) {
        re = gr;
        im = gi;
    }
    return make_float2((float)(amp * re), (float)(amp * im));
}

// soft_decision_16qam (modulation.cpp:122-146): per quadrature the hard
// decision, unless the normalized received value lies within
// sqrt(10)*uncertainty of a decision boundary (0, +-2/sqrt(10)); then it is kept.
__global__ void soft_decision_kernel(const float2* __restrict__ in, float2* __restrict__ out, int modes, int samples,
                                     size_t per, const double* __restrict__ psum, double uncertainty) {
    const double s10 = 1.0 / sqrt(10.0);
    const double pivot = 2.0 / sqrt(10.0), thr = sqrt(10.0) * uncertainty;
    const int b = blockIdx.y;
    const double power = psum[b] / samples / modes;
    const double sp = sqrt(power);
    in += (size_t)b * per;
    out += (size_t)b * per;
    // FP32 first, as in demod16_f32: a quadrature is kept when its distance
    // to 0 or +-pivot is below thr; a distance within 1e-5 (1 + |v|) of thr
    // goes to the FP64 form.  A kept value is written as the input itself,
    // which is what float(sp * (x / sp)) rounds to for every FP32 x (the FP64
    // round trip moves x by < 2^-51 |x|, below half an FP32 unit).
    __shared__ float2 s_out[16];  // decided outputs, as in hard_decision_kernel
    if (threadIdx.x < 16)
        s_out[threadIdx.x] = make_float2((float)(sp * (c_gray_re[threadIdx.x] * s10)),
                                         (float)(sp * (c_gray_im[threadIdx.x] * s10)));
    __syncthreads();
    const float inv = (float)(1.0 / sp), thr32 = (float)thr, pv32 = (float)pivot;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < per; i += (size_t)gridDim.x * blockDim.x) {
        const float2 z = in[i];
        const float r32 = z.x * inv, i32 = z.y * inv;
        bool near;
        unsigned c = demod16_f32(r32, i32, near);
        const float dr0 = fabsf(r32), dr1 = fabsf(r32 - pv32), dr2 = fabsf(r32 + pv32);
        const float di0 = fabsf(i32), di1 = fabsf(i32 - pv32), di2 = fabsf(i32 + pv32);
        near = near || near_value(dr0, thr32) || near_value(dr1, thr32) || near_value(dr2, thr32) ||
               near_value(di0, thr32) || near_value(di1, thr32) || near_value(di2, thr32);
        if (!near) {
            const bool keep_r = dr0 < thr32 || dr1 < thr32 || dr2 < thr32;
            const bool keep_i = di0 < thr32 || di1 < thr32 || di2 < thr32;
            const float2 d = s_out[c];
            out[i] = make_float2(keep_r ? z.x : d.x, keep_i ? z.y : d.y);
            continue;
        }
        out[i] = soft_decision_fp64(z, sp, thr);
    }
}

// find_certainty (src/tasks/wdm_scoring.cpp:105-126), device part: per
// realization the smallest |gray[rx_code] / scale - rx| over samples whose
// decision differs from the transmitted one, scale = sqrt(n) / ||tx||_F.
// Distances are non-negative doubles, so their bit patterns order like the
// values and atomicMin on them is a min over doubles.
__global__ void certainty_kernel(const float2* __restrict__ tx, const float2* __restrict__ rx, size_t per,
                                 const double* __restrict__ psum_tx, unsigned long long* __restrict__ dmin) {
    const int b = blockIdx.y;
    const double scale = sqrt((double)per) / sqrt(psum_tx[b]);
    const float sc32 = (float)scale;
    const double s10 = 1.0 / sqrt(10.0);
    double best = __longlong_as_double(0x7FF0000000000000LL);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < per; i += (size_t)gridDim.x * blockDim.x) {
        const size_t k = (size_t)b * per + i;
        const float2 t = tx[k], r = rx[k];
        const double rr = r.x, ri = r.y;
        bool near;
        unsigned tc = demod16_f32(t.x * sc32, t.y * sc32, near);
        if (near) tc = demod16_mul(t.x, t.y, scale);
        unsigned rc = demod16_f32(r.x * sc32, r.y * sc32, near);
        if (near) rc = demod16_mul(r.x, r.y, scale);
        if (tc ^ rc) best = fmin(best, hypot(c_gray_re[rc] * s10 / scale - rr, c_gray_im[rc] * s10 / scale - ri));
    }
    for (int o = 16; o > 0; o >>= 1) best = fmin(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0 && best < __longlong_as_double(0x7FF0000000000000LL))
        atomicMin(dmin + b, (unsigned long long)__double_as_longlong(best));
}

// sd (src/tasks/wdm_scoring.cpp:128-144): at the RMS amplitude amp, a sample
// snaps to its decided point when closer than certainty / sqrt(5).
__global__ void certainty_decision_kernel(const float2* __restrict__ in, float2* __restrict__ out, size_t per,
                                          const double* __restrict__ psum, double certainty) {
    const double s10 = 1.0 / sqrt(10.0);
    const double thr = certainty / sqrt(5.0);
    const int b = blockIdx.y;
    const double amp = sqrt(psum[b]) / sqrt((double)per);
    in += (size_t)b * per;
    out += (size_t)b * per;
    // FP32 first (demod16_f32; the distance to the decided point against thr
    // with the same 1e-5 (1 + d) guard band); a kept sample is written as the
    // input itself, which float(amp * (x / amp)) rounds to for every FP32 x.
    __shared__ float2 s_pt[16], s_out[16];  // normalized points (FP32) and snapped outputs
    if (threadIdx.x < 16) {
        s_pt[threadIdx.x] = make_float2((float)(c_gray_re[threadIdx.x] * s10), (float)(c_gray_im[threadIdx.x] * s10));
        s_out[threadIdx.x] = make_float2((float)(amp * (c_gray_re[threadIdx.x] * s10)),
                                         (float)(amp * (c_gray_im[threadIdx.x] * s10)));
    }
    __syncthreads();
    const float inv = (float)(1.0 / amp), thr32 = (float)thr;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < per; i += (size_t)gridDim.x * blockDim.x) {
        const float2 z = in[i];
        const float r32 = z.x * inv, i32 = z.y * inv;
        bool near;
        unsigned c = demod16_f32(r32, i32, near);
        if (!near) {
            const float2 p = s_pt[c];
            const float d = hypotf(p.x - r32, p.y - i32);
            if (!near_value(d, thr32)) {
                out[i] = d < thr32 ? s_out[c] : z;
                continue;
            }
        }
        out[i] = certainty_decision_fp64(z, amp, thr);
    }
}

// hd_sequence_16qam (modulation.cpp:148-156): scale = sqrt(modes / average_power).
__global__ void hd_codes_kernel(const float2* __restrict__ in, int32_t* __restrict__ codes, int modes, int samples,
                                size_t per, const double* __restrict__ psum) {
    const int b = blockIdx.y;
    const double sc = sqrt(modes / (psum[b] / samples));
    in += (size_t)b * per;
    codes += (size_t)b * per;
    const float sc32 = (float)sc;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < per; i += (size_t)gridDim.x * blockDim.x) {
        const float2 z = in[i];
        bool near;
        unsigned c = demod16_f32(z.x * sc32, z.y * sc32, near);
        if (near) c = demod16_mul(z.x, z.y, sc);
        codes[i] = (int32_t)c;
    }
}

// Decision errors over samples [cut, samples - cut) (modulation.cpp:158-223);
// both sequences scaled by sqrt(modes / average_power(tx)).
__global__ void error_count_kernel(const float2* __restrict__ tx, const float2* __restrict__ rx, int modes,
                                   int samples, int cut, const double* __restrict__ psum_tx,
                                   unsigned long long* __restrict__ counts) {
    const int b = blockIdx.y;
    const size_t per = (size_t)modes * samples;
    const double sc = sqrt(modes / (psum_tx[b] / samples));
    const float sc32 = (float)sc;
    const int span = samples - 2 * cut;
    unsigned long long be = 0, se = 0;
    if (span > 0) {
        const size_t total = (size_t)modes * span;
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
            const int m = (int)(i / span);
            const int s = cut + (int)(i % span);
            const size_t k = (size_t)b * per + (size_t)m * samples + s;
            const float2 t = tx[k], r = rx[k];
            bool near;
            unsigned tc = demod16_f32(t.x * sc32, t.y * sc32, near);
            if (near) tc = demod16_mul(t.x, t.y, sc);
            unsigned rc = demod16_f32(r.x * sc32, r.y * sc32, near);
            if (near) rc = demod16_mul(r.x, r.y, sc);
            const int d = __popc(tc ^ rc);
            be += d;
            se += d > 0;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        be += __shfl_xor_sync(0xffffffffu, be, o);
        se += __shfl_xor_sync(0xffffffffu, se, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(counts + 2 * b, be);
        atomicAdd(counts + 2 * b + 1, se);
    }
}

// FP64 pair sums over samples [lo, hi) of every mode:
// out[8b + 0] = sum |t|^2, 1 = sum |r|^2, 2 = sum |t - r|^2, 3/4 = sum conj(r) t (re/im),
// 5/6 = sum conj(t) r (re/im).
__global__ void pair_sums_kernel(const float2* __restrict__ t, const float2* __restrict__ r, int modes, int samples,
                                 int lo, int hi, double* __restrict__ out) {
    const int b = blockIdx.y;
    const size_t per = (size_t)modes * samples;
    const int span = hi - lo;
    double a[7] = {0, 0, 0, 0, 0, 0, 0};
    if (span > 0) {
        const size_t total = (size_t)modes * span;
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
            const int m = (int)(i / span);
            const int s = lo + (int)(i % span);
            const size_t k = (size_t)b * per + (size_t)m * samples + s;
            const double tr = t[k].x, ti = t[k].y, rr = r[k].x, ri = r[k].y;
            const double dr = tr - rr, di = ti - ri;
            a[0] += tr * tr + ti * ti;
            a[1] += rr * rr + ri * ri;
            a[2] += dr * dr + di * di;
            a[3] += rr * tr + ri * ti;  // conj(r) t
            a[4] += rr * ti - ri * tr;
            a[5] += tr * rr + ti * ri;  // conj(t) r
            a[6] += tr * ri - ti * rr;
        }
    }
    __shared__ double sd[32];
    for (int q = 0; q < 7; ++q) {
        const double v = block_sum_d(a[q], sd);
        if (threadIdx.x == 0) atomicAdd(out + 8 * b + q, v);
        __syncthreads();
    }
}

// PhaseShiftEqualizer::estimate argmax over i = 0..steps-1 (first maximum
// wins): q2 is monotone in Re(e^{i angle} sum conj(t) r).
__global__ void pse_argmax_kernel(const double* __restrict__ sums, int steps, double* __restrict__ angle) {
    const int b = blockIdx.x;
    const double cr = sums[8 * b + 5], ci = sums[8 * b + 6];
    const double two_pi = 2 * 3.14159265358979323846264338;
    double best = -1e308;
    int bi = 0;
    for (int i = threadIdx.x; i < steps; i += blockDim.x) {
        const double ang = two_pi * (double)i / steps;
        const double v = cr * cos(ang) - ci * sin(ang);
        if (v > best) {
            best = v;
            bi = i;
        }
    }
    __shared__ double sv[1024];
    __shared__ int si[1024];
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bi;
    __syncthreads();
    if (threadIdx.x == 0) {
        double bv = sv[0];
        int bidx = si[0];
        for (int k = 1; k < (int)blockDim.x; ++k)
            if (sv[k] > bv || (sv[k] == bv && si[k] < bidx)) {
                bv = sv[k];
                bidx = si[k];
            }
        angle[b] = two_pi * (double)bidx / steps;
    }
}

__global__ void scale_each_kernel(float2* __restrict__ d, size_t per, size_t n, const float2* __restrict__ s) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        d[i] = cmul(d[i], s[i / per]);
}

// ---------------------------------------------------------------- host helpers
focss_status check_same(Ctx* c, const Field* a, const Field* b) {
    if (a->modes != b->modes || a->samples != b->samples || a->batch != b->batch)
        return set_error(c, FOCSS_ERR_INVALID_ARG, "fields must have the same modes, samples and batch");
    return FOCSS_OK;
}

unsigned long long turns_fix64_host(double a) {
    const double ab = std::fabs(a);
    const double fr = ab - std::floor(ab);
    const double sc = std::ldexp(fr, 64);
    unsigned long long A = sc >= 18446744073709551615.0 ? 0ull : (unsigned long long)sc;
    return a < 0 ? (0ull - A) : A;
}

// Spectrum of the ifftshifted, power-normalized RRC pulse in the transposed
// two-pass layout (unnormalized forward FFT), cached per (N, n_symbols, osf, roll-off).
focss_status rrc_table(Ctx* c, int samples, int n_symbols, int osf, double roll_off, const float2** out) {
    char key[160];
    snprintf(key, sizeof(key), "rrc:%d:%d:%d:%.17g", samples, n_symbols, osf, roll_off);
    auto it = c->tables.find(key);
    if (it != c->tables.end()) {
        *out = (const float2*)it->second;
        return FOCSS_OK;
    }
    const int len = n_symbols * osf;
    double* taps = nullptr;
    float2* tab = nullptr;
    cudaError_t e = cudaMalloc(&taps, sizeof(double) * (len + 1));
    if (e == cudaSuccess) e = cudaMalloc(&tab, sizeof(float2) * samples);
    if (e != cudaSuccess) {
        cudaFree(taps);
        cudaFree(tab);
        return cuda_check(c, e, "rrc table alloc");
    }
    double* power = taps + len;
    cudaStream_t s = c->stream;
    e = cudaMemsetAsync(power, 0, sizeof(double), s);
    if (e == cudaSuccess) FG_LAUNCH(rrc_taps_kernel<<<grid_for(len, 256), 256, 0, s>>>(n_symbols, osf, roll_off, taps, len, power));
    if (e == cudaSuccess) FG_LAUNCH(zero_pad_kernel<<<grid_for(samples, 256), 256, 0, s>>>(taps, nullptr, len, samples, power, (double)len, tab));
    if (e == cudaSuccess) e = cudaGetLastError();
    focss_status st = cuda_check(c, e, "rrc taps");
    if (st == FOCSS_OK) st = fft_forward_transposed(c, tab, samples, 1, 1.0f);
    if (st == FOCSS_OK) st = cuda_check(c, cudaStreamSynchronize(s), "rrc table sync");
    cudaFree(taps);
    if (st != FOCSS_OK) {
        cudaFree(tab);
        return st;
    }
    c->tables[key] = tab;
    *out = tab;
    return FOCSS_OK;
}

// In place: data <- IFFT(FFT(data)/N * H/N) * extra for H in transposed layout
// (Field::filter_inplace, field.cpp:358-372).
focss_status apply_filter(Ctx* c, float2* d, int samples, int rows, const float2* H, double extra) {
    const double g = extra / ((double)samples * (double)samples);
    return spectral_apply(c, d, samples, rows, ROW_TABLE, H, (float)g, 0);
}

focss_status sums_for(Ctx* c, const Field* t, const Field* r, int lo, int hi, std::vector<double>& host) {
    focss_status st = ensure_red(c, 8 * (size_t)t->batch);
    if (st != FOCSS_OK) return st;
    cudaStream_t s = c->stream;
    cudaError_t e = cudaMemsetAsync(c->d_red, 0, sizeof(double) * 8 * t->batch, s);
    const int gx = std::max(1, std::min(64, (int)(((size_t)t->modes * std::max(hi - lo, 1) + 1023) / 1024)));
    if (e == cudaSuccess) FG_LAUNCH(pair_sums_kernel<<<dim3(gx, t->batch), 256, 0, s>>>(t->d, r->d, t->modes, t->samples, lo, hi, c->d_red));
    if (e == cudaSuccess) e = cudaGetLastError();
    host.assign(8 * (size_t)t->batch, 0.0);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host.data(), c->d_red, sizeof(double) * 8 * t->batch, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return cuda_check(c, e, "pair sums");
}

focss_status power_sums(Ctx* c, const Field* f, double* dst_device) {
    cudaStream_t s = c->stream;
    cudaError_t e = cudaMemsetAsync(dst_device, 0, sizeof(double) * f->batch, s);
    const size_t per = (size_t)f->modes * f->samples;
    const int gx = std::max(1, std::min(64, (int)((per + 1023) / 1024)));
    if (e == cudaSuccess) FG_LAUNCH(power_sum_kernel<<<dim3(gx, f->batch), 256, 0, s>>>(f->d, per, dst_device));
    if (e == cudaSuccess) e = cudaGetLastError();
    return cuda_check(c, e, "power sums");
}

int clamp_cut(int cut) { return cut < 0 ? 0 : cut; }

}  // namespace
}  // namespace fg

using fg::Ctx;
using fg::Field;

extern "C" {

FOCSS_API focss_status focss_qam16_map(focss_ctx* c, const int32_t* codes, size_t n, focss_field* out) {
    if (!c || !codes || !out) return FOCSS_ERR_INVALID_ARG;
    if (n != out->n()) return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "qam16_map: size mismatch");
    int32_t* d = (int32_t*)fg::scratch_buffer(c, 1, sizeof(int32_t) * n);
    if (!d) return fg::set_error(c, FOCSS_ERR_OOM, "qam16_map scratch");
    cudaError_t e = cudaMemcpyAsync(d, codes, sizeof(int32_t) * n, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) FG_LAUNCH(fg::qam_map_kernel<<<fg::grid_for(n, 256), 256, 0, c->stream>>>(d, out->d, n));
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return fg::cuda_check(c, e, "qam16_map");
}

FOCSS_API focss_status focss_upsample(focss_ctx* c, const focss_field* in, int factor, focss_field* out) {
    if (!c || !in || !out || factor <= 0) return FOCSS_ERR_INVALID_ARG;
    if (out->modes != in->modes || out->batch != in->batch || (long long)out->samples != (long long)in->samples * factor)
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "upsample: output shape");
    cudaError_t e = cudaMemsetAsync(out->d, 0, sizeof(float2) * out->n(), c->stream);
    if (e == cudaSuccess) FG_LAUNCH(fg::upsample_kernel<<<fg::grid_for(in->n(), 256), 256, 0, c->stream>>>(in->d, out->d, in->n(), factor));
    if (e == cudaSuccess) e = cudaGetLastError();
    return fg::cuda_check(c, e, "upsample");
}

FOCSS_API focss_status focss_downsample(focss_ctx* c, const focss_field* in, int factor, focss_field* out) {
    if (!c || !in || !out || factor <= 0 || in->samples % factor) return FOCSS_ERR_INVALID_ARG;
    if (out->modes != in->modes || out->batch != in->batch || out->samples != in->samples / factor)
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "downsample: output shape");
    FG_LAUNCH(fg::downsample_kernel<<<fg::grid_for(out->n(), 256), 256, 0, c->stream>>>(in->d, out->d, out->n(), factor, 1.0f));
    return fg::cuda_check(c, cudaGetLastError(), "downsample");
}

FOCSS_API focss_status focss_decimate(focss_ctx* c, const focss_field* in, int factor, focss_field* out) {
    if (!c || !in || !out || factor <= 0 || in->samples % factor) return FOCSS_ERR_INVALID_ARG;
    if (out->modes != in->modes || out->batch != in->batch || out->samples != in->samples / factor)
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "decimate: output shape");
    const fg::Plan *pi = nullptr, *po = nullptr;
    focss_status st = fg::get_plan(c, in->samples, &pi);
    if (st == FOCSS_OK) st = fg::get_plan(c, out->samples, &po);
    if (st != FOCSS_OK) return st;
    const int rows = in->batch * in->modes;
    float2* sp = (float2*)fg::scratch_buffer(c, 2, sizeof(float2) * in->n());
    if (!sp) return fg::set_error(c, FOCSS_ERR_OOM, "decimate scratch");
    cudaError_t e = cudaMemcpyAsync(sp, in->d, sizeof(float2) * in->n(), cudaMemcpyDeviceToDevice, c->stream);
    if (e != cudaSuccess) return fg::cuda_check(c, e, "decimate copy");
    st = fg::fft_forward_transposed(c, sp, in->samples, rows, 1.0f / (float)in->samples);
    if (st != FOCSS_OK) return st;
    FG_LAUNCH(fg::decimate_gather_kernel<<<fg::grid_for(out->n(), 256), 256, 0, c->stream>>>(
        sp, out->d, pi->N, pi->N1, pi->N2, po->N, po->N1, po->N2, rows));
    e = cudaGetLastError();
    if (e != cudaSuccess) return fg::cuda_check(c, e, "decimate gather");
    return fg::fft_inverse_transposed(c, out->d, out->samples, rows);
}

FOCSS_API focss_status focss_rrc_pulse(focss_ctx* c, int n_symbols, int osf, double roll_off, double* taps) {
    if (!c || !taps || n_symbols <= 0 || osf <= 0) return FOCSS_ERR_INVALID_ARG;
    const int len = n_symbols * osf;
    double* d = (double*)fg::scratch_buffer(c, 3, sizeof(double) * (3 * (size_t)len + 1));
    if (!d) return fg::set_error(c, FOCSS_ERR_OOM, "rrc scratch");
    double* power = d + len;
    double* out = d + len + 1;
    cudaStream_t s = c->stream;
    cudaError_t e = cudaMemsetAsync(power, 0, sizeof(double), s);
    if (e == cudaSuccess) FG_LAUNCH(fg::rrc_taps_kernel<<<fg::grid_for(len, 256), 256, 0, s>>>(n_symbols, osf, roll_off, d, len, power));
    if (e == cudaSuccess) FG_LAUNCH(fg::scale_taps_kernel<<<fg::grid_for(len, 256), 256, 0, s>>>(d, len, power, out));
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(taps, out, sizeof(double) * 2 * len, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return fg::cuda_check(c, e, "rrc_pulse");
}

FOCSS_API focss_status focss_filter(focss_ctx* c, focss_field* f, const double* h, int h_len) {
    if (!c || !f || !h || h_len <= 0 || h_len > f->samples) return FOCSS_ERR_INVALID_ARG;
    const fg::Plan* p = nullptr;
    focss_status st = fg::get_plan(c, f->samples, &p);
    if (st != FOCSS_OK) return st;
    std::vector<double> re(h_len), im(h_len);
    for (int i = 0; i < h_len; ++i) {
        re[i] = h[2 * i];
        im[i] = h[2 * i + 1];
    }
    double* dh = (double*)fg::scratch_buffer(c, 3, sizeof(double) * 2 * (size_t)h_len);
    float2* tab = (float2*)fg::scratch_buffer(c, 4, sizeof(float2) * (size_t)f->samples);
    if (!dh || !tab) return fg::set_error(c, FOCSS_ERR_OOM, "filter scratch");
    cudaStream_t s = c->stream;
    cudaError_t e = cudaMemcpyAsync(dh, re.data(), sizeof(double) * h_len, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dh + h_len, im.data(), sizeof(double) * h_len, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) FG_LAUNCH(fg::zero_pad_kernel<<<fg::grid_for(f->samples, 256), 256, 0, s>>>(dh, dh + h_len, h_len, f->samples, nullptr, 1.0, tab));
    if (e == cudaSuccess) e = cudaGetLastError();
    st = fg::cuda_check(c, e, "filter response");
    if (st == FOCSS_OK) st = fg::fft_forward_transposed(c, tab, f->samples, 1, 1.0f);
    if (st == FOCSS_OK) st = fg::apply_filter(c, f->d, f->samples, f->batch * f->modes, tab, 1.0);
    if (st == FOCSS_OK) st = fg::cuda_check(c, cudaStreamSynchronize(s), "filter sync");  // host vectors
    return st;
}

FOCSS_API focss_status focss_rrc_shaping(focss_ctx* c, const focss_field* symbols, int osf, double roll_off,
                                         double gain, focss_field* out) {
    // modulation.cpp:86-90: upsample(osf).filter_inplace(rrc(n, osf, roll_off)) * (sqrt(gain) * osf)
    if (!c || !symbols || !out || osf <= 0) return FOCSS_ERR_INVALID_ARG;
    focss_status st = focss_upsample(c, symbols, osf, out);
    if (st != FOCSS_OK) return st;
    const float2* H = nullptr;
    st = fg::rrc_table(c, out->samples, symbols->samples, osf, roll_off, &H);
    if (st != FOCSS_OK) return st;
    return fg::apply_filter(c, out->d, out->samples, out->batch * out->modes, H, std::sqrt(gain) * osf);
}

FOCSS_API focss_status focss_rrc_sampling(focss_ctx* c, const focss_field* signal, int osf, double roll_off,
                                          double gain, focss_field* out) {
    // modulation.cpp:92-96: signal.filter(rrc(samples/osf, osf, roll_off)).downsample(osf) * sqrt(gain)
    if (!c || !signal || !out || osf <= 0 || signal->samples % osf) return FOCSS_ERR_INVALID_ARG;
    if (out->modes != signal->modes || out->batch != signal->batch || out->samples != signal->samples / osf)
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "rrc_sampling: output shape");
    float2* tmp = (float2*)fg::scratch_buffer(c, 2, sizeof(float2) * signal->n());
    if (!tmp) return fg::set_error(c, FOCSS_ERR_OOM, "rrc_sampling scratch");
    cudaError_t e = cudaMemcpyAsync(tmp, signal->d, sizeof(float2) * signal->n(), cudaMemcpyDeviceToDevice, c->stream);
    if (e != cudaSuccess) return fg::cuda_check(c, e, "rrc_sampling copy");
    const float2* H = nullptr;
    focss_status st = fg::rrc_table(c, signal->samples, signal->samples / osf, osf, roll_off, &H);
    if (st == FOCSS_OK) st = fg::apply_filter(c, tmp, signal->samples, signal->batch * signal->modes, H, 1.0);
    if (st != FOCSS_OK) return st;
    FG_LAUNCH(fg::downsample_kernel<<<fg::grid_for(out->n(), 256), 256, 0, c->stream>>>(tmp, out->d, out->n(), osf, (float)std::sqrt(gain)));
    return fg::cuda_check(c, cudaGetLastError(), "rrc_sampling");
}

FOCSS_API focss_status focss_frequency_shift(focss_ctx* c, focss_field* f, double frequency) {
    if (!c || !f) return FOCSS_ERR_INVALID_ARG;
    // modulation.cpp:255-264: A(mode, s) *= i_exp(2 pi f dt s)
    const unsigned long long X = fg::turns_fix64_host(frequency * f->dt);
    FG_LAUNCH(fg::freq_shift_kernel<<<fg::grid_for(f->n(), 256), 256, 0, c->stream>>>(f->d, f->samples, f->n(), X));
    return fg::cuda_check(c, cudaGetLastError(), "frequency_shift");
}

FOCSS_API focss_status focss_bandpass(focss_ctx* c, focss_field* f, double frequency) {
    if (!c || !f) return FOCSS_ERR_INVALID_ARG;
    // modulation.cpp:266-277: cut = int(f * duration) + 1; zero bins [cut, N - cut].
    const int cut = (int)(frequency * (f->samples * f->dt)) + 1;
    return fg::spectral_apply(c, f->d, f->samples, f->batch * f->modes, fg::ROW_BANDPASS, nullptr,
                              1.0f / (float)f->samples, cut);
}

FOCSS_API focss_status focss_wdm_select(focss_ctx* c, const focss_field* in, int channel_index,
                                        double channel_bandwidth, focss_field* out) {
    if (!c || !in || !out) return FOCSS_ERR_INVALID_ARG;
    focss_status st = fg::check_same(c, in, out);
    if (st != FOCSS_OK) return st;
    if (out != in) {
        cudaError_t e = cudaMemcpyAsync(out->d, in->d, sizeof(float2) * in->n(), cudaMemcpyDeviceToDevice, c->stream);
        if (e != cudaSuccess) return fg::cuda_check(c, e, "wdm_select copy");
    }
    st = focss_frequency_shift(c, out, -channel_bandwidth * channel_index);
    if (st != FOCSS_OK) return st;
    return focss_bandpass(c, out, 0.5 * channel_bandwidth);
}

FOCSS_API focss_status focss_wdm_mux(focss_ctx* c, const focss_field* ch, double channel_bandwidth,
                                     focss_field* out) {
    if (!c || !ch || !out) return FOCSS_ERR_INVALID_ARG;
    if (out->batch != 1 || out->modes != ch->modes || out->samples != ch->samples)
        return fg::set_error(c, FOCSS_ERR_INVALID_ARG, "wdm_mux: output must be one realization of the channel shape");
    const int n = ch->batch;
    std::vector<unsigned long long> X(n);
    for (int i = 0; i < n; ++i) X[i] = fg::turns_fix64_host((i - n / 2) * channel_bandwidth * ch->dt);
    unsigned long long* dX = (unsigned long long*)fg::scratch_buffer(c, 5, sizeof(unsigned long long) * n);
    if (!dX) return fg::set_error(c, FOCSS_ERR_OOM, "wdm_mux scratch");
    cudaError_t e = cudaMemcpyAsync(dX, X.data(), sizeof(unsigned long long) * n, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) FG_LAUNCH(fg::wdm_mux_kernel<<<fg::grid_for(out->n(), 256), 256, 0, c->stream>>>(ch->d, n, ch->modes, ch->samples, dX, out->d));
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return fg::cuda_check(c, e, "wdm_mux");
}

FOCSS_API focss_status focss_hard_decision(focss_ctx* c, const focss_field* in, focss_field* out) {
    if (!c || !in || !out) return FOCSS_ERR_INVALID_ARG;
    focss_status st = fg::check_same(c, in, out);
    if (st == FOCSS_OK) st = fg::ensure_red(c, (size_t)in->batch);
    if (st == FOCSS_OK) st = fg::power_sums(c, in, c->d_red);
    if (st != FOCSS_OK) return st;
    const size_t per = (size_t)in->modes * in->samples;
    FG_LAUNCH(fg::hard_decision_kernel<<<fg::grid_per_realization(per, in->batch), 256, 0, c->stream>>>(in->d, out->d, in->modes, in->samples, per, c->d_red));
    return fg::cuda_check(c, cudaGetLastError(), "hard_decision");
}

FOCSS_API focss_status focss_soft_decision(focss_ctx* c, const focss_field* in, double uncertainty,
                                           focss_field* out) {
    if (!c || !in || !out || !(uncertainty >= 0)) return FOCSS_ERR_INVALID_ARG;
    focss_status st = fg::check_same(c, in, out);
    if (st == FOCSS_OK) st = fg::ensure_red(c, (size_t)in->batch);
    if (st == FOCSS_OK) st = fg::power_sums(c, in, c->d_red);
    if (st != FOCSS_OK) return st;
    const size_t per = (size_t)in->modes * in->samples;
    FG_LAUNCH(fg::soft_decision_kernel<<<fg::grid_per_realization(per, in->batch), 256, 0, c->stream>>>(in->d, out->d, in->modes, in->samples, per, c->d_red, uncertainty));
    return fg::cuda_check(c, cudaGetLastError(), "soft_decision");
}

FOCSS_API focss_status focss_find_certainty(focss_ctx* c, const focss_field* tx, const focss_field* rx,
                                           double* certainty) {
    if (!c || !tx || !rx || !certainty) return FOCSS_ERR_INVALID_ARG;
    focss_status st = fg::check_same(c, tx, rx);
    if (st == FOCSS_OK) st = fg::ensure_red(c, 2 * (size_t)tx->batch);
    if (st == FOCSS_OK) st = fg::power_sums(c, tx, c->d_red);
    if (st != FOCSS_OK) return st;
    const int B = tx->batch;
    const size_t per = (size_t)tx->modes * tx->samples;
    unsigned long long* dmin = (unsigned long long*)(c->d_red + B);
    std::vector<unsigned long long> inf(B, 0x7FF0000000000000ull);
    cudaError_t e = cudaMemcpyAsync(dmin, inf.data(), sizeof(unsigned long long) * B, cudaMemcpyHostToDevice, c->stream);
    const int gx = std::max(1, std::min(64, (int)((per + 1023) / 1024)));
    if (e == cudaSuccess)
        FG_LAUNCH(fg::certainty_kernel<<<dim3(gx, B), 256, 0, c->stream>>>(tx->d, rx->d, per, c->d_red, dmin));
    if (e == cudaSuccess) e = cudaGetLastError();
    std::vector<double> host(2 * (size_t)B);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host.data(), c->d_red, sizeof(double) * 2 * B, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fg::cuda_check(c, e, "find_certainty");
    for (int b = 0; b < B; ++b) {
        // wdm_scoring.cpp:107-125, same expression order
        const double scale = std::sqrt((double)per) / std::sqrt(host[b]);
        double threshold = 1.0 / std::sqrt(5.0) / scale;
        double d;
        std::memcpy(&d, &host[B + b], sizeof(double));
        if (threshold > d) threshold = d;
        certainty[b] = std::sqrt(5.0) * scale * threshold;
    }
    return FOCSS_OK;
}

FOCSS_API focss_status focss_certainty_decision(focss_ctx* c, const focss_field* in, double certainty,
                                               focss_field* out) {
    if (!c || !in || !out || !(certainty >= 0)) return FOCSS_ERR_INVALID_ARG;
    focss_status st = fg::check_same(c, in, out);
    if (st == FOCSS_OK) st = fg::ensure_red(c, (size_t)in->batch);
    if (st == FOCSS_OK) st = fg::power_sums(c, in, c->d_red);
    if (st != FOCSS_OK) return st;
    const size_t per = (size_t)in->modes * in->samples;
    FG_LAUNCH(fg::certainty_decision_kernel<<<fg::grid_per_realization(per, in->batch), 256, 0, c->stream>>>(in->d, out->d, per, c->d_red, certainty));
    return fg::cuda_check(c, cudaGetLastError(), "certainty_decision");
}

FOCSS_API focss_status focss_hd_codes(focss_ctx* c, const focss_field* in, int32_t* codes) {
    if (!c || !in || !codes) return FOCSS_ERR_INVALID_ARG;
    focss_status st = fg::ensure_red(c, (size_t)in->batch);
    if (st == FOCSS_OK) st = fg::power_sums(c, in, c->d_red);
    if (st != FOCSS_OK) return st;
    int32_t* d = (int32_t*)fg::scratch_buffer(c, 1, sizeof(int32_t) * in->n());
    if (!d) return fg::set_error(c, FOCSS_ERR_OOM, "hd_codes scratch");
    const size_t per = (size_t)in->modes * in->samples;
    FG_LAUNCH(fg::hd_codes_kernel<<<fg::grid_per_realization(per, in->batch), 256, 0, c->stream>>>(in->d, d, in->modes, in->samples, per, c->d_red));
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(codes, d, sizeof(int32_t) * in->n(), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return fg::cuda_check(c, e, "hd_codes");
}

FOCSS_API focss_status focss_error_counts(focss_ctx* c, const focss_field* tx, const focss_field* rx, int cut,
                                          uint64_t* bit_errors, uint64_t* symbol_errors) {
    if (!c || !tx || !rx) return FOCSS_ERR_INVALID_ARG;
    focss_status st = fg::check_same(c, tx, rx);
    if (st != FOCSS_OK) return st;
    cut = fg::clamp_cut(cut);
    const int B = tx->batch;
    st = fg::ensure_red(c, 3 * (size_t)B);
    if (st == FOCSS_OK) st = fg::power_sums(c, tx, c->d_red);
    if (st != FOCSS_OK) return st;
    unsigned long long* cnt = (unsigned long long*)(c->d_red + B);
    cudaStream_t s = c->stream;
    cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * 2 * B, s);
    const int gx = std::max(1, std::min(64, (int)(((size_t)tx->modes * tx->samples + 1023) / 1024)));
    if (e == cudaSuccess) FG_LAUNCH(fg::error_count_kernel<<<dim3(gx, B), 256, 0, s>>>(tx->d, rx->d, tx->modes, tx->samples, cut, c->d_red, cnt));
    if (e == cudaSuccess) e = cudaGetLastError();
    std::vector<unsigned long long> h(2 * (size_t)B);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), cnt, sizeof(unsigned long long) * 2 * B, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fg::cuda_check(c, e, "error_counts");
    for (int b = 0; b < B; ++b) {
        if (bit_errors) bit_errors[b] = h[2 * b];
        if (symbol_errors) symbol_errors[b] = h[2 * b + 1];
    }
    return FOCSS_OK;
}

FOCSS_API focss_status focss_bit_error_rate(focss_ctx* c, const focss_field* tx, const focss_field* rx, int cut,
                                            double* ber) {
    if (!ber) return FOCSS_ERR_INVALID_ARG;
    std::vector<uint64_t> be(tx ? tx->batch : 0);
    focss_status st = focss_error_counts(c, tx, rx, cut, be.data(), nullptr);
    if (st != FOCSS_OK) return st;
    cut = fg::clamp_cut(cut);
    const double den = 4.0 * tx->modes * tx->samples - 8.0 * cut;  // modulation.cpp:200-201
    for (int b = 0; b < tx->batch; ++b) ber[b] = (double)be[b] / den;
    return FOCSS_OK;
}

FOCSS_API focss_status focss_symbol_error_rate(focss_ctx* c, const focss_field* tx, const focss_field* rx,
                                               int cut, double* ser) {
    if (!ser) return FOCSS_ERR_INVALID_ARG;
    std::vector<uint64_t> se(tx ? tx->batch : 0);
    focss_status st = focss_error_counts(c, tx, rx, cut, nullptr, se.data());
    if (st != FOCSS_OK) return st;
    cut = fg::clamp_cut(cut);
    const double den = (double)tx->modes * tx->samples - (double)tx->modes * cut;  // modulation.cpp:221-222
    for (int b = 0; b < tx->batch; ++b) ser[b] = (double)se[b] / den;
    return FOCSS_OK;
}

FOCSS_API focss_status focss_q2_factor(focss_ctx* c, const focss_field* tx, const focss_field* rx, int cut,
                                       double* q2) {
    if (!c || !tx || !rx || !q2) return FOCSS_ERR_INVALID_ARG;
    focss_status st = fg::check_same(c, tx, rx);
    if (st != FOCSS_OK) return st;
    cut = fg::clamp_cut(cut);
    std::vector<double> h;
    st = fg::sums_for(c, tx, rx, cut, tx->samples - cut, h);
    if (st != FOCSS_OK) return st;
    for (int b = 0; b < tx->batch; ++b) q2[b] = -10 * std::log10(h[8 * b + 2] / h[8 * b + 0]);
    return FOCSS_OK;
}

FOCSS_API focss_status focss_pse_estimate(focss_ctx* c, const focss_field* desired, const focss_field* actual,
                                          int angle_steps, double* angle) {
    if (!c || !desired || !actual || !angle || angle_steps <= 0) return FOCSS_ERR_INVALID_ARG;
    focss_status st = fg::check_same(c, desired, actual);
    if (st != FOCSS_OK) return st;
    const int B = desired->batch;
    st = fg::ensure_red(c, 9 * (size_t)B);
    if (st != FOCSS_OK) return st;
    cudaStream_t s = c->stream;
    cudaError_t e = cudaMemsetAsync(c->d_red, 0, sizeof(double) * 8 * B, s);
    const int gx = std::max(1, std::min(64, (int)(((size_t)desired->modes * desired->samples + 1023) / 1024)));
    if (e == cudaSuccess) FG_LAUNCH(fg::pair_sums_kernel<<<dim3(gx, B), 256, 0, s>>>(desired->d, actual->d, desired->modes, desired->samples, 0, desired->samples, c->d_red));
    if (e == cudaSuccess) FG_LAUNCH(fg::pse_argmax_kernel<<<B, 256, 0, s>>>(c->d_red, angle_steps, c->d_red + 8 * B));
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(angle, c->d_red + 8 * B, sizeof(double) * B, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return fg::cuda_check(c, e, "pse_estimate");
}

FOCSS_API focss_status focss_scalar_estimate(focss_ctx* c, const focss_field* desired, const focss_field* actual,
                                             double* scalar) {
    if (!c || !desired || !actual || !scalar) return FOCSS_ERR_INVALID_ARG;
    focss_status st = fg::check_same(c, desired, actual);
    if (st != FOCSS_OK) return st;
    std::vector<double> h;
    // t = actual, r = desired: sum |actual|^2 and sum conj(actual) desired.
    st = fg::sums_for(c, actual, desired, 0, actual->samples, h);
    if (st != FOCSS_OK) return st;
    for (int b = 0; b < actual->batch; ++b) {
        scalar[2 * b] = h[8 * b + 5] / h[8 * b + 0];
        scalar[2 * b + 1] = h[8 * b + 6] / h[8 * b + 0];
    }
    return FOCSS_OK;
}

static focss_status scale_each(focss_ctx* c, focss_field* f, const std::vector<float2>& s) {
    float2* d = (float2*)fg::scratch_buffer(c, 6, sizeof(float2) * f->batch);
    if (!d) return fg::set_error(c, FOCSS_ERR_OOM, "scale scratch");
    cudaError_t e = cudaMemcpyAsync(d, s.data(), sizeof(float2) * f->batch, cudaMemcpyHostToDevice, c->stream);
    const size_t per = (size_t)f->modes * f->samples;
    if (e == cudaSuccess) FG_LAUNCH(fg::scale_each_kernel<<<fg::grid_for(f->n(), 256), 256, 0, c->stream>>>(f->d, per, f->n(), d));
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return fg::cuda_check(c, e, "scale_each");
}

FOCSS_API focss_status focss_field_rotate(focss_ctx* c, focss_field* f, const double* angle) {
    if (!c || !f || !angle) return FOCSS_ERR_INVALID_ARG;
    std::vector<float2> s(f->batch);
    for (int b = 0; b < f->batch; ++b) s[b] = make_float2((float)std::cos(angle[b]), (float)std::sin(angle[b]));
    return scale_each(c, f, s);
}

FOCSS_API focss_status focss_field_scale_each(focss_ctx* c, focss_field* f, const double* scalar) {
    if (!c || !f || !scalar) return FOCSS_ERR_INVALID_ARG;
    std::vector<float2> s(f->batch);
    for (int b = 0; b < f->batch; ++b) s[b] = make_float2((float)scalar[2 * b], (float)scalar[2 * b + 1]);
    return scale_each(c, f, s);
}

}  // extern "C"
