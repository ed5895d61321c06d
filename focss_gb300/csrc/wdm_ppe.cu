// wdm_ppe.cu -- WdmPPE (src/focss/equalizer/wdm_sino.cpp): the dual-
// polarization WDM perturbation equalizer with SPM and XPM triplets.
//
// Input realizations are 6-row matrices (rows channel * 2 + polarization: left
// neighbour 0-1, centre 2-3, right neighbour 4-5); outputs are the centre
// channel's two polarizations.
//
//   spm(pol, k) = sum_{|m|+|n|<=c} C(m, n) T(pol, k, m, n),       k in [c, N-c)
//   xpm(pol, k) = sum_{|m|+|n|<=d} D(m, n) (T1(pol, k, m, n) + T3(pol, k, m, -n)),
//                                                                  k in [d, N-d)
// (wdm_sino.cpp:256-295).  SPM is the single-channel triplet sum on the
// centre rows (triplet.cu, read in place through the row stride).  XPM runs
// here: one CTA per tile of XT outputs, the six rows of the tile plus a
// d-sample halo on each side staged in shared memory, one thread per output
// computing both polarizations.  Per m the neighbour products
//   L_pq(j) = A_p(j) conj(A_q(j + m))   (left, j = k + n)
//   R_pq(j) = A_p(j) conj(A_q(j + m))   (right, j = k - n)
// are weighted by D(m, n) and summed over n into four sums, which then
// multiply A_2(k+m) and A_3(k+m) (T1/T3 of wdm_sino.cpp:166-200 regrouped).
// The same kernel applies the final combination: noise = spm + xpm, then
// equalize (rx - noise) / a (wdm_sino.cpp:240-249), model a x + noise
// (:235-238, :251-254) or the noise alone.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace fg {
namespace {

constexpr int XT = 256;  // outputs (threads) per CTA

struct XpmArgs {
    const float2* x;        // xpm input (6 rows), or null
    size_t x_bstride;
    const float2* D;        // (2d+1)^2, D[(d+m)(2d+1) + d+n]
    int d;
    const float2* rx;       // equalize: rx rows rx_row0, rx_row0+1, or null
    size_t rx_bstride;
    int rx_row0;
    const float2* lin;      // model: centre rows of this (6-row) field, or null
    size_t lin_bstride;
    float2 lw, inv_lw;
    int has_spm;            // out already holds the SPM sum
    float2* out;            // batch x 2 x N
    int samples;
};

__device__ __forceinline__ int padx(int j) { return j + (j >> 5); }

__global__ void __launch_bounds__(XT) wdm_xpm_kernel(const XpmArgs a) {
    extern __shared__ float2 sh[];
    const int N = a.samples, d = a.d;
    const int b = blockIdx.y;
    const int k0 = blockIdx.x * XT;
    const int k = k0 + threadIdx.x;
    float2 x0 = make_float2(0.f, 0.f), x1 = make_float2(0.f, 0.f);
    if (a.x && d >= 0) {
        const int halo = d;  // every offset m, n, m + n, -n, m - n is within [-d, d]
        const int len = XT + 2 * halo;
        const int stride = padx(len) + 1;
        const float2* src = a.x + (size_t)b * a.x_bstride;
        for (int r = 0; r < 6; ++r)
            for (int i = threadIdx.x; i < len; i += XT) {
                const int s = k0 - halo + i;
                sh[r * stride + padx(i)] = (s >= 0 && s < N) ? src[(size_t)r * N + s] : make_float2(0.f, 0.f);
            }
        __syncthreads();
        if (k >= d && k < N - d) {
            const int kl = threadIdx.x + halo;  // tile index of sample k
#define A(r, j) sh[(r) * stride + padx(kl + (j))]
            const int w = 2 * d + 1;
            for (int m = -d; m <= d; ++m) {
                const int nb = d - abs(m);
                float2 sa0 = make_float2(0.f, 0.f), sb0 = sa0, sa1 = sa0, sb1 = sa0;
                for (int n = -nb; n <= nb; ++n) {
                    const float2 c = __ldg(a.D + (size_t)(d + m) * w + d + n);
                    // left neighbour at j = k + n, right neighbour at j = k - n
                    const float2 l0 = A(0, n), l1 = A(1, n), l0m = A(0, m + n), l1m = A(1, m + n);
                    const float2 r0 = A(4, -n), r1 = A(5, -n), r0m = A(4, m - n), r1m = A(5, m - n);
                    const float2 q00 = cadd(cmulc(l0, l0m), cmulc(r0, r0m));
                    const float2 q11 = cadd(cmulc(l1, l1m), cmulc(r1, r1m));
                    const float2 q01 = cadd(cmulc(l0, l1m), cmulc(r0, r1m));
                    const float2 q10 = cadd(cmulc(l1, l0m), cmulc(r1, r0m));
                    // pol 0: A2 (2 q00 + q11) + A3 q01; pol 1: A3 (2 q11 + q00) + A2 q10
                    sa0 = cadd(sa0, cmul(c, cadd(cscale(q00, 2.f), q11)));
                    sb0 = cadd(sb0, cmul(c, q01));
                    sa1 = cadd(sa1, cmul(c, cadd(cscale(q11, 2.f), q00)));
                    sb1 = cadd(sb1, cmul(c, q10));
                }
                const float2 a2 = A(2, m), a3 = A(3, m);
                x0 = cadd(x0, cadd(cmul(a2, sa0), cmul(a3, sb0)));
                x1 = cadd(x1, cadd(cmul(a3, sa1), cmul(a2, sb1)));
            }
#undef A
        }
    }
    if (k >= N) return;
    float2* out = a.out + (size_t)b * 2 * N;
    float2 n0 = x0, n1 = x1;
    if (a.has_spm) {
        n0 = cadd(n0, out[k]);
        n1 = cadd(n1, out[(size_t)N + k]);
    }
    if (a.rx) {
        const float2* r = a.rx + (size_t)b * a.rx_bstride + (size_t)a.rx_row0 * N;
        n0 = cmul(csub(r[k], n0), a.inv_lw);
        n1 = cmul(csub(r[(size_t)N + k], n1), a.inv_lw);
    } else if (a.lin) {
        const float2* l = a.lin + (size_t)b * a.lin_bstride + 2 * (size_t)N;
        n0 = cadd(n0, cmul(a.lw, l[k]));
        n1 = cadd(n1, cmul(a.lw, l[(size_t)N + k]));
    }
    out[k] = n0;
    out[(size_t)N + k] = n1;
}

}  // namespace
}  // namespace fg

using fg::Ctx;
using fg::Field;

extern "C" {

FOCSS_API focss_status focss_wdm_ppe_apply(focss_ctx* c, const focss_field* spm_in, const focss_field* xpm_in,
                                           const focss_field* rx, const focss_field* lin_in, int c_radius,
                                           const double* C, int d_radius, const double* D, double lw_re,
                                           double lw_im, focss_field* out) {
    using namespace fg;
    if (!c || !out || (spm_in && !C) || (xpm_in && !D)) return FOCSS_ERR_INVALID_ARG;
    const int N = out->samples, B = out->batch;
    if (out->modes != 2) return set_error(c, FOCSS_ERR_INVALID_ARG, "wdm_ppe_apply: out must have 2 rows");
    auto six = [&](const focss_field* f) { return !f || (f->modes == 6 && f->samples == N && f->batch == B && f != out); };
    if (!six(spm_in) || !six(xpm_in) || !six(lin_in))
        return set_error(c, FOCSS_ERR_INVALID_ARG, "wdm_ppe_apply: inputs must be 6-row fields of the output's length and batch");
    if (rx && ((rx->modes != 6 && rx->modes != 2) || rx->samples != N || rx->batch != B))
        return set_error(c, FOCSS_ERR_INVALID_ARG, "wdm_ppe_apply: rx must have 6 or 2 rows of the output's shape");
    if ((spm_in && (c_radius < 0 || N <= 2 * c_radius)) || (xpm_in && (d_radius < 0 || N <= 2 * d_radius)))
        return set_error(c, FOCSS_ERR_INVALID_ARG, "wdm_ppe_apply: radius vs field length");
    if (xpm_in && d_radius > 96) return set_error(c, FOCSS_ERR_UNSUPPORTED, "wdm_ppe_apply: d_radius <= 96");
    const double den = lw_re * lw_re + lw_im * lw_im;
    if (rx && !(den > 0)) return set_error(c, FOCSS_ERR_INVALID_ARG, "wdm_ppe_apply: linear weight is zero");
    cudaStream_t s = c->stream;
    focss_status st = FOCSS_OK;
    if (spm_in) {
        // the diamond |m| + |n| <= c of C (wdm_sino.cpp:261-268)
        std::vector<int32_t> m, n;
        std::vector<double> cf;
        const int w = 2 * c_radius + 1;
        for (int nn = -c_radius; nn <= c_radius; ++nn) {
            const int bd = c_radius - std::abs(nn);
            for (int mm = -bd; mm <= bd; ++mm) {
                const double* e = C + 2 * ((size_t)(c_radius + mm) * w + c_radius + nn);
                m.push_back(mm);
                n.push_back(nn);
                cf.push_back(e[0]);
                cf.push_back(e[1]);
            }
        }
        st = run_triplet_rows(c, spm_in->d + 2 * (size_t)N, (size_t)6 * N, 2, N, B, nullptr, c_radius, (int)m.size(),
                              m.data(), n.data(), cf.data(), make_float2(1.f, 0.f), out->d);
        if (st != FOCSS_OK) return st;
    }
    XpmArgs a{};
    a.samples = N;
    a.out = out->d;
    a.has_spm = spm_in != nullptr;
    a.d = xpm_in ? d_radius : -1;
    std::vector<float2> hD;
    if (xpm_in) {
        const int w = 2 * d_radius + 1;
        hD.resize((size_t)w * w);
        for (size_t i = 0; i < hD.size(); ++i) hD[i] = make_float2((float)D[2 * i], (float)D[2 * i + 1]);
        float2* dD = (float2*)scratch_buffer(c, 8, sizeof(float2) * hD.size());
        if (!dD) return set_error(c, FOCSS_ERR_OOM, "wdm_ppe scratch");
        cudaError_t e = cudaMemcpyAsync(dD, hD.data(), sizeof(float2) * hD.size(), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return cuda_check(c, e, "wdm_ppe upload");
        a.x = xpm_in->d;
        a.x_bstride = (size_t)6 * N;
        a.D = dD;
    }
    if (rx) {
        a.rx = rx->d;
        a.rx_bstride = (size_t)rx->modes * N;
        a.rx_row0 = rx->modes == 6 ? 2 : 0;
        a.inv_lw = make_float2((float)(lw_re / den), (float)(-lw_im / den));
    } else if (lin_in) {
        a.lin = lin_in->d;
        a.lin_bstride = (size_t)6 * N;
        a.lw = make_float2((float)lw_re, (float)lw_im);
    }
    size_t smem = 0;
    if (xpm_in) {
        const int len = XT + 2 * d_radius;
        smem = sizeof(float2) * 6 * (size_t)(len + (len >> 5) + 1);
        cudaFuncSetAttribute(wdm_xpm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    dim3 grid((N + XT - 1) / XT, B);
    wdm_xpm_kernel<<<grid, XT, smem, s>>>(a);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // host D table goes out of scope
    return cuda_check(c, e, "wdm_ppe_apply");
}

}  // extern "C"
