// sino_fit.cu -- normal equations of the perturbation-equalizer fit on the GPU.
//
// SINO::train (src/focss/equalizer/sino.cpp:42-159) builds, per received
// sample k in [R, N-R) of every mode, the symmetry-reduced triplet features
//   f_(m,n)[k] = term(m,n) [+ term(n,m)] [+ term(-m,-n)] [+ term(-n,-m)],
//   term(m,n)[k] = A[k+m] sum_p A_p[k+n] conj(A_p[k+m+n])      (sino.cpp:161-171)
// for |m| <= R/2, |m| <= n <= R-|m| (plus the transmitted sample itself for the
// ORDINARY type), z-scores every feature (mean, standard deviation over the
// samples, normalized by the sample count) and solves the least-squares
// problem for the centred responses.  Here the features, their statistics and
// the Gram matrix [Z y]^H [Z y] of the z-scored features with the centred
// responses appended as one more column are formed on the device; the
// (2R+1)^2/2-sized Hermitian system is then solved by the caller in FP64
// (normal equations: the same solution as the reference's least squares for a
// full-rank design).  WdmPPE::train (src/focss/equalizer/wdm_sino.cpp:28-142)
// is the same pipeline on the centre channel of a 3-channel dual-polarization
// matrix with the XPM triplets of the neighbours as further features.
// The Gram product is a tiled complex kernel on the CUDA
// cores (64 x 64 output tiles, 4 x 4 complex outputs per thread, the samples
// split over the grid's z dimension) reading the FP32 features, summing runs
// of 16 samples in FP32 and accumulating those sums as double-float pairs
// (~48 bits, converted to FP64 once per CTA).  The residual
// entry points rebuild the same design and return Z^H (y - Z x) in FP64, so
// the caller can refine its solve to the FP64 normal-equations solution.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace fg {
namespace {

constexpr int GT = 64;  // Gram tile (features)
inline int grid_for_(size_t n) {
    const size_t g = (n + 255) / 256;
    return (int)std::min<size_t>(g ? g : 1, (size_t)sm_count() * 32);
}
constexpr int GK = 16;  // samples per shared-memory chunk
constexpr int kFlush = 1;  // chunks summed in FP32 before an FP64 accumulation (16 samples; 64 measurably loses accuracy)

struct Feature {
    int m, n, kind;  // kind: 0 = (0,0), 1 = m == n, 2 = m == -n, 3 = general, 4 = transmitted sample
};

// term(m, n)[k] over the modes of one realization (a: modes x N, mode-major).
__device__ __forceinline__ float2 term(const float2* __restrict__ a, int modes, int N, int mode, int k, int m, int n) {
    float2 t = make_float2(0.f, 0.f);
    for (int p = 0; p < modes; ++p) t = cadd(t, cmulc(a[(size_t)p * N + k + n], a[(size_t)p * N + k + m + n]));
    return cmul(a[(size_t)mode * N + k + m], t);
}

// Z[f][i] (feature-major, row stride kp) for sample i = mode * nspm + (k - R).
__global__ void features_kernel(const float2* __restrict__ tx, int modes, int N, int R, const Feature* __restrict__ fs,
                                int nf, float2* __restrict__ Z, size_t kp) {
    const int nspm = N - 2 * R;
    const size_t ns = (size_t)modes * nspm;
    const int f = blockIdx.y;
    const Feature F = fs[f];
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ns; i += (size_t)gridDim.x * blockDim.x) {
        const int mode = (int)(i / nspm), k = (int)(i % nspm) + R;
        float2 v;
        if (F.kind == 4) {
            v = tx[(size_t)mode * N + k];
        } else {
            v = term(tx, modes, N, mode, k, F.m, F.n);
            if (F.kind == 1) v = cadd(v, term(tx, modes, N, mode, k, -F.m, -F.n));
            if (F.kind == 2) v = cadd(v, term(tx, modes, N, mode, k, F.n, F.m));
            if (F.kind == 3) {
                v = cadd(v, term(tx, modes, N, mode, k, F.n, F.m));
                v = cadd(v, term(tx, modes, N, mode, k, -F.m, -F.n));
                v = cadd(v, term(tx, modes, N, mode, k, -F.n, -F.m));
            }
        }
        Z[(size_t)f * kp + i] = v;
    }
}

// Responses (column nf): rx[k] (ORDINARY, HOMOGENEOUS) or rx[k] - lw tx[k] (FIXED).
__global__ void responses_kernel(const float2* __restrict__ tx, const float2* __restrict__ rx, int modes, int N, int R,
                                 float2 lw, int fixed, float2* __restrict__ y) {
    const int nspm = N - 2 * R;
    const size_t ns = (size_t)modes * nspm;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ns; i += (size_t)gridDim.x * blockDim.x) {
        const int mode = (int)(i / nspm), k = (int)(i % nspm) + R;
        float2 v = rx[(size_t)mode * N + k];
        if (fixed) v = csub(v, cmul(tx[(size_t)mode * N + k], lw));
        y[i] = v;
    }
}

// WdmPPE (src/focss/equalizer/wdm_sino.cpp:42-82) on a 6-row realization
// (rows channel * 2 + polarization: left neighbour 0-1, centre 2-3, right
// neighbour 4-5).  T1 (neighbour rows r0, r1 = 0, 1) and T3 (4, 5) of
// wdm_sino.cpp:166-200 for polarization `pol`:
//   A_c(k+m) [2 A_r0(k+n) A_r0*(k+m+n) + A_r1(k+n) A_r1*(k+m+n)] + A_o(k+m) A_r0(k+n) A_r1*(k+m+n)
// with (c, o, r0, r1) = (2, 3, r0, r1) for pol 0 and (3, 2, r1, r0) for pol 1.
__device__ __forceinline__ float2 t13(const float2* __restrict__ a, int N, int pol, int k, int m, int n, int r0,
                                      int r1) {
    const int c = 2 + pol, o = 3 - pol;
    const int p = pol ? r1 : r0, q = pol ? r0 : r1;
    const float2 inner = cadd(cscale(cmulc(a[(size_t)p * N + k + n], a[(size_t)p * N + k + m + n]), 2.f),
                              cmulc(a[(size_t)q * N + k + n], a[(size_t)q * N + k + m + n]));
    return cadd(cmul(a[(size_t)c * N + k + m], inner),
                cmul(a[(size_t)o * N + k + m], cmulc(a[(size_t)p * N + k + n], a[(size_t)q * N + k + m + n])));
}

// Z[f][i] for i = pol * nspm + (k - R): kinds 0-3 SPM (the SINO features on
// the centre rows), 4 the transmitted centre sample, 5 XPM T1(m, n) + T3(m, -n).
__global__ void wdm_features_kernel(const float2* __restrict__ tx, int N, int R, const Feature* __restrict__ fs,
                                    int nf, float2* __restrict__ Z, size_t kp) {
    const int nspm = N - 2 * R;
    const size_t ns = 2 * (size_t)nspm;
    const int f = blockIdx.y;
    const Feature F = fs[f];
    const float2* centre = tx + 2 * (size_t)N;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ns; i += (size_t)gridDim.x * blockDim.x) {
        const int pol = (int)(i / nspm), k = (int)(i % nspm) + R;
        float2 v;
        if (F.kind == 4) {
            v = centre[(size_t)pol * N + k];
        } else if (F.kind == 5) {
            v = cadd(t13(tx, N, pol, k, F.m, F.n, 0, 1), t13(tx, N, pol, k, F.m, -F.n, 4, 5));
        } else {
            v = term(centre, 2, N, pol, k, F.m, F.n);
            if (F.kind == 1) v = cadd(v, term(centre, 2, N, pol, k, -F.m, -F.n));
            if (F.kind == 2) v = cadd(v, term(centre, 2, N, pol, k, F.n, F.m));
            if (F.kind == 3) {
                v = cadd(v, term(centre, 2, N, pol, k, F.n, F.m));
                v = cadd(v, term(centre, 2, N, pol, k, -F.m, -F.n));
                v = cadd(v, term(centre, 2, N, pol, k, -F.n, -F.m));
            }
        }
        Z[(size_t)f * kp + i] = v;
    }
}

// Responses of the centre polarizations: rows row0, row0 + 1 of rx.
__global__ void wdm_responses_kernel(const float2* __restrict__ rx, int row0, int N, int R, float2* __restrict__ y) {
    const int nspm = N - 2 * R;
    const size_t ns = 2 * (size_t)nspm;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ns; i += (size_t)gridDim.x * blockDim.x) {
        const int pol = (int)(i / nspm), k = (int)(i % nspm) + R;
        y[i] = rx[(size_t)(row0 + pol) * N + k];
    }
}

// Per column: mean and, for features, the standard deviation (normalized by
// the count), in two kernels so that every column is split over many CTAs.
// column_moments_kernel sums the deviations from the column's first sample K
// (S1 = sum (z - K), S2 = sum |z - K|^2: shifted sums, so a mean large against
// the spread does not cancel), runs of 16 samples per thread in FP32 and the
// runs in FP64; the CTAs of a column (grid.y) meet in FP64 atomics on
// mom[5 f .. 5 f + 2] (zeroed by the caller), and CTA y = 0 stores K in
// mom[5 f + 3 .. 5 f + 4].
constexpr int kMom = 5;
__global__ void column_moments_kernel(const float2* __restrict__ Z, size_t kp, size_t ns, double* __restrict__ mom) {
    __shared__ double red[32];
    const int f = blockIdx.x;
    const float2* col = Z + (size_t)f * kp;
    const float2 K = col[0];
    const size_t per = (ns + gridDim.y - 1) / gridDim.y;
    const size_t i0 = per * blockIdx.y, i1 = i0 + per < ns ? i0 + per : ns;
    double s1r = 0, s1i = 0, s2 = 0;
    float pr = 0.f, pi = 0.f, p2 = 0.f;
    int run = 0;
    // four independent loads per iteration (bytes in flight); a sample past
    // the range reads as K and adds nothing
    for (size_t i = i0 + threadIdx.x; i < i1; i += 4 * (size_t)blockDim.x) {
        float2 z[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const size_t j = i + (size_t)u * blockDim.x;
            z[u] = j < i1 ? col[j] : K;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const float dr = z[u].x - K.x, di = z[u].y - K.y;
            pr += dr;
            pi += di;
            p2 = fmaf(dr, dr, fmaf(di, di, p2));
        }
        if (++run == 4) {  // 16 samples per FP32 run
            s1r += pr;
            s1i += pi;
            s2 += p2;
            pr = pi = p2 = 0.f;
            run = 0;
        }
    }
    s1r += pr;
    s1i += pi;
    s2 += p2;
    s1r = block_sum_d(s1r, red);
    __syncthreads();
    s1i = block_sum_d(s1i, red);
    __syncthreads();
    s2 = block_sum_d(s2, red);
    if (threadIdx.x == 0) {
        double* m = mom + kMom * (size_t)f;
        atomicAdd(m, s1r);
        atomicAdd(m + 1, s1i);
        atomicAdd(m + 2, s2);
        if (blockIdx.y == 0) {
            m[3] = K.x;
            m[4] = K.y;
        }
    }
}

// z-score the features and centre the responses in place:
// mean = K + S1/ns, sd = sqrt(S2/ns - |S1/ns|^2), z <- (z - mean)/sd in FP64
// (the responses, column nf, only centred); CTA (f, 0) stores mean and sd.
__global__ void column_normalize_kernel(float2* __restrict__ Z, size_t kp, size_t ns, int nf,
                                        const double* __restrict__ mom, double* __restrict__ mean,
                                        double* __restrict__ sd) {
    const int f = blockIdx.x;
    const double* m = mom + kMom * (size_t)f;
    const double d1r = m[0] / (double)ns, d1i = m[1] / (double)ns;
    const double mr = m[3] + d1r, mi = m[4] + d1i;
    const double var = m[2] / (double)ns - (d1r * d1r + d1i * d1i);
    const double s = var > 0 ? sqrt(var) : 0.0;
    const double sc = (f < nf && s > 0) ? 1.0 / s : 1.0;
    if (blockIdx.y == 0 && threadIdx.x == 0) {
        mean[2 * f] = mr;
        mean[2 * f + 1] = mi;
        if (f < nf) sd[f] = s;
    }
    float2* col = Z + (size_t)f * kp;
    const size_t per = (ns + gridDim.y - 1) / gridDim.y;
    const size_t i0 = per * blockIdx.y, i1 = i0 + per < ns ? i0 + per : ns;
    for (size_t i = i0 + threadIdx.x; i < i1; i += 4 * (size_t)blockDim.x) {
        float2 z[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const size_t j = i + (size_t)u * blockDim.x;
            if (j < i1) z[u] = col[j];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const size_t j = i + (size_t)u * blockDim.x;
            if (j < i1) col[j] = make_float2((float)((z[u].x - mr) * sc), (float)((z[u].y - mi) * sc));
        }
    }
}

// G[a][b] += sum_i conj(Z[a][i]) Z[b][i] for the upper-triangle tiles (a <= b)
// over this CTA's share of the samples (grid.z splits them; G starts at zero
// and the shares meet in FP64 atomics).  Z is zero-padded to multiples of GT
// features and GK samples.  Each run of kFlush x GK = 16 samples is summed in
// FP32 (products of FP32 features) and the run sums are accumulated as
// double-float pairs hi + lo (Knuth's two-sum, ~48 significant bits) on the
// FP32 pipes: the normal equations square the design's condition number, so
// sums over ~1e5 samples must not run in plain FP32, but GB300's FP64 rate
// is a small fraction of its FP32 rate and FP64 accumulation of the run sums
// held the kernel on the FP64 pipe.  The pairs go to FP64 once, at the end.
__device__ __forceinline__ void df_acc(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float bv = s - hi;
    lo += (hi - (s - bv)) + (x - bv);
    hi = s;
}

__global__ void __launch_bounds__(256, 2) gram_kernel(const float2* __restrict__ Z, size_t kp, int nfp,
                                                   double2* __restrict__ G) {
    const int bi = blockIdx.y, bj = blockIdx.x;
    if (bi > bj) return;
    __shared__ float2 As[GK][GT + 1];
    __shared__ float2 Bs[GK][GT + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    float4 acc[4][4];  // {re_hi, re_lo, im_hi, im_lo}
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = make_float4(0.f, 0.f, 0.f, 0.f);
    const float2* Za = Z + (size_t)bi * GT * kp;
    const float2* Zb = Z + (size_t)bj * GT * kp;
    const size_t chunks = kp / GK;
    const size_t c0 = chunks * blockIdx.z / gridDim.z, c1 = chunks * (blockIdx.z + 1) / gridDim.z;
    float2 part[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) part[r][c] = make_float2(0.f, 0.f);
    for (size_t k0 = c0 * GK, ci = 0; k0 < c1 * GK; k0 += GK, ++ci) {
        // 64 features x 16 samples per operand: 4 loads per thread, samples fastest
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = threadIdx.x + 256 * q;
            const int row = e / GK, kk = e % GK;
            As[kk][row] = Za[(size_t)row * kp + k0 + kk];
            Bs[kk][row] = Zb[(size_t)row * kp + k0 + kk];
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; ++kk) {
            float2 av[4], bv[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) av[r] = As[kk][ty * 4 + r];
#pragma unroll
            for (int c = 0; c < 4; ++c) bv[c] = Bs[kk][tx + 16 * c];  // consecutive lanes, consecutive words
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    // conj(a) * b
                    part[r][c].x = fmaf(av[r].x, bv[c].x, fmaf(av[r].y, bv[c].y, part[r][c].x));
                    part[r][c].y = fmaf(av[r].x, bv[c].y, fmaf(-av[r].y, bv[c].x, part[r][c].y));
                }
        }
        if ((ci & (kFlush - 1)) == kFlush - 1 || k0 + GK >= c1 * GK) {
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    df_acc(acc[r][c].x, acc[r][c].y, part[r][c].x);
                    df_acc(acc[r][c].z, acc[r][c].w, part[r][c].y);
                    part[r][c] = make_float2(0.f, 0.f);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            double2* g = G + (size_t)(bi * GT + ty * 4 + r) * nfp + bj * GT + tx + 16 * c;
            atomicAdd(&g->x, (double)acc[r][c].x + (double)acc[r][c].y);
            atomicAdd(&g->y, (double)acc[r][c].z + (double)acc[r][c].w);
        }
}

// Residual of the normal equations for iterative refinement, in FP64 on the
// z-scored design: v = y - Z x (one thread per sample), then r = Z^H v (one
// CTA per feature).  Z and y are the FP32 columns the Gram kernel reads, so
// a refined solution solves the normal equations of exactly that design to
// FP64 accuracy however the Gram matrix was rounded.
__global__ void design_apply_kernel(const float2* __restrict__ Z, size_t kp, size_t ns, int nf,
                                    const double2* __restrict__ x, double2* __restrict__ v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ns; i += (size_t)gridDim.x * blockDim.x) {
        const float2 y = Z[(size_t)nf * kp + i];
        double re = y.x, im = y.y;
#pragma unroll 4
        for (int f = 0; f < nf; ++f) {
            const float2 z = Z[(size_t)f * kp + i];
            const double2 xf = __ldg(x + f);
            re = fma(-(double)z.x, xf.x, fma((double)z.y, xf.y, re));
            im = fma(-(double)z.x, xf.y, fma(-(double)z.y, xf.x, im));
        }
        v[i] = make_double2(re, im);
    }
}

__global__ void design_adjoint_kernel(const float2* __restrict__ Z, size_t kp, size_t ns,
                                      const double2* __restrict__ v, double2* __restrict__ r) {
    __shared__ double red[32];
    const int f = blockIdx.x;
    const float2* col = Z + (size_t)f * kp;
    const size_t per = (ns + gridDim.y - 1) / gridDim.y;
    const size_t i0 = per * blockIdx.y, i1 = i0 + per < ns ? i0 + per : ns;
    double re = 0, im = 0;
    for (size_t i = i0 + threadIdx.x; i < i1; i += 4 * (size_t)blockDim.x) {
        float2 z[4];
        double2 vi[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const size_t j = i + (size_t)u * blockDim.x;
            z[u] = j < i1 ? col[j] : make_float2(0.f, 0.f);
            vi[u] = j < i1 ? v[j] : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            re = fma((double)z[u].x, vi[u].x, fma((double)z[u].y, vi[u].y, re));
            im = fma((double)z[u].x, vi[u].y, fma(-(double)z[u].y, vi[u].x, im));
        }
    }
    re = block_sum_d(re, red);
    __syncthreads();
    im = block_sum_d(im, red);
    if (threadIdx.x == 0) {  // r is zeroed by the caller; the CTAs of a column meet here
        atomicAdd(&r[f].x, re);
        atomicAdd(&r[f].y, im);
    }
}

// SPM feature list in the order of sino.cpp:70-100 / wdm_sino.cpp:47-71.
void spm_features(int R, std::vector<Feature>& fs) {
    const int mb = R / 2;
    for (int m = -mb; m <= mb; ++m)
        for (int n = std::abs(m); n <= R - std::abs(m); ++n) {
            const int kind = (m == 0 && n == 0) ? 0 : (m == n) ? 1 : (m == -n) ? 2 : 3;
            fs.push_back({m, n, kind});
        }
}

// Device buffers of one fit: Z holds nf feature columns and the responses
// (column nf), each kp samples long (zero-padded), nfp columns in all.
struct FitBuffers {
    float2* Z = nullptr;
    Feature* fs = nullptr;
    double2* G = nullptr;
    double* stat = nullptr;
    double* mom = nullptr;
    ~FitBuffers() {
        cudaFree(Z);
        cudaFree(fs);
        cudaFree(G);
        cudaFree(stat);
        cudaFree(mom);
    }
};

cudaError_t fit_alloc(FitBuffers& b, const std::vector<Feature>& fs, size_t kp, int nfp, cudaStream_t s) {
    const int nf = (int)fs.size();
    cudaError_t e = cudaMalloc(&b.Z, sizeof(float2) * (size_t)nfp * kp);
    if (e == cudaSuccess) e = cudaMalloc(&b.fs, sizeof(Feature) * std::max(nf, 1));
    if (e == cudaSuccess) e = cudaMalloc(&b.G, sizeof(double2) * (size_t)nfp * nfp);
    if (e == cudaSuccess) e = cudaMalloc(&b.stat, sizeof(double) * (3 * (size_t)nfp + 2));
    if (e == cudaSuccess) e = cudaMalloc(&b.mom, sizeof(double) * kMom * (size_t)nfp);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.Z, 0, sizeof(float2) * (size_t)nfp * kp, s);
    if (e == cudaSuccess && nf) e = cudaMemcpyAsync(b.fs, fs.data(), sizeof(Feature) * nf, cudaMemcpyHostToDevice, s);
    return e;
}

// z-score the feature columns, centre the responses, form the Gram matrix and
// copy gram ((nf+1)^2 complex128, upper triangle), mean (nf+1 complex128) and
// sd (nf doubles) to the host.
// z-scores the feature columns and centres the responses in place.
// Splits each of `cols` columns of ns samples over enough CTAs to give the
// GPU about 8 CTAs of 256 threads per SM, at least 4096 samples per CTA.
inline unsigned column_split(int cols, size_t ns) {
    const size_t by_work = (ns + 4095) / 4096, by_fill = ((size_t)sm_count() * 8 + cols - 1) / (size_t)cols;
    const size_t y = std::min(by_work, by_fill);
    return (unsigned)std::max<size_t>(1, std::min<size_t>(y, 65535));
}

cudaError_t fit_stats(FitBuffers& b, size_t kp, size_t ns, int nf, int nfp, cudaStream_t s) {
    const dim3 grid(nf + 1, column_split(nf + 1, ns));
    cudaError_t e = cudaMemsetAsync(b.mom, 0, sizeof(double) * kMom * (size_t)(nf + 1), s);
    if (e != cudaSuccess) return e;
    column_moments_kernel<<<grid, 256, 0, s>>>(b.Z, kp, ns, b.mom);
    count_launch();
    column_normalize_kernel<<<grid, 256, 0, s>>>(b.Z, kp, ns, nf, b.mom, b.stat, b.stat + 2 * (size_t)nfp);
    count_launch();
    return cudaGetLastError();
}

// r = Z^H (y - Z x) for the prepared design (x, r: nf complex128 on the host).
cudaError_t fit_residual(FitBuffers& b, size_t kp, size_t ns, int nf, const double* x, double* r, cudaStream_t s) {
    double2 *dx = nullptr, *dv = nullptr, *dr = nullptr;
    cudaError_t e = cudaMalloc(&dx, sizeof(double2) * nf);
    if (e == cudaSuccess) e = cudaMalloc(&dv, sizeof(double2) * ns);
    if (e == cudaSuccess) e = cudaMalloc(&dr, sizeof(double2) * nf);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, sizeof(double2) * nf, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(dr, 0, sizeof(double2) * nf, s);
    if (e == cudaSuccess) {
        design_apply_kernel<<<grid_for_(ns), 256, 0, s>>>(b.Z, kp, ns, nf, dx, dv);
        count_launch();
        design_adjoint_kernel<<<dim3(nf, column_split(nf, ns)), 256, 0, s>>>(b.Z, kp, ns, dv, dr);
        count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(r, dr, sizeof(double2) * nf, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(dx);
    cudaFree(dv);
    cudaFree(dr);
    return e;
}

cudaError_t fit_finish(FitBuffers& b, size_t kp, size_t ns, int nf, int nfp, double* gram, double* mean, double* sd,
                       cudaStream_t s) {
    // Split the samples over grid.z so that the upper-triangle tiles fill
    // whole waves of 2 CTAs per SM: the GPU time goes as waves(ks) / ks, and
    // the smallest split within 5 % of the best one keeps the FP64 atomics
    // that merge the splits few.
    const int tiles = (nfp / GT) * (nfp / GT + 1) / 2;
    const int kmax = std::max(1, std::min(256, (int)(kp / GK)));
    const int kWave = sm_count() * 2;
    auto per_wave = [&](int k) { return (double)k / (double)((tiles * k + kWave - 1) / kWave); };
    double best = 0.0;
    for (int k = 1; k <= kmax; ++k) best = std::max(best, per_wave(k));
    int ks = 1;
    while (ks < kmax && per_wave(ks) < 0.95 * best) ++ks;
    dim3 g2(nfp / GT, nfp / GT, ks);
    cudaError_t e0 = cudaMemsetAsync(b.G, 0, sizeof(double2) * (size_t)nfp * nfp, s);
    if (e0 != cudaSuccess) return e0;
    gram_kernel<<<g2, 256, 0, s>>>(b.Z, kp, nfp, b.G);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(gram, sizeof(double2) * (nf + 1), b.G, sizeof(double2) * nfp,
                              sizeof(double2) * (nf + 1), nf + 1, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(mean, b.stat, sizeof(double) * 2 * (nf + 1), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sd, b.stat + 2 * (size_t)nfp, sizeof(double) * nf, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e;
}

// The z-scored SINO design (sino.cpp:42-118) in b; returns the sizes.
focss_status sino_design(Ctx* c, const Field* tx, const Field* rx, int R, int type, double lw_re, double lw_im,
                         FitBuffers& b, int& nf, size_t& ns, size_t& kp, int& nfp) {
    if (type < 0 || type > 2 || R < 0) return FOCSS_ERR_INVALID_ARG;
    if (tx->modes != rx->modes || tx->samples != rx->samples || tx->batch != 1 || rx->batch != 1)
        return set_error(c, FOCSS_ERR_INVALID_ARG, "sino fit: tx and rx must be single realizations of one domain");
    const int N = tx->samples, modes = tx->modes;
    if (N <= 2 * R + 1) return set_error(c, FOCSS_ERR_INVALID_ARG, "sino fit: field shorter than the radius");
    std::vector<Feature> fs;
    spm_features(R, fs);
    if (type == 0) fs.push_back({0, 0, 4});
    nf = (int)fs.size();
    ns = (size_t)modes * (N - 2 * R);
    kp = (ns + GK - 1) / GK * GK;
    nfp = (nf + 1 + GT - 1) / GT * GT;  // features + responses, padded
    cudaStream_t s = c->stream;
    cudaError_t e = fit_alloc(b, fs, kp, nfp, s);
    if (e == cudaSuccess) {
        dim3 grid((unsigned)std::min<size_t>((ns + 255) / 256, 1024), nf);
        features_kernel<<<grid, 256, 0, s>>>(tx->d, modes, N, R, b.fs, nf, b.Z, kp);
        count_launch();
        responses_kernel<<<grid_for_(ns), 256, 0, s>>>(tx->d, rx->d, modes, N, R,
                                                        make_float2((float)lw_re, (float)lw_im), type == 1,
                                                        b.Z + (size_t)nf * kp);
        count_launch();
        e = fit_stats(b, kp, ns, nf, nfp, s);
    }
    return cuda_check(c, e, "sino fit design");
}

// The z-scored WdmPPE design (wdm_sino.cpp:28-93) in b.
focss_status wdm_design(Ctx* c, const Field* tx, const Field* rx, int c_radius, int d_radius, FitBuffers& b,
                        int& nf, size_t& ns, size_t& kp, int& nfp) {
    if (c_radius < -1 || d_radius < -1) return FOCSS_ERR_INVALID_ARG;
    if (tx->modes != 6 || (rx->modes != 6 && rx->modes != 2) || tx->samples != rx->samples || tx->batch != 1 ||
        rx->batch != 1)
        return set_error(c, FOCSS_ERR_INVALID_ARG,
                         "wdm_ppe fit: tx must be one 6-row realization (3 channels x 2 polarizations), rx 6 or 2 rows");
    const int N = tx->samples, R = std::max(c_radius, d_radius);
    if (R < 0 || N <= 2 * R + 1) return set_error(c, FOCSS_ERR_INVALID_ARG, "wdm_ppe fit: radius vs field length");
    // feature order of wdm_sino.cpp:43-80
    std::vector<Feature> fs;
    if (c_radius >= 0) spm_features(c_radius, fs);
    for (int m = -d_radius; m <= d_radius; ++m) {
        const int nb = d_radius - std::abs(m);
        for (int n = -nb; n <= nb; ++n) fs.push_back({m, n, 5});
    }
    fs.push_back({0, 0, 4});
    nf = (int)fs.size();
    ns = 2 * (size_t)(N - 2 * R);
    kp = (ns + GK - 1) / GK * GK;
    nfp = (nf + 1 + GT - 1) / GT * GT;
    cudaStream_t s = c->stream;
    cudaError_t e = fit_alloc(b, fs, kp, nfp, s);
    if (e == cudaSuccess) {
        dim3 grid((unsigned)std::min<size_t>((ns + 255) / 256, 1024), nf);
        wdm_features_kernel<<<grid, 256, 0, s>>>(tx->d, N, R, b.fs, nf, b.Z, kp);
        count_launch();
        wdm_responses_kernel<<<grid_for_(ns), 256, 0, s>>>(rx->d, rx->modes == 6 ? 2 : 0, N, R, b.Z + (size_t)nf * kp);
        count_launch();
        e = fit_stats(b, kp, ns, nf, nfp, s);
    }
    return cuda_check(c, e, "wdm_ppe fit design");
}

}  // namespace
}  // namespace fg

extern "C" {

FOCSS_API int focss_sino_num_features(int radius, int type) {
    if (radius < 0) return -1;
    return radius * (radius + 2) / 2 + 1 + (type == 0 ? 1 : 0);
}

FOCSS_API focss_status focss_sino_gram(focss_ctx* c, const focss_field* tx, const focss_field* rx, int radius,
                                       int type, double lw_re, double lw_im, double* gram, double* mean, double* sd) {
    using namespace fg;
    if (!c || !tx || !rx || !gram || !mean || !sd) return FOCSS_ERR_INVALID_ARG;
    FitBuffers b;
    int nf, nfp;
    size_t ns, kp;
    focss_status st = sino_design(c, tx, rx, radius, type, lw_re, lw_im, b, nf, ns, kp, nfp);
    if (st != FOCSS_OK) return st;
    return cuda_check(c, fit_finish(b, kp, ns, nf, nfp, gram, mean, sd, c->stream), "sino_gram");
}

FOCSS_API focss_status focss_sino_residual(focss_ctx* c, const focss_field* tx, const focss_field* rx, int radius,
                                           int type, double lw_re, double lw_im, const double* x, double* r) {
    using namespace fg;
    if (!c || !tx || !rx || !x || !r) return FOCSS_ERR_INVALID_ARG;
    FitBuffers b;
    int nf, nfp;
    size_t ns, kp;
    focss_status st = sino_design(c, tx, rx, radius, type, lw_re, lw_im, b, nf, ns, kp, nfp);
    if (st != FOCSS_OK) return st;
    return cuda_check(c, fit_residual(b, kp, ns, nf, x, r, c->stream), "sino_residual");
}

FOCSS_API int focss_wdm_ppe_num_features(int c_radius, int d_radius) {
    // wdm_sino.cpp:32-34
    const int n_spm = c_radius < 0 ? 0 : c_radius * (c_radius + 2) / 2 + 1;
    const int n_xpm = d_radius < 0 ? 0 : 2 * d_radius * d_radius + 2 * d_radius + 1;
    return n_spm + n_xpm + 1;
}

FOCSS_API focss_status focss_wdm_ppe_gram(focss_ctx* c, const focss_field* tx, const focss_field* rx, int c_radius,
                                          int d_radius, double* gram, double* mean, double* sd) {
    using namespace fg;
    if (!c || !tx || !rx || !gram || !mean || !sd) return FOCSS_ERR_INVALID_ARG;
    FitBuffers b;
    int nf, nfp;
    size_t ns, kp;
    focss_status st = wdm_design(c, tx, rx, c_radius, d_radius, b, nf, ns, kp, nfp);
    if (st != FOCSS_OK) return st;
    return cuda_check(c, fit_finish(b, kp, ns, nf, nfp, gram, mean, sd, c->stream), "wdm_ppe_gram");
}

FOCSS_API focss_status focss_wdm_ppe_residual(focss_ctx* c, const focss_field* tx, const focss_field* rx,
                                              int c_radius, int d_radius, const double* x, double* r) {
    using namespace fg;
    if (!c || !tx || !rx || !x || !r) return FOCSS_ERR_INVALID_ARG;
    FitBuffers b;
    int nf, nfp;
    size_t ns, kp;
    focss_status st = wdm_design(c, tx, rx, c_radius, d_radius, b, nf, ns, kp, nfp);
    if (st != FOCSS_OK) return st;
    return cuda_check(c, fit_residual(b, kp, ns, nf, x, r, c->stream), "wdm_ppe_residual");
}

}  // extern "C"
