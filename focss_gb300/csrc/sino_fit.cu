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
// full-rank design).  The Gram product is a tiled complex kernel on the CUDA
// cores (64 x 64 output tiles, 4 x 4 complex outputs per thread) reading the
// FP32 features and accumulating in FP64.
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
    return (int)std::min<size_t>(g ? g : 1, (size_t)152 * 32);
}
constexpr int GK = 16;  // samples per shared-memory chunk

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

// Per column: mean (FP64) and, for features, the standard deviation
// (normalized by the count); then z-score features and centre the responses.
__global__ void column_stats_kernel(float2* __restrict__ Z, size_t kp, size_t ns, int nf, double* __restrict__ mean,
                                   double* __restrict__ sd) {
    __shared__ double red[64];
    const int f = blockIdx.x;
    float2* col = Z + (size_t)f * kp;
    double sr = 0, si = 0;
    for (size_t i = threadIdx.x; i < ns; i += blockDim.x) {
        sr += col[i].x;
        si += col[i].y;
    }
    sr = block_sum_d(sr, red);
    __syncthreads();
    si = block_sum_d(si, red);
    __shared__ double mu[2];
    if (threadIdx.x == 0) {
        mu[0] = sr / (double)ns;
        mu[1] = si / (double)ns;
    }
    __syncthreads();
    const double mr = mu[0], mi = mu[1];
    double ss = 0;
    for (size_t i = threadIdx.x; i < ns; i += blockDim.x) {
        const double dr = col[i].x - mr, di = col[i].y - mi;
        ss += dr * dr + di * di;
    }
    __syncthreads();
    ss = block_sum_d(ss, red);
    __shared__ double scale;
    if (threadIdx.x == 0) {
        mean[2 * f] = mr;
        mean[2 * f + 1] = mi;
        const double s = sqrt(ss / (double)ns);
        if (f < nf) sd[f] = s;
        scale = (f < nf && s > 0) ? 1.0 / s : 1.0;  // the responses are only centred
    }
    __syncthreads();
    const double sc = scale;
    for (size_t i = threadIdx.x; i < ns; i += blockDim.x)
        col[i] = make_float2((float)((col[i].x - mr) * sc), (float)((col[i].y - mi) * sc));
}

// G[a][b] = sum_i conj(Z[a][i]) Z[b][i] for the upper-triangle tiles (a <= b);
// Z is zero-padded to multiples of GT features and GK samples.
__global__ void __launch_bounds__(256) gram_kernel(const float2* __restrict__ Z, size_t kp, int nfp,
                                                   double2* __restrict__ G) {
    const int bi = blockIdx.y, bj = blockIdx.x;
    if (bi > bj) return;
    __shared__ float2 As[GK][GT + 1];
    __shared__ float2 Bs[GK][GT + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    // FP64 accumulation: the normal equations square the design's condition
    // number, so FP32 sums over ~1e5 samples are too coarse for the solve.
    double2 acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = make_double2(0.0, 0.0);
    const float2* Za = Z + (size_t)bi * GT * kp;
    const float2* Zb = Z + (size_t)bj * GT * kp;
    for (size_t k0 = 0; k0 < kp; k0 += GK) {
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
            double2 av[4], bv[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const float2 x = As[kk][ty * 4 + r];
                av[r] = make_double2(x.x, x.y);
            }
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const float2 x = Bs[kk][tx + 16 * c];  // consecutive lanes, consecutive words
                bv[c] = make_double2(x.x, x.y);
            }
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    // conj(a) * b
                    acc[r][c].x = fma(av[r].x, bv[c].x, fma(av[r].y, bv[c].y, acc[r][c].x));
                    acc[r][c].y = fma(av[r].x, bv[c].y, fma(-av[r].y, bv[c].x, acc[r][c].y));
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c)
            G[(size_t)(bi * GT + ty * 4 + r) * nfp + bj * GT + tx + 16 * c] = acc[r][c];
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
    if (!c || !tx || !rx || !gram || !mean || !sd || radius < 0 || type < 0 || type > 2)
        return FOCSS_ERR_INVALID_ARG;
    if (tx->modes != rx->modes || tx->samples != rx->samples || tx->batch != 1 || rx->batch != 1)
        return set_error(c, FOCSS_ERR_INVALID_ARG, "sino_gram: tx and rx must be single realizations of one domain");
    const int N = tx->samples, modes = tx->modes, R = radius;
    if (N <= 2 * R + 1) return set_error(c, FOCSS_ERR_INVALID_ARG, "sino_gram: field shorter than the radius");
    // feature list in the order of sino.cpp:70-100
    std::vector<Feature> fs;
    const int mb = R / 2;
    for (int m = -mb; m <= mb; ++m)
        for (int n = std::abs(m); n <= R - std::abs(m); ++n) {
            const int kind = (m == 0 && n == 0) ? 0 : (m == n) ? 1 : (m == -n) ? 2 : 3;
            fs.push_back({m, n, kind});
        }
    if (type == 0) fs.push_back({0, 0, 4});
    const int nf = (int)fs.size();
    if (nf != focss_sino_num_features(R, type)) return set_error(c, FOCSS_ERR_INVALID_ARG, "sino_gram: feature count");
    const size_t ns = (size_t)modes * (N - 2 * R);
    const size_t kp = (ns + GK - 1) / GK * GK;
    const int nfp = (nf + 1 + GT - 1) / GT * GT;  // features + responses, padded
    cudaStream_t s = c->stream;
    float2* Z = nullptr;
    Feature* dfs = nullptr;
    double2* dG = nullptr;
    double* dstat = nullptr;
    cudaError_t e = cudaMalloc(&Z, sizeof(float2) * (size_t)nfp * kp);
    if (e == cudaSuccess) e = cudaMalloc(&dfs, sizeof(Feature) * nf);
    if (e == cudaSuccess) e = cudaMalloc(&dG, sizeof(double2) * (size_t)nfp * nfp);
    if (e == cudaSuccess) e = cudaMalloc(&dstat, sizeof(double) * (3 * (size_t)nfp + 2));
    if (e == cudaSuccess) e = cudaMemsetAsync(Z, 0, sizeof(float2) * (size_t)nfp * kp, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dfs, fs.data(), sizeof(Feature) * nf, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        dim3 grid((unsigned)std::min<size_t>((ns + 255) / 256, 1024), nf);
        features_kernel<<<grid, 256, 0, s>>>(tx->d, modes, N, R, dfs, nf, Z, kp);
        count_launch();
        responses_kernel<<<grid_for_(ns), 256, 0, s>>>(tx->d, rx->d, modes, N, R,
                                                        make_float2((float)lw_re, (float)lw_im), type == 1,
                                                        Z + (size_t)nf * kp);
        count_launch();
        column_stats_kernel<<<nf + 1, 256, 0, s>>>(Z, kp, ns, nf, dstat, dstat + 2 * (size_t)nfp);
        count_launch();
        dim3 g2(nfp / GT, nfp / GT);
        gram_kernel<<<g2, 256, 0, s>>>(Z, kp, nfp, dG);
        count_launch();
        e = cudaGetLastError();
    }
    // gram: (nf+1) x (nf+1) complex128 (upper triangle valid); mean: nf+1 complex; sd: nf
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(gram, sizeof(double2) * (nf + 1), dG, sizeof(double2) * nfp,
                              sizeof(double2) * (nf + 1), nf + 1, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(mean, dstat, sizeof(double) * 2 * (nf + 1), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sd, dstat + 2 * (size_t)nfp, sizeof(double) * nf, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(Z);
    cudaFree(dfs);
    cudaFree(dG);
    cudaFree(dstat);
    return cuda_check(c, e, "sino_gram");
}

}  // extern "C"
