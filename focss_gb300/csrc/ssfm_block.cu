// ssfm_block.cu -- single-CTA split-step runs for N <= 2^14 (block_kernel in
// ssfm_kernels.cuh): one CTA per realization, the field in shared memory for
// the whole run.  Splits: 2^12 = 64 x 64, 2^13 = 128 x 64 (112 KB: two CTAs
// per SM), 2^14 = 128 x 128.
#include "ssfm_kernels.cuh"

namespace fg {

int block_split(int N) {
    switch (N) {
        case 1 << 12: return 6;
        case 1 << 13: return 7;
        case 1 << 14: return 7;
        default: return 0;
    }
}

namespace {
template <int N1, int N2>
cudaError_t launch_block_t(const PassArgs& a, int batch, int cap, cudaStream_t s) {
    const size_t smem = BlockShape<N1, N2>::SMEM;
    // set on every launch: the attribute is per device, and the call is cheap
    cudaError_t e = cudaFuncSetAttribute((const void*)block_kernel<N1, N2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    block_kernel<N1, N2><<<batch, kBlockThreads, smem, s>>>(a, cap);
    count_launch();
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_block(const Plan& p, PassArgs a, int batch, int cap, cudaStream_t s) {
    if (!a.state || p.log2N1 != block_split(p.N) || (a.modes > 1)) return cudaErrorInvalidValue;
    a.N = p.N;
    a.N1 = p.N1;
    a.N2 = p.N2;
    a.log2N2 = p.log2N2;
    a.tw = p.tw;
    a.batch = batch;
    switch (p.N) {
        case 1 << 12: return launch_block_t<64, 64>(a, batch, cap, s);
        case 1 << 13: return launch_block_t<128, 64>(a, batch, cap, s);
        case 1 << 14: return launch_block_t<128, 128>(a, batch, cap, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace fg
