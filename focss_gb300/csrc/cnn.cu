// cnn.cu -- 1D convolutional correction network for the learned-DBP output.
//
// z = y + s * (Delta_re + i Delta_im), Delta = conv4(relu(conv3(relu(conv2(
//     relu(conv1(x0))))))), x0 = [Re y / s, Im y / s] (2 channels, padded to
// 16), 64 channels, kernel 9, zero padding at the sequence ends.  Weights are
// BF16 (FP32 master copy for Adam), activations BF16 channels-last, all
// products accumulate in FP32 on the tensor cores as tcgen05 MMAs with
// tensor-memory accumulators (the convolutions, forward and input gradient,
// and the weight gradients).  Loss L = mean |z - tx|^2.
//
// Forward conv: out[p][co] = b[co] + sum_{kk<9, ci} W[co][kk][ci] in[p+kk-4][ci]
//   GEMM D[p][co], M = 128 positions per tile, N = COUT, K = 9*CIN.
// Input gradient: the same conv with W'[ci][kk][co] = W[co][8-kk][ci].
// Weight gradient: gW[co][kk][ci] = sum_p g[p][co] in[p+kk-4][ci]
//   GEMM per tap, K = positions (chunked, atomics).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <new>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "tma_map.h"

namespace fg {
namespace {

typedef __nv_bfloat16 bf16;
constexpr int KW = 9;       // kernel width
constexpr int HALF = 4;     // (KW - 1) / 2
constexpr int CW = 64;      // hidden channels
constexpr int CIN0 = 16;    // padded input channels (2 used)
constexpr int COUT4 = 16;   // padded output channels (2 used)

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// ------------------------------------------------------------ tcgen05 forward conv
// Every forward-type convolution (the four layers, and the input gradients)
// as a tcgen05 implicit GEMM: D[p][co] with M = 128 positions per tile,
// N = COUT output channels, K = 9 taps x CIN input channels, accumulated in
// tensor memory (FP32 columns), read back with tcgen05.ld for the epilogue
// (bias, ReLU, mask, BF16 or FP32).  The activation tile holds 136 rows (the
// tile plus the 4-sample halo on each side), so the operand of tap kk is the
// same layout starting kk rows further: the im2col is an address offset.
// 64 input channels: rows of 128 bytes in the 128-byte-swizzled K-major
// layout, written by one TMA box per tile (CU_TENSOR_MAP_SWIZZLE_128B); the
// swizzle follows the absolute shared-memory address bits, so a start kk rows
// into a 1024-byte-aligned tile needs no base offset, and a 16-channel step
// is 32 bytes along the row.  16 input channels: the no-swizzle K-major
// canonical layout [k group][row][8] (8-row core matrices SBO = 128 B apart
// along M, LBO apart along K), one TMA box per 8-channel group.  Weights are
// stored [tap][k group][co][8] (no swizzle).  The kernel's pipeline is
// described at conv_fwd_tc_kernel.
namespace tc {
constexpr int M = 128, ROWS = M + 2 * HALF;
constexpr uint32_t SBO = 128;
constexpr long long kWaitCap = 1ll << 22;  // mbarrier polls before giving up

constexpr int STAGES = 4;                  // activation tiles in flight per CTA
constexpr int FWD_THREADS = 320;           // producer, MMA, two groups of four epilogue warps

template <int CIN, int COUT>
struct Shape {
    // 64 input channels: an activation tile is 136 rows of 128 bytes in the
    // 128-byte-swizzled K-major layout (one TMA box per tile); fewer: the
    // unswizzled layout [k group][row][8] (one box per 8-channel group)
    static constexpr bool SW128 = CIN == 64;
    [[maybe_unused]] static constexpr uint32_t LBO_A = ROWS * 16;
    static constexpr uint32_t LBO_B = COUT * 16;
    static constexpr size_t SMEM_B = (size_t)KW * (CIN / 8) * COUT * 16;
    static constexpr uint32_t STAGE_BYTES = (CIN / 8) * ROWS * 16;  // one activation tile
    static constexpr size_t SMEM = SMEM_B + STAGES * (size_t)STAGE_BYTES + 1024;  // + alignment slack
    static constexpr uint32_t ACC_COLS = COUT < 32 ? 32 : COUT;   // one FP32 accumulator
    static constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;           // two: a power of two >= 32
};

// Shared-memory matrix descriptor: start address, LBO and SBO in 16-byte
// units, the descriptor version 1 at bit 46, base offset 0, no swizzling.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}
// The same for a K-major operand in the 128-byte swizzled layout (TMA
// CU_TENSOR_MAP_SWIZZLE_128B): rows of 128 bytes, 8-row groups SBO = 1024 B
// apart, swizzling mode 2 at bit 61; LBO is not used (encoded 1).  `addr`
// must be 1024-byte aligned (base offset 0).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | (1ull << 16) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46) |
           (2ull << 61);
}
// kind::f16 instruction descriptor: FP32 accumulator (bits 4-5 = 1), BF16 A
// and B (bits 7-9 and 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at
// bit 24.
__host__ __device__ constexpr uint32_t idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// Waits for the phase of parity `parity` of `bar`, at most kWaitCap polls.
// Gives up early when *abort is set, and sets it when the polls run out.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity, volatile int* abort) {
    const uint32_t a = smem_addr(bar);
    for (long long it = 0; it < kWaitCap; ++it) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.b32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (abort && *abort) return false;
    }
    if (abort) *abort = 1;
    return false;
}
// D (tensor memory) = A B (+ D when `accumulate`), kind::f16, one CTA.
__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, bool accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)accumulate));
}
// Arrives on `bar` once every tcgen05 operation this thread issued so far completes.
__device__ __forceinline__ void mma_commit(unsigned long long* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_addr(bar))
                 : "memory");
}
constexpr int FWD_EPI = FWD_THREADS - 64;  // epilogue threads

// TMA tensor copy of one box at (x, y, z) of a 3-D tensor map into shared
// memory, completing on `bar` (x * element size must be a multiple of 16 bytes).
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

// 16-byte asynchronous copy global -> shared; `bytes` = 0 writes zeros.
__device__ __forceinline__ void cp16(uint32_t dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}

// tcgen05.ld of 16 columns without the wait; wait_ld then waits for every
// load in flight and ties these registers to the wait, so that no use of
// them can be scheduled before it.
__device__ __forceinline__ void ld_x16_async(uint32_t taddr, uint32_t (&u)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
          "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15])
        : "r"(taddr));
}
__device__ __forceinline__ void wait_ld(uint32_t (&u)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;\n"
                 : "+r"(u[0]), "+r"(u[1]), "+r"(u[2]), "+r"(u[3]), "+r"(u[4]), "+r"(u[5]), "+r"(u[6]), "+r"(u[7]),
                   "+r"(u[8]), "+r"(u[9]), "+r"(u[10]), "+r"(u[11]), "+r"(u[12]), "+r"(u[13]), "+r"(u[14]), "+r"(u[15])
                 :
                 : "memory");
}
__device__ __forceinline__ void ld_x16(uint32_t taddr, float (&r)[16]) {
    uint32_t u[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
          "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) r[i] = __uint_as_float(u[i]);
}
}  // namespace tc

// in: [B][L][CIN] bf16 (read through `amap`, a 3-D tensor map {CIN, L, B}
// with box {8, ROWS, 1}), W: [COUT][KW][CIN] bf16, bias: [COUT] f32 or null,
// out [B][L][COUT] (bf16, or f32 when OUT_F32); mask (optional, [B][L][COUT]
// bf16): multiply the result by (mask > 0).
//
// Persistent and warp-specialized: the grid covers the SMs, each CTA takes
// position tiles i = blockIdx.x + k gridDim.x of all B x ceil(L/128) tiles.
// Warp 0 (one thread) loads each tile's activations with TMA tensor copies
// (cp.async.bulk.tensor: one 128-byte-swizzled box of 64 channels x 136 rows,
// or one box of 8 channels per 8-channel group, zero-filled outside [0, L))
// into a ring of STAGES buffers (mbarriers full / empty); warp 1 (one thread)
// waits for the weights, then issues each tile's 9 CIN/16 MMAs into one of
// two tensor-memory accumulators and commits them to the stage's `empty`
// barrier and the accumulator's `full` barrier; warps 2-9 stage the weights
// once (barrier `wready`) and then run the epilogue in two groups of four
// (group g takes accumulator g, i.e. every other tile; a warp's lane quarter
// of tensor memory is warp & 3), so the epilogues of two tiles overlap the
// MMAs and loads of the tiles after them; each group releases its
// accumulator through `acc_empty`.  Every wait is bounded: past kWaitCap
// polls a role sets `abort`, the others leave their loops, the CTA waits
// (bounded) for its copies and MMAs in flight, frees its tensor memory and
// writes its tiles as NaN.
template <int CIN, int COUT, bool OUT_F32>
__global__ void __launch_bounds__(tc::FWD_THREADS, 1)
    conv_fwd_tc_kernel(const __grid_constant__ CUtensorMap amap, const bf16* __restrict__ W,
                       const float* __restrict__ bias, void* __restrict__ out, int L, int B, int relu,
                       const bf16* __restrict__ mask) {
    using S = tc::Shape<CIN, COUT>;
    constexpr int KG = CIN / 8, ST = tc::STAGES;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // operands from a 1024-byte boundary (TMA destinations want 128)
    const uint32_t raw = tc::smem_addr(smem_raw), sbase = (raw + 1023u) & ~1023u;
    bf16* Bs = reinterpret_cast<bf16*>(smem_raw + (sbase - raw));  // [tap][kgroup][co][8]
    unsigned char* As = smem_raw + (sbase - raw) + S::SMEM_B;      // ST x [kgroup][row][8]
    __shared__ __align__(8) unsigned long long full[ST], empty[ST], acc_full[2], acc_empty[2], drain, wready;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_flag;
    __shared__ float s_bias[COUT];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles = (L + tc::M - 1) / tc::M, T = ntiles * B;
    for (int i = threadIdx.x; i < COUT; i += blockDim.x) s_bias[i] = bias ? bias[i] : 0.f;
    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int i = 0; i < ST; ++i) {
            tc::mbar_init(&full[i], 1);
            tc::mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            tc::mbar_init(&acc_full[i], 1);
            tc::mbar_init(&acc_empty[i], 4);
        }
        tc::mbar_init(&drain, 1);
        tc::mbar_init(&wready, tc::FWD_EPI);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tc::smem_addr(&tmem_base)),
                     "r"(S::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_base;
    const uint32_t a_base = tc::smem_addr(As), bs0 = tc::smem_addr(Bs);
    if (warp >= 2) {
        // the epilogue warps stage the weights while the first tiles load:
        // 16-byte rows W[co][kk][8g .. 8g+7] -> Bs[(kk*KG + g)*COUT + co],
        // made visible to the tensor core's proxy before `wready` completes
        const uint4* W4 = reinterpret_cast<const uint4*>(W);
        for (int i = threadIdx.x - 64; i < KW * KG * COUT; i += tc::FWD_EPI) {
            const int co = i % COUT, kg = i / COUT;  // kg = kk*KG + g
            tc::cp16(bs0 + 16u * i, W4 + ((size_t)co * KW + kg / KG) * KG + kg % KG, 16u);
        }
        asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        tc::mbar_arrive(&wready);
    }

    int issued = 0;  // producer: tiles whose loads were queued
    if (warp == 0) {
        if (lane == 0) {
            for (int i = blockIdx.x, k = 0; i < T; i += gridDim.x, ++k) {
                const int s = k % ST;
                if (k >= ST && !tc::mbar_wait(&empty[s], ((k / ST) & 1) ^ 1, &abort_flag)) break;
                const int b = i / ntiles, p0 = (i % ntiles) * tc::M;
                tc::mbar_expect_tx(&full[s], S::STAGE_BYTES);
                const uint32_t dst = a_base + (uint32_t)s * S::STAGE_BYTES;
                if constexpr (S::SW128) {
                    tc::tma_load_3d(dst, &amap, 0, p0 - HALF, b, &full[s]);
                } else {
#pragma unroll
                    for (int g = 0; g < KG; ++g)
                        tc::tma_load_3d(dst + (uint32_t)g * (tc::ROWS * 16), &amap, 8 * g, p0 - HALF, b, &full[s]);
                }
                issued = k + 1;
            }
        }
    } else if (warp == 1) {
        if (lane == 0 && tc::mbar_wait(&wready, 0, &abort_flag)) {
            const uint64_t bdesc = tc::smem_desc(bs0, S::LBO_B, tc::SBO);
            for (int i = blockIdx.x, k = 0; i < T; i += gridDim.x, ++k) {
                const int s = k % ST, ac = k & 1;
                if (!tc::mbar_wait(&full[s], (k / ST) & 1, &abort_flag)) break;
                if (k >= 2 && !tc::mbar_wait(&acc_empty[ac], ((k >> 1) & 1) ^ 1, &abort_flag)) break;
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t d = tmem + (uint32_t)ac * S::ACC_COLS;
                // descriptors of the stage and of the weights; each MMA adds a
                // constant offset to the start-address field (addresses stay
                // below 2^18, so the 14-bit field cannot carry)
                const uint32_t a0 = a_base + (uint32_t)s * S::STAGE_BYTES;
                if constexpr (S::SW128) {
                    // tap kk starts kk rows (kk x 128 B) into the tile and the
                    // 16-channel step kc 32 B into each row; the stage is
                    // 1024-byte aligned, so the start's row phase inside the
                    // 8-row swizzle pattern (the descriptor's base offset) is kk & 7
                    const uint64_t adesc = tc::smem_desc_sw128(a0);
#pragma unroll
                    for (int kk = 0; kk < KW; ++kk)
#pragma unroll
                        for (int kc = 0; kc < CIN / 16; ++kc)
                            tc::mma_bf16(d, adesc + (uint64_t)((kk * 128 + kc * 32) >> 4),
                                         bdesc + (uint64_t)(((kk * KG + kc * 2) * S::LBO_B) >> 4), tc::idesc(COUT),
                                         (kk | kc) != 0);
                } else {
                    const uint64_t adesc = tc::smem_desc(a0, S::LBO_A, tc::SBO);
#pragma unroll
                    for (int kk = 0; kk < KW; ++kk)
#pragma unroll
                        for (int kc = 0; kc < CIN / 16; ++kc)  // 16 input channels = 2 K core matrices per MMA
                            tc::mma_bf16(d, adesc + (uint64_t)((kk * 16 + kc * 2 * S::LBO_A) >> 4),
                                         bdesc + (uint64_t)(((kk * KG + kc * 2) * S::LBO_B) >> 4), tc::idesc(COUT),
                                         (kk | kc) != 0);
                }
                tc::mma_commit(&empty[s]);    // the stage is free once these MMAs have read it
                tc::mma_commit(&acc_full[ac]);
            }
        }
    } else {
        // epilogue group ac = (warp - 2) / 4 takes the tiles of accumulator ac
        // (every other tile); warp & 3 selects its tensor-memory lanes
        // 32q .. 32q+31 = tile rows
        const int q = warp & 3, ac = (warp - 2) >> 2;
        for (int i = blockIdx.x + ac * gridDim.x, k = ac; i < T; i += 2 * gridDim.x, k += 2) {
            if (!tc::mbar_wait(&acc_full[ac], (k >> 1) & 1, &abort_flag)) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const int b = i / ntiles, p = (i % ntiles) * tc::M + 32 * q + lane;
            const size_t ob = (size_t)b * L * COUT + (size_t)p * COUT;
            // the whole row of the accumulator in flight at once, one wait
            uint32_t raw[COUT / 16][16];
#pragma unroll
            for (int c = 0; c < COUT / 16; ++c)
                tc::ld_x16_async(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(ac * S::ACC_COLS + 16 * c), raw[c]);
#pragma unroll
            for (int c = 0; c < COUT / 16; ++c) tc::wait_ld(raw[c]);
#pragma unroll
            for (int c0 = 0; c0 < COUT; c0 += 16) {
                float v[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(raw[c0 / 16][j]);
                if (p < L) {
                    uint4 mk[2] = {};
                    if (mask) {
                        const uint4* m4 = reinterpret_cast<const uint4*>(mask + ob + c0);
                        mk[0] = m4[0];
                        mk[1] = m4[1];
                    }
                    const bf16* mb = reinterpret_cast<const bf16*>(mk);
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        float x = v[j] + s_bias[c0 + j];
                        if (relu) x = fmaxf(x, 0.f);
                        if (mask && !(__bfloat162float(mb[j]) > 0.f)) x = 0.f;
                        v[j] = x;
                    }
                    if (OUT_F32) {
                        float4* o = reinterpret_cast<float4*>(reinterpret_cast<float*>(out) + ob + c0);
#pragma unroll
                        for (int u = 0; u < 4; ++u) o[u] = make_float4(v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]);
                    } else {
                        uint32_t packed[8];
#pragma unroll
                        for (int j = 0; j < 8; ++j) packed[j] = pack2(__float2bfloat16(v[2 * j]), __float2bfloat16(v[2 * j + 1]));
                        uint4* o = reinterpret_cast<uint4*>(reinterpret_cast<bf16*>(out) + ob + c0);
                        o[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
                        o[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
                    }
                }
            }
            // this warp's reads of the accumulator are complete: release it
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&acc_empty[ac]);
        }
    }
    __syncthreads();
    if (abort_flag) {
        // drain: the producer's queued copies and the issued MMAs land before
        // the CTA leaves (bounded again), then its tiles are marked invalid
        if (warp == 0 && lane == 0)
            for (int k = issued > ST ? issued - ST : 0; k < issued; ++k) tc::mbar_wait(&full[k % ST], (k / ST) & 1, nullptr);
        if (warp == 1 && lane == 0) {
            tc::mma_commit(&drain);  // completes once every MMA this thread issued has
            tc::mbar_wait(&drain, 0, nullptr);
        }
        __syncthreads();
        for (int i = blockIdx.x; i < T; i += gridDim.x) {
            const int b = i / ntiles, p0 = (i % ntiles) * tc::M;
            for (int e = threadIdx.x; e < tc::M * COUT; e += blockDim.x) {
                const int p = p0 + e / COUT;
                if (p >= L) continue;
                const size_t o = (size_t)b * L * COUT + (size_t)p * COUT + e % COUT;
                if (OUT_F32)
                    reinterpret_cast<float*>(out)[o] = __int_as_float(0x7fc00000);
                else
                    reinterpret_cast<bf16*>(out)[o] = __float2bfloat16(__int_as_float(0x7fc00000));
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(S::TMEM_COLS));
}

// ------------------------------------------------------------ tcgen05 weight gradient
// gW[co][kk][ci] += sum_p g[p][co] in[p+kk-4][ci]: per tap a GEMM with
// M = 64 (the 64-channel side: output channels when COUT = 64, else input
// channels with the result transposed), N = the other side (64 or 16),
// K = positions.  Both operands are MN-major (channels contiguous, as
// stored), no-swizzle canonical layout: 16-byte rows of 8 channels, one row
// per position, 8-row core matrices LBO = 128 B apart along K (positions),
// channel groups SBO apart.  The input operand of tap kk is the same buffer
// starting kk rows further (kk x 16 B), so the tap shift along K is an
// address offset.  A CTA accumulates three taps in tensor memory over its
// chunk of positions (a whole number of 128-position tiles).  One thread
// loads the tiles with TMA tensor copies (one box of 8 channels x 128 or 136
// rows per channel group, zero-filled outside [0, L)) into a ring of
// WSTAGES buffers (mbarriers full / empty); one thread issues each tile's
// MMAs and commits them to the tile's `empty` barrier, and after the last
// tile to `done`; then all warps add the accumulators to gW.  With M = 64
// the accumulator row m sits in tensor-memory lane 32 (m / 16) + m % 16.
// Every wait is bounded (kWaitCap polls); a CTA that gives up drains its
// copies and MMAs (bounded) and adds NaN, so the failure shows in gW.
namespace tcw {
constexpr int P = 128;                // positions per tile
constexpr int PR = P + 2 * HALF;      // input rows per tile (halo)
constexpr int TAPS = 3;               // taps per CTA
constexpr int WSTAGES = 3;            // tiles in flight per CTA
constexpr uint32_t LBO = 128;
template <int COUT, int CIN>
struct Shape {
    static constexpr bool G_IS_A = COUT == 64;           // M side = output-gradient channels
    static constexpr int NC = G_IS_A ? CIN : COUT;        // N
    static constexpr uint32_t SMEM_G = (uint32_t)(COUT / 8) * P * 16;
    static constexpr uint32_t SMEM_I = (uint32_t)(CIN / 8) * PR * 16;
    static constexpr uint32_t STAGE = SMEM_G + SMEM_I;   // multiples of 128 bytes (TMA destinations)
    static constexpr size_t SMEM = (size_t)WSTAGES * STAGE + 128;  // + alignment slack
    static constexpr uint32_t TMEM_COLS = TAPS * NC <= 64 ? 64 : 256;
    // kind::f16: FP32 D, BF16 A/B, both MN-major (bits 15, 16), N = NC, M = 64.
    static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
                                      ((uint32_t)(NC >> 3) << 17) | ((uint32_t)(64 >> 4) << 24);
    static_assert((COUT == 64 && (CIN == 64 || CIN == 16)) || (COUT == 16 && CIN == 64), "wgrad shapes");
    static_assert(SMEM_G % 128 == 0 && SMEM_I % 128 == 0, "TMA destinations on 128-byte boundaries");
};
}  // namespace tcw

template <int CIN, int COUT>
__global__ void __launch_bounds__(128) conv_wgrad_tc_kernel(const __grid_constant__ CUtensorMap gmap,
                                                            const __grid_constant__ CUtensorMap imap,
                                                            float* __restrict__ gW, int L, int chunk) {
    using S = tcw::Shape<COUT, CIN>;
    constexpr int GG = COUT / 8, IG = CIN / 8, ST = tcw::WSTAGES;  // 16-byte channel groups
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long full[ST], empty[ST], done, drain;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_flag;
    const int tap0 = blockIdx.x * tcw::TAPS;
    const int b = blockIdx.z;
    const int c0 = blockIdx.y * chunk;
    const int c1 = min(L, c0 + chunk);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t raw = tc::smem_addr(smem_raw), base = (raw + 127u) & ~127u;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tc::smem_addr(&tmem_base)),
                     "r"(S::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int i = 0; i < ST; ++i) {
            tc::mbar_init(&full[i], 1);
            tc::mbar_init(&empty[i], 1);
        }
        tc::mbar_init(&done, 1);
        tc::mbar_init(&drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_base;
    const int n = c1 > c0 ? (c1 - c0 + tcw::P - 1) / tcw::P : 0;
    int issued = 0;
    if (warp == 0 && lane == 0) {
        // tile t -> stage t % ST: G[cg][r] = g[p0 + r][8cg ..], I[cg][r] = in[p0 - 4 + r][8cg ..]
        for (int t = 0; t < n; ++t) {
            const int s = t % ST;
            if (t >= ST && !tc::mbar_wait(&empty[s], ((t / ST) & 1) ^ 1, &abort_flag)) break;
            const int p0 = c0 + t * tcw::P;
            const uint32_t gb = base + (uint32_t)s * S::STAGE, ib = gb + S::SMEM_G;
            tc::mbar_expect_tx(&full[s], S::STAGE);
#pragma unroll
            for (int cg = 0; cg < GG; ++cg) tc::tma_load_3d(gb + (uint32_t)cg * (tcw::P * 16), &gmap, 8 * cg, p0, b, &full[s]);
#pragma unroll
            for (int cg = 0; cg < IG; ++cg)
                tc::tma_load_3d(ib + (uint32_t)cg * (tcw::PR * 16), &imap, 8 * cg, p0 - HALF, b, &full[s]);
            issued = t + 1;
        }
    } else if (warp == 1 && lane == 0) {
        for (int t = 0; t < n; ++t) {
            const int s = t % ST;
            if (!tc::mbar_wait(&full[s], (t / ST) & 1, &abort_flag)) break;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t gb = base + (uint32_t)s * S::STAGE, ib = gb + S::SMEM_G;
#pragma unroll
            for (int j = 0; j < tcw::TAPS; ++j) {
                const int kk = tap0 + j;
#pragma unroll
                for (int ks = 0; ks < tcw::P / 16; ++ks) {  // 16 positions = 2 K core matrices per MMA
                    const uint64_t gd = tc::smem_desc(gb + ks * 2 * tcw::LBO, tcw::LBO, tcw::P * 16);
                    const uint64_t id = tc::smem_desc(ib + kk * 16 + ks * 2 * tcw::LBO, tcw::LBO, tcw::PR * 16);
                    tc::mma_bf16(tmem + (uint32_t)(S::NC * j), S::G_IS_A ? gd : id, S::G_IS_A ? id : gd, S::IDESC,
                                 (t | ks) != 0);
                }
            }
            tc::mma_commit(&empty[s]);  // the stage is free once these MMAs have read it
            if (t == n - 1) tc::mma_commit(&done);
        }
    }
    __syncthreads();
    bool ok = !abort_flag && (n == 0 || tc::mbar_wait(&done, 0, &abort_flag));
    ok = !__syncthreads_or(!ok);
    if (!ok) {
        // drain: the queued copies and the issued MMAs complete (bounded) before the CTA leaves
        if (warp == 0 && lane == 0)
            for (int t = issued > ST ? issued - ST : 0; t < issued; ++t) tc::mbar_wait(&full[t % ST], (t / ST) & 1, nullptr);
        if (warp == 1 && lane == 0) {
            tc::mma_commit(&drain);
            tc::mbar_wait(&drain, 0, nullptr);
        }
        __syncthreads();
    }
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    // epilogue: lanes 0-15 of warp w hold M-side channel m = 16 w + lane
    if (n > 0) {
        const int m = 16 * warp + lane;
        for (int j = 0; j < tcw::TAPS; ++j)
#pragma unroll
            for (int q = 0; q < S::NC; q += 16) {
                float v[16];
                tc::ld_x16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(S::NC * j + q), v);
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                if (lane < 16) {
                    if (!ok)
#pragma unroll
                        for (int e = 0; e < 16; ++e) v[e] = __int_as_float(0x7fc00000);
                    if constexpr (S::G_IS_A) {
                        // 16 consecutive input channels of output channel m: 4 vector reductions
                        float* dst = gW + ((size_t)m * KW + tap0 + j) * CIN + q;
#pragma unroll
                        for (int e = 0; e < 16; e += 4)
                            asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst + e), "f"(v[e]),
                                         "f"(v[e + 1]), "f"(v[e + 2]), "f"(v[e + 3])
                                         : "memory");
                    } else {
#pragma unroll
                        for (int e = 0; e < 16; ++e) atomicAdd(gW + ((size_t)(q + e) * KW + tap0 + j) * CIN + m, v[e]);
                    }
                }
            }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(S::TMEM_COLS));
}

// bias gradient: gb[co] += sum_p g[p][co].  Each lane sums one channel pair
// over a slot of positions, so a warp reads whole 128-byte rows; warps and
// then CTAs combine in shared memory and one atomic per channel per CTA.
template <int C>
__global__ void __launch_bounds__(256) bias_grad_kernel(const bf16* __restrict__ g, size_t positions,
                                                        float* __restrict__ gb) {
    constexpr int HC = C / 2, PW = 32 / HC;  // channel pairs; positions per warp step
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int cp = lane % HC, po = lane / HC;
    float a0 = 0.f, a1 = 0.f;
    const size_t step = (size_t)gridDim.x * nw * PW;
    for (size_t p = ((size_t)blockIdx.x * nw + warp) * PW + po; p < positions; p += step) {
        const __nv_bfloat162 v = reinterpret_cast<const __nv_bfloat162*>(g + p * C)[cp];
        a0 += __low2float(v);
        a1 += __high2float(v);
    }
    for (int o = HC; o < 32; o <<= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
    }
    __shared__ float sh[8][C];
    if (po == 0) {
        sh[warp][2 * cp] = a0;
        sh[warp][2 * cp + 1] = a1;
    }
    __syncthreads();
    if (threadIdx.x < C) {
        float t = 0.f;
        for (int w = 0; w < nw; ++w) t += sh[w][threadIdx.x];
        atomicAdd(&gb[threadIdx.x], t);
    }
}

// First-order perturbation triplets fed to the network's idle input channels:
// feature j of symbol k is T(m_j, n_j) + T(-m_j, -n_j) (T(0, 0) alone) with
// T(m, n)[k] = y[k+m] y[k+n] conj(y[k+m+n]) (src/focss/equalizer/sino.cpp:161-171,
// one mode), symbols outside the realization counting as zero, scaled by 1/s^3.
constexpr int kMaxTriplets = (CIN0 - 2) / 2;
struct Triplets {
    int count;
    int m[kMaxTriplets], n[kMaxTriplets];
};

__device__ __forceinline__ float2 sym_at(const float2* __restrict__ row, int L, int k) {
    return (k >= 0 && k < L) ? row[k] : make_float2(0.f, 0.f);
}
__device__ __forceinline__ float2 triplet_at(const float2* __restrict__ row, int L, int k, int m, int n) {
    const float2 c = sym_at(row, L, k + m + n);
    return cmul(cmul(sym_at(row, L, k + m), sym_at(row, L, k + n)), make_float2(c.x, -c.y));
}

// x0 = [Re y / s, Im y / s, Re f_0 / s^3, Im f_0 / s^3, ..., 0 ...] (16 channels)
__global__ void cnn_input_kernel(const float2* __restrict__ y, size_t n, int L, float inv_s, Triplets tr,
                                 bf16* __restrict__ x0) {
    static_assert(CIN0 == 2 + 2 * kMaxTriplets, "x0 channels: y and the triplets");
    const float inv_s3 = inv_s * inv_s * inv_s;
    // positions < 2^31 (the field's batch x length), so 32-bit index arithmetic
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (int)n; i += gridDim.x * blockDim.x) {
        const float2 v = y[i];
        const int r = i / L, k = i - r * L;
        const float2* row = y + (size_t)r * L;
        uint32_t w[CIN0 / 2];
        w[0] = pack2(__float2bfloat16(v.x * inv_s), __float2bfloat16(v.y * inv_s));
#pragma unroll
        for (int j = 0; j < kMaxTriplets; ++j) {
            float2 f = make_float2(0.f, 0.f);
            if (j < tr.count) {
                f = triplet_at(row, L, k, tr.m[j], tr.n[j]);
                if (tr.m[j] != 0 || tr.n[j] != 0) f = cadd(f, triplet_at(row, L, k, -tr.m[j], -tr.n[j]));
            }
            w[1 + j] = pack2(__float2bfloat16(f.x * inv_s3), __float2bfloat16(f.y * inv_s3));
        }
        uint4* o = reinterpret_cast<uint4*>(x0 + (size_t)i * CIN0);  // 32 bytes per position
        o[0] = make_uint4(w[0], w[1], w[2], w[3]);
        o[1] = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

// z = y + s (d0 + i d1); with tx: loss += |z - tx|^2 / M, g4 = dL/dDelta (bf16, 16 ch)
__global__ void cnn_output_kernel(const float2* __restrict__ y, const float* __restrict__ d4, size_t n, float s,
                                  const float2* __restrict__ tx, float inv_m, float2* __restrict__ z,
                                  bf16* __restrict__ g4, double* __restrict__ loss) {
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = make_float2(fmaf(s, d4[i * COUT4], y[i].x), fmaf(s, d4[i * COUT4 + 1], y[i].y));
        if (z) z[i] = v;
        if (tx) {
            const float2 d = csub(v, tx[i]);
            acc += (double)cnorm(d);
            static_assert(COUT4 == 16, "g4: 2 live channels and 14 zeros, 32 bytes per position");
            uint4* o = reinterpret_cast<uint4*>(g4 + i * COUT4);
            o[0] = make_uint4(pack2(__float2bfloat16(2.f * s * d.x * inv_m), __float2bfloat16(2.f * s * d.y * inv_m)), 0u,
                              0u, 0u);
            o[1] = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    __shared__ double sd[32];
    acc = block_sum_d(acc, sd);
    if (threadIdx.x == 0 && loss) atomicAdd(loss, acc * inv_m);
}

// BF16 weights and flipped transposes from the FP32 masters.
__global__ void refresh_weights_kernel(const float* __restrict__ Wm, int cout, int cin, bf16* __restrict__ Wb,
                                       bf16* __restrict__ Wt) {
    const int n = cout * KW * cin;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int co = i / (KW * cin), kk = (i / cin) % KW, ci = i % cin;
        const bf16 v = __float2bfloat16(Wm[i]);
        Wb[i] = v;
        Wt[((size_t)ci * KW + (KW - 1 - kk)) * cout + co] = v;   // W'[ci][8-kk][co]
    }
}

__global__ void cnn_adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                                float* __restrict__ m2, int n, float lr, float b1, float b2, float eps, float c1,
                                float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = b1 * m1[i] + (1.f - b1) * gi;
        const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = v;
        p[i] -= lr * (a * c1) / (sqrtf(v * c2) + eps);
    }
}

inline int gridn(size_t n) {
    return (int)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, (size_t)sm_count() * 16));
}

template <int CIN, int COUT, bool F32>
cudaError_t conv_fwd(const bf16* in, const bf16* W, const float* bias, void* out, int L, int B, int relu,
                     const bf16* mask, cudaStream_t s) {
    using S = tc::Shape<CIN, COUT>;
    auto kern = conv_fwd_tc_kernel<CIN, COUT, F32>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
    if (e != cudaSuccess) return e;
    PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    e = tensor_map_encoder(&encode);
    if (e != cudaSuccess) return e;
    // activations [B][L][CIN] as a 3-D tensor {CIN, L, B}; one box = all 64
    // channels (128 bytes, swizzled) or 8 channels (16 bytes) x ROWS positions
    // of one realization
    CUtensorMap amap;
    const cuuint64_t dims[3] = {(cuuint64_t)CIN, (cuuint64_t)L, (cuuint64_t)B};
    const cuuint64_t strides[2] = {(cuuint64_t)CIN * sizeof(bf16), (cuuint64_t)L * CIN * sizeof(bf16)};
    const cuuint32_t box[3] = {S::SW128 ? (cuuint32_t)CIN : 8u, (cuuint32_t)tc::ROWS, 1}, estr[3] = {1, 1, 1};
    if (encode(&amap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16*>(in), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, S::SW128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    // persistent: at most the CTAs that are resident at once (tensor memory
    // for two accumulators each, 512 columns per SM)
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, tc::FWD_THREADS, S::SMEM);
    if (e != cudaSuccess) return e;
    per_sm = std::max(1, std::min(per_sm, std::min(2, (int)(512 / S::TMEM_COLS))));
    const long long tiles = (long long)((L + tc::M - 1) / tc::M) * B;
    const int grid = (int)std::max(1ll, std::min(tiles, (long long)sm_count() * per_sm));
    kern<<<grid, tc::FWD_THREADS, S::SMEM, s>>>(amap, W, bias, out, L, B, relu, mask);
    count_launch();
    return cudaGetLastError();
}

// [B][L][C] bf16 as a 3-D tensor {C, L, B}; one box = 8 channels (16 bytes)
// x `rows` positions of one realization, zero-filled outside the tensor.
cudaError_t channel_group_map(CUtensorMap* map, const bf16* p, int C, int L, int B, int rows) {
    PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    const cudaError_t e = tensor_map_encoder(&encode);
    if (e != cudaSuccess) return e;
    const cuuint64_t dims[3] = {(cuuint64_t)C, (cuuint64_t)L, (cuuint64_t)B};
    const cuuint64_t strides[2] = {(cuuint64_t)C * sizeof(bf16), (cuuint64_t)L * C * sizeof(bf16)};
    const cuuint32_t box[3] = {8, (cuuint32_t)rows, 1}, estr[3] = {1, 1, 1};
    if (encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16*>(p), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    return cudaSuccess;
}

template <int CIN, int COUT>
cudaError_t conv_wgrad(const bf16* g, const bf16* in, float* gW, int L, int B, cudaStream_t s) {
    using S = tcw::Shape<COUT, CIN>;
    static_assert(KW % tcw::TAPS == 0, "taps per CTA");
    const int chunk = 2048;  // a whole number of 128-position tiles: no tile crosses a chunk
    cudaError_t e = cudaFuncSetAttribute(conv_wgrad_tc_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)S::SMEM);
    if (e != cudaSuccess) return e;
    CUtensorMap gmap, imap;
    e = channel_group_map(&gmap, g, COUT, L, B, tcw::P);
    if (e == cudaSuccess) e = channel_group_map(&imap, in, CIN, L, B, tcw::PR);
    if (e != cudaSuccess) return e;
    conv_wgrad_tc_kernel<CIN, COUT><<<dim3(KW / tcw::TAPS, (L + chunk - 1) / chunk, B), 128, S::SMEM, s>>>(
        gmap, imap, gW, L, chunk);
    count_launch();
    return cudaGetLastError();
}

}  // namespace
}  // namespace fg

// ---------------------------------------------------------------- model
namespace {
using fg::bf16;
// parameter blocks (FP32 masters): W1 [64][9][16], b1 [64], W2 [64][9][64], b2,
// W3 [64][9][64], b3, W4 [16][9][64], b4 [16]
struct CnnLayout {
    size_t w[4], b[4], total;
    int cout[4] = {fg::CW, fg::CW, fg::CW, fg::COUT4}, cin[4] = {fg::CIN0, fg::CW, fg::CW, fg::CW};
    CnnLayout() {
        size_t o = 0;
        for (int l = 0; l < 4; ++l) {
            w[l] = o;
            o += (size_t)cout[l] * fg::KW * cin[l];
            b[l] = o;
            o += cout[l];
        }
        total = o;
    }
};
}  // namespace

struct focss_cnn {
    focss_ctx* ctx = nullptr;
    int length = 0, batch = 0;
    float scale = 1.f;
    fg::Triplets triplets{};   // input features beside [Re y, Im y] (none by default)
    CnnLayout lay;
    float* params = nullptr;   // masters, grads, m1, m2
    float* grads = nullptr;
    float* m1 = nullptr;
    float* m2 = nullptr;
    bf16* wb[4] = {};          // bf16 weights
    bf16* wt[4] = {};          // bf16 flipped transposes
    bf16* act[4] = {};         // x0 (16 ch), out1..out3 (64 ch)
    float* d4 = nullptr;       // output (16 ch f32)
    bf16* g64a = nullptr;      // gradient buffers
    bf16* g64b = nullptr;
    bf16* g16 = nullptr;
    double* loss = nullptr;
    void* block = nullptr;
    int adam_t = 0;
    size_t positions() const { return (size_t)length * batch; }
};

static cudaError_t cnn_forward(focss_cnn* m, const focss_field* y) {
    cudaStream_t s = m->ctx->stream;
    const int L = m->length, B = m->batch;
    const size_t n = m->positions();
    fg::cnn_input_kernel<<<fg::gridn(n), 256, 0, s>>>(y->d, n, L, 1.f / m->scale, m->triplets, m->act[0]);
    fg::count_launch();
    cudaError_t e = cudaGetLastError();
    const float* P = m->params;
    if (e == cudaSuccess)
        e = fg::conv_fwd<fg::CIN0, fg::CW, false>(m->act[0], m->wb[0], P + m->lay.b[0], m->act[1], L, B, 1, nullptr, s);
    if (e == cudaSuccess)
        e = fg::conv_fwd<fg::CW, fg::CW, false>(m->act[1], m->wb[1], P + m->lay.b[1], m->act[2], L, B, 1, nullptr, s);
    if (e == cudaSuccess)
        e = fg::conv_fwd<fg::CW, fg::CW, false>(m->act[2], m->wb[2], P + m->lay.b[2], m->act[3], L, B, 1, nullptr, s);
    if (e == cudaSuccess)
        e = fg::conv_fwd<fg::CW, fg::COUT4, true>(m->act[3], m->wb[3], P + m->lay.b[3], m->d4, L, B, 0, nullptr, s);
    return e;
}

static cudaError_t cnn_refresh(focss_cnn* m) {
    cudaError_t e = cudaSuccess;
    for (int l = 0; l < 4 && e == cudaSuccess; ++l) {
        const int n = m->lay.cout[l] * fg::KW * m->lay.cin[l];
        fg::refresh_weights_kernel<<<fg::gridn(n), 256, 0, m->ctx->stream>>>(m->params + m->lay.w[l], m->lay.cout[l],
                                                                            m->lay.cin[l], m->wb[l], m->wt[l]);
        fg::count_launch();
        e = cudaGetLastError();
    }
    return e;
}

extern "C" {

FOCSS_API focss_status focss_cnn_create(focss_ctx* c, int channels, int kernel, int length, int batch,
                                        double input_scale, focss_cnn** out) {
    if (!c || !out || length <= 0 || batch <= 0 || !(input_scale > 0)) return FOCSS_ERR_INVALID_ARG;
    if (channels != fg::CW || kernel != fg::KW)
        return fg::set_error(c, FOCSS_ERR_UNSUPPORTED, "cnn: 64 channels and kernel 9 are implemented");
    focss_cnn* m = new (std::nothrow) focss_cnn();
    if (!m) return FOCSS_ERR_OOM;
    m->ctx = c;
    m->length = length;
    m->batch = batch;
    m->scale = (float)input_scale;
    const size_t P = m->lay.total, n = m->positions();
    size_t bytes = sizeof(float) * 4 * P;
    size_t wbytes = 0;
    for (int l = 0; l < 4; ++l) wbytes += 2 * sizeof(bf16) * m->lay.cout[l] * fg::KW * m->lay.cin[l];
    const size_t abytes = sizeof(bf16) * n * (fg::CIN0 + 3 * fg::CW) + sizeof(float) * n * fg::COUT4 +
                          sizeof(bf16) * n * (2 * fg::CW + fg::COUT4) + 64;
    cudaError_t e = cudaMalloc(&m->block, bytes + wbytes + abytes + 1024);
    if (e != cudaSuccess) {
        delete m;
        return fg::cuda_check(c, e, "cnn alloc");
    }
    char* p = (char*)m->block;
    auto take = [&](size_t b) { char* r = p; p += (b + 255) / 256 * 256; return (void*)r; };
    m->params = (float*)take(sizeof(float) * 4 * P);
    m->grads = m->params + P;
    m->m1 = m->grads + P;
    m->m2 = m->m1 + P;
    for (int l = 0; l < 4; ++l) {
        const size_t nw = (size_t)m->lay.cout[l] * fg::KW * m->lay.cin[l];
        m->wb[l] = (bf16*)take(sizeof(bf16) * nw);
        m->wt[l] = (bf16*)take(sizeof(bf16) * nw);
    }
    m->act[0] = (bf16*)take(sizeof(bf16) * n * fg::CIN0);
    for (int l = 1; l < 4; ++l) m->act[l] = (bf16*)take(sizeof(bf16) * n * fg::CW);
    m->d4 = (float*)take(sizeof(float) * n * fg::COUT4);
    m->g64a = (bf16*)take(sizeof(bf16) * n * fg::CW);
    m->g64b = (bf16*)take(sizeof(bf16) * n * fg::CW);
    m->g16 = (bf16*)take(sizeof(bf16) * n * fg::COUT4);
    m->loss = (double*)take(sizeof(double) * 2);
    e = cudaMemsetAsync(m->params, 0, sizeof(float) * 4 * P, c->stream);
    if (e == cudaSuccess) e = cnn_refresh(m);
    if (e != cudaSuccess) {
        cudaFree(m->block);
        delete m;
        return fg::cuda_check(c, e, "cnn init");
    }
    *out = m;
    return FOCSS_OK;
}

FOCSS_API focss_status focss_cnn_destroy(focss_cnn* m) {
    if (!m) return FOCSS_OK;
    cudaStreamSynchronize(m->ctx->stream);
    cudaFree(m->block);
    delete m;
    return FOCSS_OK;
}

FOCSS_API int focss_cnn_num_params(const focss_cnn* m) { return m ? (int)m->lay.total : 0; }

FOCSS_API focss_status focss_cnn_set_triplets(focss_cnn* m, int count, const int32_t* tm, const int32_t* tn) {
    if (!m || count < 0 || count > fg::kMaxTriplets || (count > 0 && (!tm || !tn))) return FOCSS_ERR_INVALID_ARG;
    for (int j = 0; j < count; ++j)
        if (std::abs(tm[j]) > m->length || std::abs(tn[j]) > m->length) return FOCSS_ERR_INVALID_ARG;
    fg::Triplets t{};
    t.count = count;
    for (int j = 0; j < count; ++j) {
        t.m[j] = tm[j];
        t.n[j] = tn[j];
    }
    m->triplets = t;
    return FOCSS_OK;
}

FOCSS_API focss_status focss_cnn_set_params(focss_cnn* m, const float* host, int n) {
    if (!m || !host || n != (int)m->lay.total) return FOCSS_ERR_INVALID_ARG;
    cudaStream_t s = m->ctx->stream;
    cudaError_t e = cudaMemcpyAsync(m->params, host, sizeof(float) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->m1, 0, sizeof(float) * 2 * n, s);
    if (e == cudaSuccess) e = cnn_refresh(m);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    m->adam_t = 0;
    return fg::cuda_check(m->ctx, e, "cnn set params");
}

FOCSS_API focss_status focss_cnn_get_params(focss_cnn* m, float* params, float* grads, int n) {
    if (!m || n != (int)m->lay.total) return FOCSS_ERR_INVALID_ARG;
    cudaStream_t s = m->ctx->stream;
    cudaError_t e = cudaSuccess;
    if (params) e = cudaMemcpyAsync(params, m->params, sizeof(float) * n, cudaMemcpyDeviceToHost, s);
    if (grads && e == cudaSuccess) e = cudaMemcpyAsync(grads, m->grads, sizeof(float) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return fg::cuda_check(m->ctx, e, "cnn get params");
}

static bool cnn_shape_ok(const focss_cnn* m, const focss_field* f) {
    return f && f->modes == 1 && f->samples == m->length && f->batch == m->batch;
}

FOCSS_API focss_status focss_cnn_forward(focss_cnn* m, const focss_field* y, focss_field* z) {
    if (!m || !cnn_shape_ok(m, y) || !cnn_shape_ok(m, z)) return FOCSS_ERR_INVALID_ARG;
    cudaError_t e = cnn_forward(m, y);
    const size_t n = m->positions();
    if (e == cudaSuccess) {
        fg::cnn_output_kernel<<<fg::gridn(n), 256, 0, m->ctx->stream>>>(y->d, m->d4, n, m->scale, nullptr, 0.f, z->d,
                                                                         nullptr, nullptr);
        fg::count_launch();
        e = cudaGetLastError();
    }
    return fg::cuda_check(m->ctx, e, "cnn forward");
}

FOCSS_API focss_status focss_cnn_loss_grad(focss_cnn* m, const focss_field* y, const focss_field* tx, double* loss) {
    if (!m || !cnn_shape_ok(m, y) || !cnn_shape_ok(m, tx)) return FOCSS_ERR_INVALID_ARG;
    cudaStream_t s = m->ctx->stream;
    const int L = m->length, B = m->batch;
    const size_t n = m->positions();
    const CnnLayout& Y = m->lay;
    cudaError_t e = cnn_forward(m, y);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->grads, 0, sizeof(float) * Y.total, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->loss, 0, sizeof(double), s);
    if (e == cudaSuccess) {
        fg::cnn_output_kernel<<<fg::gridn(n), 256, 0, s>>>(y->d, m->d4, n, m->scale, tx->d, 1.f / (float)n, nullptr,
                                                          m->g16, m->loss);
        fg::count_launch();
        e = cudaGetLastError();
    }
    float* G = m->grads;
    // layer 4 (no activation): weights, bias, input gradient masked by out3 > 0
    if (e == cudaSuccess) e = fg::conv_wgrad<fg::CW, fg::COUT4>(m->g16, m->act[3], G + Y.w[3], L, B, s);
    if (e == cudaSuccess) {
        fg::bias_grad_kernel<fg::COUT4><<<fg::sm_count() * 4, 256, 0, s>>>(m->g16, n, G + Y.b[3]);
        fg::count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = fg::conv_fwd<fg::COUT4, fg::CW, false>(m->g16, m->wt[3], nullptr, m->g64a, L, B, 0, m->act[3], s);
    // layers 3, 2 (64 -> 64)
    bf16* g = m->g64a;
    bf16* g2 = m->g64b;
    for (int l = 2; l >= 1 && e == cudaSuccess; --l) {
        e = fg::conv_wgrad<fg::CW, fg::CW>(g, m->act[l], G + Y.w[l], L, B, s);
        if (e == cudaSuccess) {
            fg::bias_grad_kernel<fg::CW><<<fg::sm_count() * 4, 256, 0, s>>>(g, n, G + Y.b[l]);
            fg::count_launch();
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = fg::conv_fwd<fg::CW, fg::CW, false>(g, m->wt[l], nullptr, g2, L, B, 0, m->act[l], s);
        std::swap(g, g2);
    }
    // layer 1: weights and bias only
    if (e == cudaSuccess) e = fg::conv_wgrad<fg::CIN0, fg::CW>(g, m->act[0], G + Y.w[0], L, B, s);
    if (e == cudaSuccess) {
        fg::bias_grad_kernel<fg::CW><<<fg::sm_count() * 4, 256, 0, s>>>(g, n, G + Y.b[0]);
        fg::count_launch();
        e = cudaGetLastError();
    }
    double h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, m->loss, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (loss) *loss = h;
    return fg::cuda_check(m->ctx, e, "cnn loss/grad");
}

FOCSS_API focss_status focss_cnn_adam_step(focss_cnn* m, double lr, double beta1, double beta2, double eps) {
    if (!m) return FOCSS_ERR_INVALID_ARG;
    m->adam_t += 1;
    const float c1 = (float)(1.0 / (1.0 - std::pow(beta1, m->adam_t)));
    const float c2 = (float)(1.0 / (1.0 - std::pow(beta2, m->adam_t)));
    const int n = (int)m->lay.total;
    fg::cnn_adam_kernel<<<fg::gridn(n), 256, 0, m->ctx->stream>>>(m->params, m->grads, m->m1, m->m2, n, (float)lr,
                                                                  (float)beta1, (float)beta2, (float)eps, c1, c2);
    fg::count_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cnn_refresh(m);
    return fg::cuda_check(m->ctx, e, "cnn adam");
}

}  // extern "C"
