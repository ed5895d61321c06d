// noalloc.cu -- split-step propagation over caller-owned device memory with
// no allocation by the library (focss_ssfm_run_noalloc).
//
// Some callers cannot let a library call cudaMalloc: a host framework that
// owns the whole device heap through its own pool, a latency-critical loop
// where an allocation (and the synchronization it implies) is not allowed, or
// a process whose device-memory budget is fixed up front.  This entry point
// takes the field as a plain device pointer and keeps everything else it
// needs -- the per-realization step state, the step counter and the twiddle
// tables -- in one file-scope __device__ array of fixed size, so a call only
// memsets, launches, copies a few bytes back and synchronizes its stream.
//
// The array is shared by every call in the process (each device that loads
// the library holds its own copy until exit) and keeps the last call's
// contents; every call clears the state it needs and rewrites the tables, and
// calls that overlap on the GPU race on it.
#include <cmath>
#include <mutex>

#include "fft.cuh"
#include "internal.h"

namespace fg {
namespace {

constexpr int kNoallocMaxLog2Samples = 17;   // N <= 2^17 samples per realization
constexpr int kNoallocMaxBatch = 256;        // realizations per call
// Largest table set: N = 2^17 -> N1 = 256, N2 = 512: 2*N1 + 2*N2 + 512 entries.
constexpr int kNoallocTableEntries = 2 * 256 + 2 * 512 + 512;

struct NoallocScratch {
    float4 tw[kNoallocTableEntries];
    SsfmState state[kNoallocMaxBatch];
    int counters[16];
};

// ~59 KB of device memory per device, for the lifetime of the process.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoallocScratch)];

std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[256] = {};

// Device address of g_noalloc_scratch on the current device (set up once per device).
cudaError_t noalloc_scratch(NoallocScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = p;
    }
    *out = (NoallocScratch*)g_noalloc_ptr[dev];
    return cudaSuccess;
}

__device__ __forceinline__ float4 df_rotation(double turns_times_2) {
    double s, c;
    sincospi(turns_times_2, &s, &c);
    const float ch = (float)c, sh = (float)s;
    return make_float4(ch, sh, (float)(c - (double)ch), (float)(s - (double)sh));
}

__host__ __device__ __forceinline__ int group_p(int L) { return L <= 32 ? 4 : L <= 128 ? 8 : L <= 512 ? 16 : 32; }

// The plan tables of internal.h, computed on the device in FP64.
__global__ void noalloc_tables_kernel(float4* __restrict__ tw, int N, int N1, int N2) {
    const int total = 2 * N1 + 2 * N2 + 512;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        if (i < N1 + N2) {
            const int L = i < N1 ? N1 : N2;
            const int k = i < N1 ? i : i - N1;
            const int P = i < N1 ? col_group_p(L) : group_p(L);
            const long long e = (long long)(k % P) * (k / P) % L;
            tw[i] = df_rotation(-2.0 * (double)e / L);
        } else if (i < 2 * N1 + 2 * N2) {
            tw[i] = make_float4(0.f, 0.f, 0.f, 0.f);  // reserved
        } else {
            const int j = i - 2 * N1 - 2 * N2;
            tw[i] = df_rotation(2.0 * (double)j / 512);
        }
    }
}

}  // namespace
}  // namespace fg

extern "C" FOCSS_API focss_status focss_ssfm_run_noalloc(void* stream, void* data, int samples, int batch,
                                                         double time_step, const focss_fiber* fiber,
                                                         const focss_ssfm_opts* opts, double direction,
                                                         int* steps_out) {
    using namespace fg;
    if (!data || !fiber || !opts || !(time_step > 0) || batch <= 0) return FOCSS_ERR_INVALID_ARG;
    if (direction != 1.0 && direction != -1.0) return FOCSS_ERR_INVALID_ARG;
    int lg = 0;
    while (lg < 31 && (1 << lg) < samples) ++lg;
    if ((1 << lg) != samples || lg < 8) return FOCSS_ERR_INVALID_ARG;
    if (lg > kNoallocMaxLog2Samples || batch > kNoallocMaxBatch) return FOCSS_ERR_UNSUPPORTED;
    const focss_ssfm_opts& o = *opts;
    const focss_fiber& fib = *fiber;
    if (o.grid < 0 || o.grid > 2 || !(fib.length > 0)) return FOCSS_ERR_INVALID_ARG;
    if (o.grid == FOCSS_UNIFORM && o.total_steps <= 0) return FOCSS_ERR_INVALID_ARG;
    if (o.grid != FOCSS_UNIFORM && (!(o.maximum_step_size > 0) || !(o.maximum_phase_shift > 0)))
        return FOCSS_ERR_INVALID_ARG;
    if (o.grid == FOCSS_LOGARITHMIC && !(fib.alpha != 0)) return FOCSS_ERR_INVALID_ARG;

    NoallocScratch* sc = nullptr;
    cudaError_t e = noalloc_scratch(&sc);
    if (e != cudaSuccess) return FOCSS_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;

    Plan p;
    p.N = samples;
    p.log2N1 = lg / 2;
    p.log2N2 = lg - lg / 2;
    p.N1 = 1 << p.log2N1;
    p.N2 = 1 << p.log2N2;
    p.tw = sc->tw;

    e = cudaMemsetAsync(sc->state, 0, sizeof(SsfmState) * batch, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(sc->counters, 0, sizeof(int) * 16, s);
    if (e == cudaSuccess) {
        noalloc_tables_kernel<<<8, 256, 0, s>>>(sc->tw, p.N, p.N1, p.N2);
        count_launch();
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return FOCSS_ERR_CUDA;

    PassArgs a{};
    a.data = (float2*)data;
    a.state = sc->state;
    a.prm.alpha = fib.alpha;
    a.prm.beta2 = fib.beta2;
    a.prm.gamma = fib.gamma;
    a.prm.kappa = fib.kappa;
    a.prm.length = fib.length;
    a.prm.direction = direction;
    a.prm.max_phase = o.maximum_phase_shift;
    a.prm.max_step = o.maximum_step_size;
    a.prm.dw = 2.0 * 3.14159265358979323846 / (time_step * samples);
    a.prm.grid = o.grid;
    a.prm.total_steps = o.total_steps;
    a.prm.samples = samples;
    a.prm.n_done = sc->counters;
    ssfm_derive(a.prm);

    if (o.grid == FOCSS_UNIFORM) {
        for (long long i = 0; i < (long long)o.total_steps + 2 && e == cudaSuccess; ++i) {
            e = launch_col(p, a, batch, s);
            if (e == cudaSuccess) e = launch_row(p, a, batch, s);
        }
        if (e != cudaSuccess) return FOCSS_ERR_CUDA;
    } else {
        const long long cap = 1ll << 17;
        long long launched = 0;
        int done = 0;
        while (done < batch) {
            for (int i = 0; i < 16 && e == cudaSuccess; ++i) {
                e = launch_col(p, a, batch, s);
                if (e == cudaSuccess) e = launch_row(p, a, batch, s);
            }
            if (e == cudaSuccess) e = cudaMemcpyAsync(&done, sc->counters, sizeof(int), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return FOCSS_ERR_CUDA;
            launched += 16;
            if (launched > cap) return FOCSS_ERR_NOT_CONVERGED;
        }
    }
    SsfmState hs[kNoallocMaxBatch];
    e = cudaMemcpyAsync(hs, sc->state, sizeof(SsfmState) * batch, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return FOCSS_ERR_CUDA;
    for (int b = 0; b < batch; ++b) {
        if (hs[b].action != COL_IDLE) return FOCSS_ERR_TIMEOUT;
        if (steps_out) steps_out[b] = (o.grid == FOCSS_ADAPTIVE) ? hs[b].steps : hs[b].n_steps;
    }
    return FOCSS_OK;
}
