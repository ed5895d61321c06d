// internal.h -- host-side objects behind the C ABI (not installed).
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <set>
#include <memory>
#include <string>
#include <vector>

#include "../../include/focss_gpu.h"

namespace fg {

// Per-realization SSFM state machine, device resident.  The last CTA of each
// column pass advances it (no CTA ever waits on another).
struct SsfmState {
    double distance;               // |z| travelled (ADAPTIVE)
    double h;                      // signed size of the next nonlinear step
    double hl;                     // signed linear step of the next row pass
    double sum;                    // sum |A|^2 accumulator (LOGARITHMIC estimate)
    double gain_ratio;             // prod(exact gains) / prod(applied FP32 gains) (error feedback)
    double g_exact;                // exp(-alpha*hl/2)/N of the current hl (reused while hl repeats)
    unsigned long long disp_hi;    // beta2/2*hl*dw^2/(2pi) turns per k'^2 as a 96-bit
    unsigned long long disp_lo;    //   fraction: disp_hi * 2^-64 + disp_lo * 2^-96
    float lin_gain;                // exp(-alpha*hl/2)/N for the next row pass (FP32, fed back)
    int action;                    // next column-pass operation (ColOp)
    int row_active;                // 1: data is spectral, next row pass applies hl
    int final_step;                // current nonlinear step is the last of the span
    int index;                     // step index (UNIFORM/LOGARITHMIC)
    int n_steps;                   // step count (UNIFORM/LOGARITHMIC)
    int steps;                     // steps done (ADAPTIVE, reference counting)
    unsigned int peak_bits;        // atomicMax accumulator of the peak power (float bits)
    unsigned int blocks_done;      // last-block ticket
    float kerr_coef;               // (float)(kappa*gamma*h) of the next nonlinear step
    int recorded;                  // step sizes written to SsfmParams::h_record so far
};

enum ColOp : int { COL_FWD = 0, COL_KERR = 1, COL_INV = 2, COL_IDLE = 3 };
enum RowOp : int { ROW_SSFM = 0, ROW_TABLE = 1, ROW_SCALE = 2, ROW_FWD = 3, ROW_INV = 4, ROW_BANDPASS = 5 };

struct SsfmParams {
    double alpha, beta2, gamma, kappa, length;
    double direction;
    double max_phase, max_step;
    double dw;
    int grid, total_steps;
    int samples;
    int* n_done;
    // Derived per-run constants (ssfm_derive): kappa gamma, |kappa gamma|,
    // beta2/2 dw^2 / (2 pi) (the dispersion phase per metre of hl, in turns),
    // -alpha/2 and 1/samples.
    double kg, kg_abs, disp_c, loss_c, inv_samples;
    // Step-grid record / replay (both null on ordinary runs).  Realization b
    // writes |h_i| of its nonlinear steps to h_record[b*h_cap + i] (i < h_cap;
    // SsfmState::recorded counts them all), or takes the h_count[b] step sizes
    // h_replay[b*h_cap + i] instead of its grid's rule.
    double* h_record;
    const double* h_replay;
    const int* h_count;
    int h_cap;
};

// Fills the derived constants of p from its fiber and grid fields.
inline void ssfm_derive(SsfmParams& p) {
    p.kg = p.kappa * p.gamma;
    p.kg_abs = p.kg < 0 ? -p.kg : p.kg;
    p.disp_c = 0.5 * p.beta2 * p.dw * p.dw / (2.0 * 3.14159265358979323846);
    p.loss_c = -0.5 * p.alpha;
    p.inv_samples = 1.0 / (double)p.samples;  // exact: samples is a power of 2
}

// Twiddle tables, double-float {re_hi, im_hi, re_lo, im_lo}, packed in one
// device buffer (offsets in entries):
//   0            column sub-FFT table, entry u*P+t = W_N1^{t u}   (N1 entries)
//   N1           row sub-FFT table,    entry u*P+t = W_N2^{t u}   (N2 entries)
//   N1+N2        reserved (N1 entries; the column pass computes its six-step
//                factors on the device, sixstep_factor in fft.cuh)
//   2N1+N2       reserved (N2 entries)
//   2N1+2N2      exp(+2 pi i j/512), j < 512                      (512 entries)
struct PassArgs {
    float2* data;           // batch x N complex64
    const float4* tw;
    const float2* table;    // ROW_TABLE multiplier, transposed layout (k1*N2 + k2), length N
    SsfmState* state;       // null: plain transform driven by `op`
    SsfmParams prm;
    int N, N1, N2, log2N2;
    int batch;              // realizations (set by the launch helpers)
    int modes;              // modes per realization of an SSFM run (0 or 1: single mode)
    int op;
    float scale;
    int bp_cut;
    int* fault;             // set to 1 by a kernel whose bounded wait ran out (may be null)
};

struct Plan {
    int N = 0, N1 = 0, N2 = 0, log2N1 = 0, log2N2 = 0;
    float4* tw = nullptr;   // device tables (layout above)
    int staging = 0;        // FOCSS_STAGING_*: how the passes move their data
};

struct LoopGraph;  // span_loop.cu

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    // field storage: a stream-ordered pool that keeps released blocks for
    // reuse, so creating and destroying fields costs no device-wide sync
    cudaMemPool_t pool = nullptr;
    std::map<long long, Plan> plans;  // key (log2 N1 << 32) | N
    std::string last_error;
    SsfmState* d_state = nullptr;
    int state_cap = 0;
    int* d_counters = nullptr;       // small device scratch (n_done etc)
    int* h_pinned = nullptr;         // pinned polling buffer
    double* d_red = nullptr;         // reduction scratch
    size_t red_cap = 0;
    std::vector<void*> scratch;      // generic device scratch buffers
    std::vector<size_t> scratch_cap;
    // device-resident derived tables keyed by their parameters (RRC spectra, ...)
    std::map<std::string, void*> tables;
    // instrumentation (focss_profile_*)
    bool profiling = false;
    std::vector<cudaEvent_t> prof_events;
    double prof_ms[2] = {0, 0};          // column, row
    long long prof_launches[2] = {0, 0};
    // split-step FFT split (log2 N1) per length picked by the autotuner or
    // pinned by the caller; lengths absent here use the balanced split
    std::map<int, int> ssfm_split;
    int staging = 0;                 // FOCSS_STAGING_* for new plans (focss_set_pass_staging)
    // instantiated span-loop graphs keyed by shape and parameters, and the
    // streams/events their capture uses (span_loop.cu)
    std::map<std::string, LoopGraph*> loops;
    std::vector<cudaStream_t> side_streams;
    std::vector<cudaEvent_t> side_events;
    // live fields of this context: detached (ctx = null) when the context is
    // destroyed first, so that their later destroy does not touch it
    std::set<struct Field*> fields;
};

// Process-wide launch counter (focss_launch_count).  While a graph is being
// captured on this thread, launches are not counted; count_launch_graph adds
// the kernels a graph ran.
void count_launch(long long n = 1);
void count_launch_graph(long long n);
void set_capturing(bool on);

struct Field {
    Ctx* ctx = nullptr;
    int modes = 0, samples = 0, batch = 0;
    double dt = 0, f0 = 0;
    float2* d = nullptr;
    size_t n() const { return (size_t)batch * modes * samples; }
};

// ---- helpers implemented in capi.cu
// Streaming multiprocessors of the current device (queried once per device;
// grid sizes are multiples of it).
int sm_count();
focss_status set_error(Ctx* ctx, focss_status st, const std::string& msg);
focss_status cuda_check(Ctx* ctx, cudaError_t e, const char* what);
focss_status get_plan(Ctx* ctx, int N, const Plan** out);  // balanced split
focss_status get_plan_split(Ctx* ctx, int N, int log2N1, const Plan** out);
int default_split(int N);
bool split_supported(int N, int log2N1);
focss_status ensure_state(Ctx* ctx, int batch);
focss_status ensure_red(Ctx* ctx, size_t doubles);
void* scratch_buffer(Ctx* ctx, int slot, size_t bytes);

// ---- ssfm.cu
bool fft_size_supported(int N);
cudaError_t launch_col(const Plan& p, PassArgs a, int batch, cudaStream_t s);
cudaError_t launch_row(const Plan& p, PassArgs a, int batch, cudaStream_t s);
// Step-grid record / replay of one ssfm_run: device arrays as in SsfmParams.
struct StepGrid {
    double* record = nullptr;
    const double* replay = nullptr;
    const int* count = nullptr;
    int cap = 0;
    int max_steps = 0;  // replay: the largest entry of count
};
focss_status ssfm_run(Ctx* ctx, Field* f, const focss_fiber& fib, const focss_ssfm_opts& o, double dir,
                      int* steps_out, const StepGrid* grid = nullptr, int* recorded_out = nullptr);
// Argument checks of ssfm_run and the pass arguments of one run (state and
// finished-realization counter supplied by the caller).
focss_status ssfm_validate(Ctx* ctx, const Field* f, const focss_fiber& fib, const focss_ssfm_opts& o);
PassArgs ssfm_args(const Field* f, const focss_fiber& fib, const focss_ssfm_opts& o, double dir, SsfmState* state,
                   int* n_done);
// The plan ssfm_run uses for length N (autotuned or pinned split, else balanced).
focss_status ssfm_plan(Ctx* ctx, int N, const Plan** out);
// Split value selecting the single-CTA kernel (ssfm_block.cu) for a length.
constexpr int kSingleCta = -1;
// log2 N1 of the single-CTA kernel's split for length N, 0 if it has none.
int block_split(int N);
// One launch running the whole SSFM of `batch` single-mode realizations, at
// most `cap` column phases each (plan split must be block_split(N)).
cudaError_t launch_block(const Plan& p, PassArgs a, int batch, int cap, cudaStream_t s);
// True when field f's SSFM runs take the single-CTA kernel.
bool ssfm_single_cta(const Ctx* ctx, const Field* f);

// Amplifier operation `op` (FOCSS_AMP_*) as A <- scale*A + sigma*(z0 + i z1);
// false for an unknown op (capi.cu).
bool amplifier_coeffs(int op, double gain, double noise_factor, double f0, double dt, double* scale,
                      double* sigma);

// ---- triplet.cu
// Triplet sum over `modes` consecutive rows of each realization of `in`
// (realizations in_bstride apart) into out (batch x modes x samples); with rx
// the equalizer (rx - y) * inv_lw.
focss_status run_triplet_rows(Ctx* c, const float2* in, size_t in_bstride, int modes, int samples, int batch,
                              const float2* rx, int radius, int n_terms, const int32_t* m, const int32_t* n,
                              const double* coef, float2 inv_lw, float2* out);

// ---- span_loop.cu
void free_loop_graphs(Ctx* ctx);
// Plain transforms on a field buffer of `batch` x N (modes folded into batch).
focss_status fft_forward(Ctx* ctx, float2* data, int N, int batch);   // natural order, x 1/N
focss_status fft_inverse(Ctx* ctx, float2* data, int N, int batch);   // natural order, unnormalized
// Forward then pointwise op then inverse, spectrum never leaves the two-pass layout.
focss_status spectral_apply(Ctx* ctx, float2* data, int N, int batch, int row_op, const float2* table,
                            float scale, int bp_cut);
// Transposed-layout spectrum (k1*N2 + k2 holds bin k1 + N1*k2), x scale.
focss_status fft_forward_transposed(Ctx* ctx, float2* data, int N, int batch, float scale);
focss_status fft_inverse_transposed(Ctx* ctx, float2* data, int N, int batch);

// ---- dsp.cu
cudaError_t launch_scale(float2* d, size_t n, float2 s, cudaStream_t st);
cudaError_t launch_amplifier(float2* d, int modes, int samples, int batch, double scale, float sigma,
                             uint64_t seed, uint64_t counter, cudaStream_t st);
cudaError_t launch_power(const float2* d, int modes, int samples, int batch, double* avg,
                         unsigned int* peak_bits, cudaStream_t st);
cudaError_t launch_transpose_to_natural(const float2* src, float2* dst, int N1, int N2, int batch,
                                        cudaStream_t st);
cudaError_t launch_transpose_from_natural(const float2* src, float2* dst, int N1, int N2, int batch,
                                          cudaStream_t st);

}  // namespace fg

// The opaque handles of the C ABI.
struct focss_ctx : fg::Ctx {};
struct focss_field : fg::Field {};
