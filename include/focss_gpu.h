/*
 * focss_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the focss
 * split-step Fourier / digital back-propagation / perturbation-equalizer path.
 *
 * The reference (focss) is a C++ class library with no FFI of its own; every
 * entry point below replaces one reference member or free function, named in
 * its comment (paths relative to the focss source tree).  Conventions:
 *
 *  - Plain C types only: opaque handles, pointers and sizes.
 *  - Every call returns focss_status; nothing throws across the ABI.
 *    focss_ctx_last_error() gives a human-readable reason for the last failure.
 *  - A focss_field is device-resident (complex64, FP32) and holds `batch`
 *    independent realizations of one Domain, each stored mode-major exactly
 *    like focss::Field (data[sample + mode*samples], src/focss/field.cpp:140-155).
 *    Host buffers passed to upload/download are interleaved (re, im).
 *  - Calls on one context are ordered on the context's CUDA stream.  Calls
 *    that return host values (reductions, step counts) synchronize the stream.
 *  - One context per host thread; a context is not thread-safe.
 *  - The library owns device memory; the caller owns host memory.
 *  - There is no CPU fallback: without a usable GPU, focss_ctx_create fails.
 */
#ifndef FOCSS_GPU_H_
#define FOCSS_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define FOCSS_API __attribute__((visibility("default")))
#else
#define FOCSS_API
#endif

typedef enum focss_status {
    FOCSS_OK = 0,
    FOCSS_ERR_INVALID_ARG = 1,  /* bad size, null pointer, mismatched domains   */
    FOCSS_ERR_OOM = 2,          /* device or pinned allocation failed           */
    FOCSS_ERR_CUDA = 3,         /* CUDA runtime error (see last_error)          */
    FOCSS_ERR_TIMEOUT = 4,      /* a bounded device/host loop hit its cap       */
    FOCSS_ERR_NOT_CONVERGED = 5,/* adaptive step loop exceeded its step cap     */
    FOCSS_ERR_UNSUPPORTED = 6,  /* shape outside the implemented range          */
    FOCSS_ERR_NO_DEVICE = 7     /* no CUDA device                                */
} focss_status;

typedef struct focss_ctx focss_ctx;
typedef struct focss_field focss_field;

/* focss::Domain (src/focss/field.h:39-61) */
typedef struct focss_domain {
    int modes;
    int samples;
    double time_step;
    double center_frequency;
} focss_domain;

/* focss::Fiber (src/focss/module/fiber.h:5-12), SI units. */
typedef struct focss_fiber {
    double alpha;
    double beta2;
    double gamma;
    double length;
    double wavelength;
    double kappa;
} focss_fiber;

/* SSFM grids and directions (src/focss/solver/ssfm.cpp:6-11). */
#define FOCSS_UNIFORM 0
#define FOCSS_LOGARITHMIC 1
#define FOCSS_ADAPTIVE 2
#define FOCSS_FORWARD 1.0
#define FOCSS_BACKWARD (-1.0)

/* SSFM configuration: the setters of focss::SSFM (src/focss/solver/ssfm.h:25-29). */
typedef struct focss_ssfm_opts {
    int grid;                    /* FOCSS_UNIFORM / _LOGARITHMIC / _ADAPTIVE      */
    int total_steps;             /* set_total_steps (UNIFORM)                     */
    double maximum_phase_shift;  /* set_maximum_phase_shift (ADAPTIVE, LOG)       */
    double maximum_step_size;    /* set_maximum_step_size (ADAPTIVE, LOG)         */
} focss_ssfm_opts;

/* Amplifier operations (src/focss/module/amplifier.cpp:15-42). */
#define FOCSS_AMP_AMPLIFY 0
#define FOCSS_AMP_ADD_NOISE 1
#define FOCSS_AMP_GIVE_POWER 2
#define FOCSS_AMP_DROP_POWER 3

/* ---------------------------------------------------------------- context */
/* No reference counterpart (the reference is single-threaded host code);
 * owns a CUDA stream, FFT twiddle tables and scratch. */
FOCSS_API focss_status focss_ctx_create(int device, focss_ctx** out);
FOCSS_API focss_status focss_ctx_destroy(focss_ctx* ctx);
FOCSS_API focss_status focss_ctx_sync(focss_ctx* ctx);
FOCSS_API void* focss_ctx_stream(focss_ctx* ctx); /* cudaStream_t */
FOCSS_API const char* focss_ctx_last_error(const focss_ctx* ctx);
FOCSS_API const char* focss_status_string(int status);
FOCSS_API int focss_abi_version(void);

/* ------------------------------------------------------------------ field */
/* focss::Field(const Domain&) (src/focss/field.cpp:24-38): zero-filled;      */
/* batch x modes <= 65535 (FOCSS_ERR_INVALID_ARG otherwise).  The storage     */
/* comes from the context's stream-ordered memory pool (allocated and, on     */
/* destroy, released in order on the context's stream, with no device-wide   */
/* synchronization).  A field destroyed after its context is released with  */
/* a synchronizing free; no other call may use it once the context is gone. */
FOCSS_API focss_status focss_field_create(focss_ctx* ctx, const focss_domain* domain, int batch,
                                          focss_field** out);
/* ~Field (src/focss/field.cpp:130, 543-547) */
FOCSS_API focss_status focss_field_destroy(focss_field* field);
/* Field::domain() (src/focss/field.cpp:232-234) plus the batch count. */
FOCSS_API focss_status focss_field_domain(const focss_field* field, focss_domain* domain, int* batch);
/* Field(const Domain&, const ComplexVector&) (src/focss/field.cpp:40-54) and
 * element reads Field::operator[] (:135-155): FP64 host <-> FP32 device.
 * n_complex must equal batch*modes*samples. */
FOCSS_API focss_status focss_field_upload(focss_field* field, const double* interleaved, size_t n_complex);
FOCSS_API focss_status focss_field_download(focss_field* field, double* interleaved, size_t n_complex);
/* Same, FP32 host buffers (no conversion; pinned buffers give full PCIe/C2C rate). */
FOCSS_API focss_status focss_field_upload_c64(focss_field* field, const float* interleaved, size_t n_complex);
FOCSS_API focss_status focss_field_download_c64(focss_field* field, float* interleaved, size_t n_complex);
/* Field::operator=(const Field&) (src/focss/field.cpp:87-105); same shape. */
FOCSS_API focss_status focss_field_copy(focss_field* dst, const focss_field* src);
/* Copy `count` realizations src[src_first ...] to dst[dst_first ...] (same
 * modes and samples): Field copies (src/focss/field.cpp:56-68) of batch slices. */
FOCSS_API focss_status focss_field_copy_realizations(focss_field* dst, int dst_first, const focss_field* src,
                                                     int src_first, int count);
/* Copy modes src[src_first ... src_first+count) to dst[dst_first ...] in every
 * realization (same batch and samples): gathers channels' polarizations into
 * the rows of a dataset matrix (channel * modes + mode, the layout of
 * src/tasks/wdm_run.cpp:55-77) and back. */
FOCSS_API focss_status focss_field_copy_modes(focss_field* dst, int dst_first, const focss_field* src, int src_first,
                                              int count);
/* Device pointer to the complex64 data (for interop); valid until destroy,  */
/* ordered on the context's stream (synchronize the context before using it */
/* from another stream).                                                    */
FOCSS_API void* focss_field_device_ptr(focss_field* field);
/* Field::operator*=(const complex_t&) (src/focss/field.cpp:387-391). */
FOCSS_API focss_status focss_field_scale(focss_field* field, double re, double im);
/* Field::average_power / peak_power (src/focss/field.cpp:173-187), per
 * realization, FP64 accumulation.  Either output may be NULL. */
FOCSS_API focss_status focss_field_power(focss_field* field, double* average, double* peak);
/* Field::fft_inplace / ifft_inplace (src/focss/field.cpp:343-352): forward
 * normalized by 1/N, inverse unnormalized, natural bin order. */
FOCSS_API focss_status focss_field_fft(focss_field* field);
FOCSS_API focss_status focss_field_ifft(focss_field* field);

/* ------------------------------------------------------------------- SSFM */
/* SSFM::run(Field&, Direction) (src/focss/solver/ssfm.cpp:39-60) for every
 * realization of `field`: UNIFORM (:62-72), LOGARITHMIC (:74-90) or ADAPTIVE
 * (:92-118).  steps_out (length batch, may be NULL) receives the step counts
 * (UNIFORM: total_steps; LOGARITHMIC: the estimated count; ADAPTIVE: the
 * reference's steps_done). */
FOCSS_API focss_status focss_ssfm_run(focss_ctx* ctx, focss_field* field, const focss_fiber* fiber,
                                      const focss_ssfm_opts* opts, double direction, int* steps_out);

/* How the split-step passes move their data between HBM and shared memory
 * (no reference counterpart): FOCSS_STAGING_LOADS (default) with coalesced
 * 8-byte loads and stores by every thread; FOCSS_STAGING_BULK with the row
 * pass's rows moved by the TMA bulk-copy engine (cp.async.bulk, one copy per
 * row behind an mbarrier); FOCSS_STAGING_TMA as BULK, and the column pass's
 * tiles (C columns x N1 rows) loaded as 2-D TMA tensor boxes
 * (cp.async.bulk.tensor.2d).  The arithmetic is the same, so the results are
 * the same bit for bit.  Applies to this context's split-step and transform
 * passes from the next launch on.  focss_set_row_staging is the same call
 * restricted to LOADS and BULK. */
#define FOCSS_STAGING_LOADS 0
#define FOCSS_STAGING_BULK 1
#define FOCSS_STAGING_TMA 2
FOCSS_API focss_status focss_set_pass_staging(focss_ctx* ctx, int mode);
FOCSS_API focss_status focss_set_row_staging(focss_ctx* ctx, int mode);

/* Step-grid record and replay.  The reference has no counterpart: SSFM::run
 * only prints the adaptive step count (src/focss/solver/ssfm.cpp:117).  An
 * ADAPTIVE grid takes each step size from the current field's peak power
 * (:92-118, :136-140), so two runs that differ in rounding walk slightly
 * different grids; recording one run's grid and replaying it in another (or in
 * an FP64 oracle) puts both on the same grid.
 * focss_ssfm_run_record: focss_ssfm_run that also writes the nonlinear step
 * sizes |h_i| (metres, in order) of realization b to steps_h[b*capacity + i]
 * (host array of batch*capacity doubles; steps_out as focss_ssfm_run).
 * Returns FOCSS_ERR_INVALID_ARG after the run when a realization took more
 * than `capacity` steps.
 * focss_ssfm_run_steps: SSFM::run with the given step sizes in place of a
 * grid rule.  Realization b takes n_steps[b] (1..capacity) steps of size
 * h_i = steps_h[b*capacity + i] (> 0; their sum is the distance covered) in
 * the Strang pattern of the ADAPTIVE grid: L(h_0/2) N(h_0) L(h_0/2) ...
 * N(h_last) L(h_last/2), with the fiber's loss, dispersion and Kerr
 * coefficients.  Replaying a recorded grid on the GPU repeats the recorded
 * run's arithmetic bit for bit. */
FOCSS_API focss_status focss_ssfm_run_record(focss_ctx* ctx, focss_field* field, const focss_fiber* fiber,
                                             const focss_ssfm_opts* opts, double direction, int capacity,
                                             double* steps_h, int* steps_out);
FOCSS_API focss_status focss_ssfm_run_steps(focss_ctx* ctx, focss_field* field, const focss_fiber* fiber,
                                            const double* steps_h, const int* n_steps, int capacity,
                                            double direction);

/* ------------------------------------------------------------- amplifier */
/* Amplifier::amplify / add_noise / give_power / drop_power
 * (src/focss/module/amplifier.cpp:15-42).  `gain` and `noise_factor` are the
 * linear values the Amplifier constructor takes.  ASE noise comes from the
 * counter-based Philox4x32-10 stream keyed by `seed`; `counter` selects an
 * independent draw (e.g. the span index); realization b of the field uses an
 * independent substream. */
FOCSS_API focss_status focss_amplifier_apply(focss_ctx* ctx, focss_field* field, double gain,
                                             double noise_factor, uint64_t seed, uint64_t counter,
                                             int op);

/* ----------------------------------------------------------- span loops */
/* forward_propagation (src/tasks/systems.cpp:26-61): for each span, SSFM
 * FORWARD with `opts`, then Amplifier(gain, noise_factor).amplify with noise
 * counter = counter0 + span. */
FOCSS_API focss_status focss_forward_propagation(focss_ctx* ctx, focss_field* field,
                                                 const focss_fiber* fiber, const focss_ssfm_opts* opts,
                                                 double gain, double noise_factor, uint64_t seed,
                                                 uint64_t counter0, int spans);
/* backward_propagation (src/tasks/systems.cpp:73-91): for each span,
 * Amplifier(gain).drop_power then SSFM BACKWARD with `opts` (DBP). */
FOCSS_API focss_status focss_backward_propagation(focss_ctx* ctx, focss_field* field,
                                                  const focss_fiber* fiber, const focss_ssfm_opts* opts,
                                                  double gain, int spans);
/* cd_compensation (src/tasks/systems.cpp:63-71):
 * SSFM(fiber.dispersive() * spans, 1).run(BACKWARD). */
FOCSS_API focss_status focss_cd_compensation(focss_ctx* ctx, focss_field* field,
                                             const focss_fiber* fiber, int spans);

/* ------------------------------------------ graph-captured span loops */
#define FOCSS_AMP_NONE (-1)
typedef struct focss_amp {
    double gain;          /* linear span gain G (Amplifier(gain, noise_factor))      */
    double noise_factor;  /* linear noise factor; 0 = no ASE                         */
    uint64_t seed;        /* ASE key; field i of a focss_span_loop call uses seed+i  */
    uint64_t counter0;    /* ASE counter of span 0; span s uses counter0 + s         */
    int before;           /* FOCSS_AMP_* applied before each span's SSFM, or _NONE   */
    int after;            /* FOCSS_AMP_* applied after each span's SSFM, or _NONE    */
} focss_amp;

/* The span loops of forward_propagation / backward_propagation
 * (src/tasks/systems.cpp:26-61, 73-91) for n_fields fields at once: for each
 * span, amp->before, SSFM::run(field, direction) with opts[i] (one entry per
 * field), amp->after.  Fields may differ in length and batch; they run as
 * concurrent branches of ONE CUDA graph launch.  UNIFORM grids are fixed
 * sequences of passes; ADAPTIVE and LOGARITHMIC spans run as a device-side
 * loop (a conditional WHILE graph node) that a kernel ends once every
 * realization of the field has finished the span, capped at 2^17 passes per
 * span (FOCSS_ERR_NOT_CONVERGED beyond).  The graph is recorded on the first
 * call for a given set of fields, shapes and parameters and replayed after
 * that; seed and counter0 are read from device memory, so changing them does
 * not re-record.  steps_out (may be NULL) receives, per realization, the steps
 * summed over all spans, fields concatenated in order.  Returns after the
 * propagation finished.  No reference counterpart for the multi-field form. */
FOCSS_API focss_status focss_span_loop(focss_ctx* ctx, int n_fields, focss_field* const* fields,
                                       const focss_fiber* fiber, const focss_ssfm_opts* opts,
                                       const focss_amp* amp, int spans, double direction, int* steps_out);

/* Split-step FFT autotuner (no reference counterpart).  The two-pass FFT of
 * length N = N1*N2 can use any split with N1, N2 in [2^4, 2^10]; for N in
 * [2^12, 2^14] a single-CTA kernel (FOCSS_SPLIT_SINGLE_CTA: one CTA per
 * realization runs the whole SSFM with the field in shared memory) is a
 * further candidate.  This times every candidate on a scratch batch of
 * `batch` realizations (a few UNIFORM steps each, CUDA events) and keeps the
 * fastest for this context's split-step runs of length `samples`.
 * log2_n1 / ms_per_step (may be NULL) receive the choice and its time per
 * step for the whole batch. */
#define FOCSS_SPLIT_SINGLE_CTA (-1)
FOCSS_API focss_status focss_autotune(focss_ctx* ctx, int samples, int batch, int* log2_n1, double* ms_per_step);
/* Pin the split used for split-step runs of length `samples` (log2_n1 = 0
 * restores the balanced default; FOCSS_SPLIT_SINGLE_CTA selects the
 * single-CTA kernel for single-mode fields of 2^12..2^14 samples, other
 * fields of that length keep the balanced two-pass split). */
FOCSS_API focss_status focss_set_fft_split(focss_ctx* ctx, int samples, int log2_n1);

/* --------------------------------------------------- TX / resampling DSP */
/* Output fields must be created by the caller with the shape the reference
 * would produce (same modes and batch; samples as stated).  Inputs are not
 * modified unless stated. */

/* gray_symbols_16qam (src/focss/processing/modulation.cpp:9-17):
 * out[i] = Gray 16QAM point of codes[i] & 15, unit average power.
 * codes: host int32 array of batch*modes*samples entries in field order. */
FOCSS_API focss_status focss_qam16_map(focss_ctx* ctx, const int32_t* codes, size_t n, focss_field* out);
/* Field::upsample / downsample (src/focss/field.cpp:272-297):
 * out->samples = in->samples * factor  /  in->samples / factor. */
FOCSS_API focss_status focss_upsample(focss_ctx* ctx, const focss_field* in, int factor, focss_field* out);
FOCSS_API focss_status focss_downsample(focss_ctx* ctx, const focss_field* in, int factor, focss_field* out);
/* Field::decimate (src/focss/field.cpp:299-320): spectral truncation,
 * out->samples = in->samples / factor. */
FOCSS_API focss_status focss_decimate(focss_ctx* ctx, const focss_field* in, int factor, focss_field* out);
/* pulse::rrc (src/focss/processing/modulation.cpp:47-74), computed on the
 * device in FP64; taps: host array of n_symbols*osf complex (interleaved). */
FOCSS_API focss_status focss_rrc_pulse(focss_ctx* ctx, int n_symbols, int osf, double roll_off, double* taps);
/* Field::filter_inplace (src/focss/field.cpp:358-372): circular convolution
 * with an ifftshifted impulse response h (host, interleaved, h_len <= samples). */
FOCSS_API focss_status focss_filter(focss_ctx* ctx, focss_field* field, const double* h, int h_len);
/* rrc_shaping / rrc_sampling (src/focss/processing/modulation.cpp:85-96).
 * The reference fixes the roll-off at 0.01 (:85); here it is a parameter. */
FOCSS_API focss_status focss_rrc_shaping(focss_ctx* ctx, const focss_field* symbols, int osf, double roll_off,
                                         double gain, focss_field* out);
FOCSS_API focss_status focss_rrc_sampling(focss_ctx* ctx, const focss_field* signal, int osf, double roll_off,
                                          double gain, focss_field* out);
/* frequency_shift / bandpass_filter (src/focss/processing/modulation.cpp:255-277), in place. */
FOCSS_API focss_status focss_frequency_shift(focss_ctx* ctx, focss_field* field, double frequency);
FOCSS_API focss_status focss_bandpass(focss_ctx* ctx, focss_field* field, double frequency);
/* wdm_select (src/focss/processing/modulation.cpp:248-253): out = channel
 * `channel_index` of in, shifted to baseband and brick-wall filtered. */
FOCSS_API focss_status focss_wdm_select(focss_ctx* ctx, const focss_field* in, int channel_index,
                                        double channel_bandwidth, focss_field* out);
/* wdm_mux (src/focss/processing/modulation.cpp:225-235): channel c is
 * realization c of `channels` (batch = number of channels); out has batch 1. */
FOCSS_API focss_status focss_wdm_mux(focss_ctx* ctx, const focss_field* channels, double channel_bandwidth,
                                     focss_field* out);

/* ------------------------------------------------- RX decisions / metrics */
/* Per-realization outputs are host arrays of length batch.  A negative `cut`
 * selects the reference's overload without a cut (same as cut = 0). */

/* hard_decision_16qam (src/focss/processing/modulation.cpp:112-120). */
FOCSS_API focss_status focss_hard_decision(focss_ctx* ctx, const focss_field* in, focss_field* out);
/* soft_decision_16qam (src/focss/processing/modulation.cpp:122-146): the
 * hard decision per quadrature, except where the received value normalized by
 * sqrt(average power / modes) lies within sqrt(10)*uncertainty of a decision
 * boundary (0, +-2/sqrt(10)); there the received value is kept. */
FOCSS_API focss_status focss_soft_decision(focss_ctx* ctx, const focss_field* in, double uncertainty,
                                          focss_field* out);
/* Certainty-based decisions of the WDM scoring task.  Each realization is one
 * matrix of the task (rows = modes; a dataset field has channel * modes + mode
 * rows), scaled by its RMS amplitude over all rows and samples.
 * find_certainty (src/tasks/wdm_scoring.cpp:105-126): certainty[b] =
 * sqrt(5) * min(1/sqrt(5), smallest RMS-normalized distance from a wrongly
 * decided received sample to its decided point); host array of batch.
 * sd (src/tasks/wdm_scoring.cpp:128-144) = focss_certainty_decision: a sample
 * snaps to its decided point when closer than certainty / sqrt(5), else it is
 * kept.  hd (src/tasks/wdm_scoring.cpp:146-156) is focss_hard_decision (the
 * RMS amplitude equals sqrt(average power / modes)). */
FOCSS_API focss_status focss_find_certainty(focss_ctx* ctx, const focss_field* tx, const focss_field* rx,
                                           double* certainty);
FOCSS_API focss_status focss_certainty_decision(focss_ctx* ctx, const focss_field* in, double certainty,
                                               focss_field* out);
/* hd_sequence_16qam (src/focss/processing/modulation.cpp:148-156): codes is a
 * host int32 array of batch*modes*samples. */
FOCSS_API focss_status focss_hd_codes(focss_ctx* ctx, const focss_field* in, int32_t* codes);
/* Decision error counts behind bit_error_rate_16qam / symbol_error_rate_16qam
 * (src/focss/processing/modulation.cpp:158-223), over samples [cut, samples-cut). */
FOCSS_API focss_status focss_error_counts(focss_ctx* ctx, const focss_field* tx, const focss_field* rx, int cut,
                                          uint64_t* bit_errors, uint64_t* symbol_errors);
/* bit_error_rate_16qam (denominator 4*size - 8*cut, :200-201) and
 * symbol_error_rate_16qam (denominator size - modes*cut, :221-222). */
FOCSS_API focss_status focss_bit_error_rate(focss_ctx* ctx, const focss_field* tx, const focss_field* rx, int cut,
                                            double* ber);
FOCSS_API focss_status focss_symbol_error_rate(focss_ctx* ctx, const focss_field* tx, const focss_field* rx,
                                               int cut, double* ser);
/* q2_factor / evm2_factor (src/focss/functions.cpp:27-80), FP64 sums. */
FOCSS_API focss_status focss_q2_factor(focss_ctx* ctx, const focss_field* tx, const focss_field* rx, int cut,
                                       double* q2);
/* PhaseShiftEqualizer::estimate (src/focss/equalizer/phase_shift_equalizer.cpp:30-46):
 * argmax over the angle grid 2 pi i / angle_steps of q2(desired, actual e^{i angle}). */
FOCSS_API focss_status focss_pse_estimate(focss_ctx* ctx, const focss_field* desired, const focss_field* actual,
                                          int angle_steps, double* angle);
/* ScalarEqualizer::estimate (src/focss/equalizer/scalar_equalizer.cpp:22-33):
 * sum conj(a) d / sum |a|^2; scalar is 2*batch doubles (re, im). */
FOCSS_API focss_status focss_scalar_estimate(focss_ctx* ctx, const focss_field* desired, const focss_field* actual,
                                             double* scalar);
/* Field * i_exp(angle[b]) and Field * scalar[b] per realization
 * (PhaseShiftEqualizer::equalize :17-19, ScalarEqualizer::equalize :12-14). */
FOCSS_API focss_status focss_field_rotate(focss_ctx* ctx, focss_field* field, const double* angle);
FOCSS_API focss_status focss_field_scale_each(focss_ctx* ctx, focss_field* field, const double* scalar);

/* ---------------------------------------- perturbation (triplet) equalizer */
/* SINO::cubic (src/focss/equalizer/sino.cpp:161-171, 203-220) over an
 * explicit term list: out[mode][k] = sum_i C_i A_mode[k+m_i]
 * sum_p A_p[k+n_i] conj(A_p[k+m_i+n_i]) for k in [radius, samples-radius),
 * zero elsewhere.  Samples outside the field count as zero (box-shaped term
 * sets are accepted as well as the reference's |m|+|n| <= radius diamond).
 * coef: n_terms complex (interleaved FP64 on the host, complex64 on the
 * device); duplicate (m, n) entries add.  |m|, |n| <= 4096.  1 or 2 modes. */
FOCSS_API focss_status focss_triplet_apply(focss_ctx* ctx, const focss_field* in, int radius, int n_terms,
                                           const int32_t* m, const int32_t* n, const double* coef,
                                           focss_field* out);
/* SINO::equalize (src/focss/equalizer/sino.cpp:193-196):
 * out = (rx - cubic(tx)) / linear_weight. */
FOCSS_API focss_status focss_sino_equalize(focss_ctx* ctx, const focss_field* rx, const focss_field* tx, int radius,
                                           int n_terms, const int32_t* m, const int32_t* n, const double* coef,
                                           double linear_weight_re, double linear_weight_im, focss_field* out);

/* Normal equations of SINO::train (src/focss/equalizer/sino.cpp:42-159) on the
 * device: the symmetry-reduced triplet features of tx (|m| <= R/2,
 * |m| <= n <= R-|m|, plus tx itself for type 0 = ORDINARY) over the samples
 * [R, N-R) of every mode, z-scored per feature (mean, standard deviation
 * normalized by the count), and the responses rx (type 1 = FIXED: rx - lw*tx;
 * type 2 = HOMOGENEOUS: rx) centred, appended as column nf.  Outputs:
 * gram = [Z y]^H [Z y] (FP32 products, 16-sample runs accumulated to ~48
 * bits, returned as FP64), (nf+1) x (nf+1) complex
 * (interleaved FP64) row-major, upper triangle valid; mean = nf+1 complex means (interleaved FP64, the last one the
 * responses'); sd = nf standard deviations.  nf = focss_sino_num_features.
 * tx and rx: single realizations of one domain.  The caller solves
 * gram[:nf,:nf] w = gram[:nf,nf] (FP64) and unscales as sino.cpp:122-153. */
FOCSS_API int focss_sino_num_features(int radius, int type);
FOCSS_API focss_status focss_sino_gram(focss_ctx* ctx, const focss_field* tx, const focss_field* rx, int radius,
                                       int type, double lw_re, double lw_im, double* gram, double* mean, double* sd);
/* Iterative refinement of that fit: r = Z^H (y - Z x) in FP64 for the same
 * z-scored design Z and centred responses y that focss_sino_gram forms
 * (rebuilt deterministically), x and r nf complex128 in the z-scored basis.
 * Solving G d = r with the Gram matrix and taking x + d converges to the
 * FP64 normal-equations solution of the design even where the Gram matrix's
 * FP32 chunk sums are too coarse for an ill-conditioned fit. */
FOCSS_API focss_status focss_sino_residual(focss_ctx* ctx, const focss_field* tx, const focss_field* rx, int radius,
                                           int type, double lw_re, double lw_im, const double* x, double* r);

/* WdmPPE (src/focss/equalizer/wdm_sino.h:8-71, wdm_sino.cpp): the
 * dual-polarization WDM perturbation equalizer.  Its fields are 6-row
 * realizations, rows channel * 2 + polarization: left neighbour 0-1, centre
 * 2-3, right neighbour 4-5 (the dataset layout of
 * src/tasks/wdm_scoring.cpp:79-103); its outputs are 2-row (the centre
 * channel).
 * focss_wdm_ppe_num_features: wdm_sino.cpp:32-34 (SPM triangle of c_radius,
 * XPM diamond of d_radius, the linear term; a radius of -1 drops that group).
 * focss_wdm_ppe_gram: the normal equations of WdmPPE::train
 * (wdm_sino.cpp:28-98) for one realization, in the layout of
 * focss_sino_gram: gram = [Z y]^H [Z y] of the z-scored features Z (SPM, XPM
 * T1(m,n) + T3(m,-n), transmitted centre sample) with the centred responses
 * y (rx rows 2-3, or rows 0-1 of a 2-row rx) over samples [R, N-R), R =
 * max(c_radius, d_radius), both polarizations stacked; complex128
 * (nf+1)^2, upper triangle valid; mean = nf+1 complex128 column means; sd =
 * nf standard deviations (normalized by the count).
 * focss_wdm_ppe_apply: with C ((2c+1)^2 complex128, C[(c+m)(2c+1) + c+n])
 * and D ((2d+1)^2, likewise) the trained tables and a the linear weight,
 *   noise = spm(spm_in) + xpm(xpm_in)       (null inputs contribute nothing)
 *   out   = (rx_centre - noise) / a          if rx       (equalize, :240-249)
 *         = a * lin_in_centre + noise        if lin_in   (model, :235-238)
 *         = noise                            otherwise   (spm / xpm / cubic). */
FOCSS_API int focss_wdm_ppe_num_features(int c_radius, int d_radius);
FOCSS_API focss_status focss_wdm_ppe_gram(focss_ctx* ctx, const focss_field* tx, const focss_field* rx,
                                          int c_radius, int d_radius, double* gram, double* mean, double* sd);
/* The same refinement residual for the WdmPPE design. */
FOCSS_API focss_status focss_wdm_ppe_residual(focss_ctx* ctx, const focss_field* tx, const focss_field* rx,
                                              int c_radius, int d_radius, const double* x, double* r);
FOCSS_API focss_status focss_wdm_ppe_apply(focss_ctx* ctx, const focss_field* spm_in, const focss_field* xpm_in,
                                           const focss_field* rx, const focss_field* lin_in, int c_radius,
                                           const double* C, int d_radius, const double* D, double lw_re,
                                           double lw_im, focss_field* out);

/* ---------------------------------------------------------- learned DBP */
/* No reference counterpart: a few-step learned replacement of
 * backward_propagation (src/tasks/systems.cpp:73-91).  Per realization (one
 * mode, `samples` at 2 samples/symbol): for each span, x *= span_scale
 * (drop_power), then steps_per_span x [circular FIR of `taps` complex taps,
 * x *= exp(i xi |x|^2)]; then a matched FIR of `mf_taps` taps and symbols =
 * y[0::2].  FIR(x, h)[n] = sum_t h[t] x[(n + t - (T-1)/2) mod samples].
 * Parameters (float, host layout): [taps: spans*steps*taps complex]
 * [xi: spans*steps, padded to an even count][matched taps: mf_taps complex].
 * Training: focss_ldbp_loss_grad runs forward and backward (hand-written
 * kernels, Wirtinger gradients dL/dconj(z)) for L = mean |symbols - tx|^2;
 * focss_ldbp_adam_step updates the parameters on the device. */
typedef struct focss_ldbp focss_ldbp;
FOCSS_API focss_status focss_ldbp_create(focss_ctx* ctx, int spans, int steps_per_span, int taps, int mf_taps,
                                         int samples, int batch, double span_scale, focss_ldbp** out);
FOCSS_API focss_status focss_ldbp_destroy(focss_ldbp* model);
FOCSS_API int focss_ldbp_num_params(const focss_ldbp* model);
FOCSS_API focss_status focss_ldbp_set_params(focss_ldbp* model, const float* params, int n);
FOCSS_API focss_status focss_ldbp_get_params(focss_ldbp* model, float* params, float* grads, int n);
FOCSS_API focss_status focss_ldbp_forward(focss_ldbp* model, const focss_field* in, focss_field* symbols);
FOCSS_API focss_status focss_ldbp_loss_grad(focss_ldbp* model, const focss_field* in, const focss_field* tx,
                                            double* loss);
/* Adam step; `lr` for the filter taps, `lr_gain` for the nonlinear gains
 * (their scale, kappa*gamma*h ~ 10^1 /W, differs from the taps' ~ 10^-1). */
FOCSS_API focss_status focss_ldbp_adam_step(focss_ldbp* model, double lr, double lr_gain, double beta1,
                                            double beta2, double eps);

/* No reference counterpart: the convolutional correction stage after the
 * learned DBP.  z = y + s (d_re + i d_im) with d = a 4-layer 1D CNN
 * (64 channels, kernel 9, ReLU, zero padding) of x = [Re y/s, Im y/s] and
 * optional perturbation triplets of y (focss_cnn_set_triplets);
 * BF16 weights (FP32 masters), FP32 accumulation on the tensor cores.
 * y, z, tx: fields of `length` symbols x `batch`, one mode.
 * Parameters (float): per layer l = 1..4 W_l[cout][9][cin] then b_l[cout],
 * with (cin, cout) = (16, 64), (64, 64), (64, 64), (64, 16); input channels
 * beyond the triplets and output channels 2..15 are padding. */
typedef struct focss_cnn focss_cnn;
FOCSS_API focss_status focss_cnn_create(focss_ctx* ctx, int channels, int kernel, int length, int batch,
                                        double input_scale, focss_cnn** out);
FOCSS_API focss_status focss_cnn_destroy(focss_cnn* model);
FOCSS_API int focss_cnn_num_params(const focss_cnn* model);
/* First-order perturbation triplets as further input channels (no reference
 * counterpart; the terms are those of SINO::term, src/focss/equalizer/
 * sino.cpp:161-171): input channels 2+2j and 3+2j (j < count <= 7) carry
 * Re and Im of (T(m_j, n_j) + T(-m_j, -n_j)) / input_scale^3, T(0, 0) alone
 * for m_j = n_j = 0, with T(m, n)[k] = y[k+m] y[k+n] conj(y[k+m+n]) and
 * symbols outside the realization counting as zero.  count = 0 (the default)
 * leaves those channels zero.  |m_j|, |n_j| <= length. */
FOCSS_API focss_status focss_cnn_set_triplets(focss_cnn* model, int count, const int32_t* m, const int32_t* n);
FOCSS_API focss_status focss_cnn_set_params(focss_cnn* model, const float* params, int n);
FOCSS_API focss_status focss_cnn_get_params(focss_cnn* model, float* params, float* grads, int n);
FOCSS_API focss_status focss_cnn_forward(focss_cnn* model, const focss_field* y, focss_field* z);
FOCSS_API focss_status focss_cnn_loss_grad(focss_cnn* model, const focss_field* y, const focss_field* tx,
                                           double* loss);
FOCSS_API focss_status focss_cnn_adam_step(focss_cnn* model, double lr, double beta1, double beta2, double eps);

/* ------------------------------------------------- allocation-free SSFM */
/* No counterpart in the reference.  SSFM::run on every realization, like
 * focss_ssfm_run, for callers that cannot let a library allocate device
 * memory: frameworks that own the device heap through their own pool,
 * latency-critical loops where an allocation and the synchronization it
 * implies are not allowed, or processes with a fixed device-memory budget.
 * It always uses the balanced two-pass FFT split; where focss_set_fft_split
 * or focss_autotune chose another split (or the single-CTA kernel) for
 * focss_ssfm_run, the two fields agree to FP32 rounding, not bit for bit.
 * `data` is the caller's device buffer of batch*samples complex64
 * (interleaved float pairs), propagated in place on `stream` (a
 * cudaStream_t; NULL = legacy default stream).  The library allocates
 * nothing: step state and twiddle tables live in one fixed 59 KB
 * __device__ array per device, held until the process exits.
 * Limits: samples a power of two in [2^8, 2^17], batch <= 256; larger shapes
 * return FOCSS_ERR_UNSUPPORTED before any GPU work.  Single-mode fields only.
 * The first call on a device looks up that array's device address (a
 * one-time set-up); make that first call before any stream capture.  Every
 * call shares the array, so calls that overlap on the GPU race.  Each call
 * synchronizes `stream` before it returns (ADAPTIVE and LOGARITHMIC grids
 * also poll a step counter from the host while they run). */
FOCSS_API focss_status focss_ssfm_run_noalloc(void* stream, void* data, int samples, int batch, double time_step,
                                              const focss_fiber* fiber, const focss_ssfm_opts* opts,
                                              double direction, int* steps_out);

/* ------------------------------------------------------- instrumentation */
/* No reference counterpart (the reference only prints progress to std::cout,
 * src/focss/solver/ssfm.cpp:117).
 * When enabled, each split-step column/row pass launch is bracketed by CUDA
 * events on the context stream; focss_profile_read returns the accumulated
 * device time and launch counts per pass kind (and resets them if asked). */
FOCSS_API focss_status focss_profile_enable(focss_ctx* ctx, int enable);
FOCSS_API focss_status focss_profile_read(focss_ctx* ctx, double* col_ms, long long* col_launches,
                                          double* row_ms, long long* row_launches, int reset);
/* FP32 FMA throughput of this GPU (TFLOP/s, 2 flops per FMA), measured by a
 * micro-kernel of independent FMA chains over whole waves of CTAs, best of 3
 * timed launches; the denominator for FP32-bound kernels such as the triplet
 * sum.  Changes no device setting. */
FOCSS_API focss_status focss_measure_fp32_fma(focss_ctx* ctx, double* tflops);
/* Total kernel launches issued by this library in this process. */
FOCSS_API long long focss_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* FOCSS_GPU_H_ */
