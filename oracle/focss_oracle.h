/*
 * focss_oracle.h -- FP64 CPU restatement of the focss SSFM / DBP / DSP /
 * perturbation-equalizer path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: it is loaded by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, never
 * by the product library (libfocss_gpu), which has no CPU fallback.
 *
 * Every function restates one reference function and names it (file:line,
 * paths relative to the focss source tree).  Complex data is interleaved
 * (re, im) doubles in the reference's mode-major order:
 * data[2*(sample + mode*samples) + {0,1}]  (src/focss/field.cpp:140-155).
 *
 * Parity pins: the restatement is checked in tests/test_oracle_pins.py against
 * golden vectors produced by the reference's own sources (compiled against a
 * project-written FFTW-API shim, see oracle/build_ref.py), committed under
 * tests/golden/.  The triplet sum (SINO::cubic) cannot be built from the
 * reference (it needs Armadillo); it is pinned against a literal pure-Python
 * loop restatement instead.
 */
#ifndef FOCSS_ORACLE_H_
#define FOCSS_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double alpha;       /* [1/m] power attenuation (natural units)      */
    double beta2;       /* [s^2/m]                                      */
    double gamma;       /* [1/W/m]                                      */
    double length;      /* [m]                                          */
    double wavelength;  /* [m]                                          */
    double kappa;       /* [1] polarization coupling factor             */
} ofc_fiber;            /* src/focss/module/fiber.h:5-12 */

enum { OFC_UNIFORM = 0, OFC_LOGARITHMIC = 1, OFC_ADAPTIVE = 2 }; /* ssfm.cpp:6-8 */

/* ---- FFT (FFTW conventions: sign -1 = FFTW_FORWARD = e^{-2 pi i jk/n}, unnormalized) */
void ofc_dft(int n, double* x, int sign);
void ofc_field_fft(int modes, int samples, double* a);   /* field.cpp:343-347 (x 1/N) */
void ofc_field_ifft(int modes, int samples, double* a);  /* field.cpp:349-352 */

/* ---- SSFM (src/focss/solver/ssfm.cpp:39-172).  Returns the number of
 * nonlinear steps taken (adaptive: the reference's printed steps_done). */
int ofc_ssfm_run(int modes, int samples, double dt, double* a,
                 const ofc_fiber* fiber, int grid, int total_steps,
                 double max_phase_shift, double max_step_size,
                 double direction);

/* The same, also writing the nonlinear step sizes |h_i| to h_out[i] (i < h_cap;
 * h_out may be NULL). */
int ofc_ssfm_run_rec(int modes, int samples, double dt, double* a,
                     const ofc_fiber* fiber, int grid, int total_steps,
                     double max_phase_shift, double max_step_size,
                     double direction, double* h_out, int h_cap);
/* The ADAPTIVE loop (ssfm.cpp:92-118) on the given step sizes h[0..n_steps). */
int ofc_ssfm_run_steps(int modes, int samples, double dt, double* a,
                       const ofc_fiber* fiber, const double* h, int n_steps,
                       double direction);

/* Fiber transforms (src/focss/module/fiber.cpp:4-45). */
ofc_fiber ofc_fiber_scale(ofc_fiber f, double length_factor);
ofc_fiber ofc_fiber_dispersive(ofc_fiber f);

/* Span drivers (src/tasks/systems.cpp:63-91), oracle-side. */
void ofc_cd_compensation(int modes, int samples, double dt, double* a,
                         const ofc_fiber* fiber, int spans);

/* ---- Amplifier (src/focss/module/amplifier.cpp:15-42).  Noise is drawn from
 * the counter-based Philox4x32-10 stream shared with the GPU (the reference's
 * std::normal_distribution on default_random_engine cannot be matched). */
void ofc_amplify(int modes, int samples, double dt, double f0, double* a,
                 double gain, double noise_factor, uint64_t seed,
                 uint64_t counter, int realization);
void ofc_add_noise(int modes, int samples, double dt, double f0, double* a,
                   double gain, double noise_factor, uint64_t seed,
                   uint64_t counter, int realization);
void ofc_drop_power(int modes, int samples, double* a, double gain);
void ofc_give_power(int modes, int samples, double* a, double gain);
void ofc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]);
void ofc_gaussian_pair(uint32_t x0, uint32_t x1, double* z0, double* z1);

/* ---- Modulation / DSP (src/focss/processing/modulation.cpp) */
void ofc_gray16(double* table);                          /* :9-17, 16 complex */
void ofc_qam16_map(int n, const int32_t* codes, double* out);
void ofc_rrc_pulse(int n_symbols, int osf, double roll_off, double* out); /* :47-74 */
void ofc_filter_inplace(int modes, int samples, double* a, int h_len,
                        const double* h);                /* field.cpp:358-372 */
void ofc_upsample(int modes, int samples, const double* a, int factor,
                  double* out);                           /* field.cpp:272-283 */
void ofc_downsample(int modes, int samples, const double* a, int factor,
                    double* out);                         /* field.cpp:285-297 */
void ofc_decimate(int modes, int samples, const double* a, int factor,
                  double* out);                           /* field.cpp:299-320 */
void ofc_rrc_shaping(int modes, int n_symbols, const double* symbols, int osf,
                     double roll_off, double gain, double* out);     /* :85-90 */
void ofc_rrc_sampling(int modes, int samples, const double* signal, int osf,
                      double roll_off, double gain, double* out);    /* :92-96 */
uint32_t ofc_demodulate16(double re, double im);          /* :98-110 */
void ofc_hd_sequence(int modes, int samples, const double* a, int32_t* codes);
void ofc_hard_decision(int modes, int samples, const double* a, double* out);
void ofc_soft_decision(int modes, int samples, const double* a, double uncertainty, double* out);
double ofc_find_certainty(int rows, int cols, const double* tx, const double* rx);
void ofc_certainty_decision(int rows, int cols, const double* a, double certainty, double* out);
void ofc_hd_rms(int rows, int cols, const double* a, double* out);
void ofc_error_counts(int modes, int samples, const double* tx,
                      const double* rx, int cut, uint64_t* bit_errors,
                      uint64_t* symbol_errors);
double ofc_bit_error_rate(int modes, int samples, const double* tx,
                          const double* rx, int cut);     /* :158-202 */
double ofc_symbol_error_rate(int modes, int samples, const double* tx,
                             const double* rx, int cut);  /* :204-223 */
double ofc_evm2(int modes, int samples, const double* tx, const double* rx,
                int cut);                                 /* functions.cpp:27-67 */
double ofc_q2(int modes, int samples, const double* tx, const double* rx,
              int cut);                                   /* functions.cpp:69-80 */
double ofc_average_power(int modes, int samples, const double* a);
double ofc_peak_power(int modes, int samples, const double* a);
void ofc_frequency_shift(int modes, int samples, double dt, double* a,
                         double frequency);               /* :255-264 */
void ofc_bandpass(int modes, int samples, double dt, double* a,
                  double frequency);                      /* :266-277 */
void ofc_wdm_select(int modes, int samples, double dt, double* a,
                    int channel_index, double channel_bandwidth); /* :248-253 */
void ofc_wdm_mux(int n_channels, int modes, int samples, double dt,
                 const double* channels, double channel_bandwidth,
                 double* out);                            /* :225-235 */

/* ---- Linear equalizers (src/focss/equalizer/phase_shift_equalizer.cpp:30-46,
 * scalar_equalizer.cpp:22-33) */
double ofc_pse_estimate(int modes, int samples, const double* desired,
                        const double* actual, int angle_steps);
void ofc_rotate(int modes, int samples, double* a, double angle);
void ofc_scalar_estimate(int modes, int samples, const double* desired,
                         const double* actual, double* scalar);

/* ---- Perturbation (triplet) equalizer (src/focss/equalizer/sino.cpp:161-220)
 * weights: (2R+1)x(2R+1) complex, weights[(m+R)*(2R+1) + (n+R)].
 * Output rows k in [R, samples-R) are written, others are zero. */
void ofc_sino_cubic(int modes, int samples, const double* a, int radius,
                    const double* weights, double* out);
/* Sparse form over an explicit term list (m_i, n_i, C_i), any |m|,|n| <= R,
 * over the same k range as SINO::cubic. */
void ofc_triplet_sparse(int modes, int samples, const double* a, int radius,
                        int n_terms, const int32_t* m, const int32_t* n,
                        const double* c, double* out);

/* ---- Batched helpers used by the CPU baseline (OpenMP over realizations). */
int ofc_num_threads(void);
void ofc_ssfm_batch(int batch, int modes, int samples, double dt, double* a,
                    const ofc_fiber* fiber, int grid, int total_steps,
                    double max_phase_shift, double max_step_size,
                    double direction, int threads, int* steps);
/* A bounded number of uniform split steps (L(h) N(h) pairs with FFTs) for
 * timing; the same work per sample-step as uniform_solve. */
void ofc_uniform_steps_batch(int batch, int modes, int samples, double dt,
                             double* a, const ofc_fiber* fiber, double step,
                             int n_steps, int threads);

#ifdef __cplusplus
}
#endif
#endif
