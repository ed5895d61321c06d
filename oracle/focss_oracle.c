/*
 * focss_oracle.c -- FP64 CPU restatement of the focss hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path, and the timed CPU
 * baseline in bench.py.  Nothing in the product library links or calls it.
 *
 * Each function follows the reference function cited beside it (paths are
 * relative to the focss source tree) with the same operation order, so that
 * FP64 results agree with the reference's own code to rounding.
 */
#include "focss_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* definitions.h:13-15 */
static const double REF_PI = 3.14159265358979323846264338;
static const double REF_PLANCK = 6.62607004081818181818181e-34;

/* ------------------------------------------------------------------------ */
/* FFT: iterative radix-2 for powers of two, direct DFT otherwise.           */
/* ------------------------------------------------------------------------ */
static pthread_mutex_t tw_lock = PTHREAD_MUTEX_INITIALIZER;
static double* tw_cache[40];

static const double* twiddles(int log2n) {
    pthread_mutex_lock(&tw_lock);
    if (!tw_cache[log2n]) {
        int n = 1 << log2n;
        double* t = (double*)malloc(sizeof(double) * (size_t)n);
        for (int k = 0; k < n / 2; ++k) {
            double ang = 2.0 * REF_PI * (double)k / (double)n;
            t[2 * k] = cos(ang);
            t[2 * k + 1] = -sin(ang);
        }
        tw_cache[log2n] = t;
    }
    const double* r = tw_cache[log2n];
    pthread_mutex_unlock(&tw_lock);
    return r;
}

static int ilog2_exact(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return ((1 << l) == n) ? l : -1;
}

void ofc_dft(int n, double* x, int sign) {
    if (n <= 1) return;
    int lg = ilog2_exact(n);
    if (lg < 0) {
        double* out = (double*)malloc(sizeof(double) * 2 * (size_t)n);
        for (int k = 0; k < n; ++k) {
            double sr = 0, si = 0;
            for (int j = 0; j < n; ++j) {
                double ang = sign * 2.0 * REF_PI * (double)(((long long)j * k) % n) / n;
                double c = cos(ang), s = sin(ang);
                sr += x[2 * j] * c - x[2 * j + 1] * s;
                si += x[2 * j] * s + x[2 * j + 1] * c;
            }
            out[2 * k] = sr;
            out[2 * k + 1] = si;
        }
        memcpy(x, out, sizeof(double) * 2 * (size_t)n);
        free(out);
        return;
    }
    /* bit reversal */
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double tr = x[2 * i], ti = x[2 * i + 1];
            x[2 * i] = x[2 * j];
            x[2 * i + 1] = x[2 * j + 1];
            x[2 * j] = tr;
            x[2 * j + 1] = ti;
        }
    }
    const double* tw = twiddles(lg);
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1, stride = n / len;
        for (int i = 0; i < n; i += len) {
            for (int j = 0; j < half; ++j) {
                double wr = tw[2 * j * stride], wi = tw[2 * j * stride + 1];
                if (sign > 0) wi = -wi;
                double* u = x + 2 * (i + j);
                double* v = x + 2 * (i + j + half);
                double vr = v[0] * wr - v[1] * wi;
                double vi = v[0] * wi + v[1] * wr;
                v[0] = u[0] - vr;
                v[1] = u[1] - vi;
                u[0] += vr;
                u[1] += vi;
            }
        }
    }
}

void ofc_field_fft(int modes, int samples, double* a) {
    for (int m = 0; m < modes; ++m) ofc_dft(samples, a + 2 * (size_t)m * samples, -1);
    double s = 1.0 / (double)samples;
    for (size_t i = 0; i < 2 * (size_t)modes * samples; ++i) a[i] *= s;
}

void ofc_field_ifft(int modes, int samples, double* a) {
    for (int m = 0; m < modes; ++m) ofc_dft(samples, a + 2 * (size_t)m * samples, +1);
}

/* ------------------------------------------------------------------------ */
/* Small helpers                                                             */
/* ------------------------------------------------------------------------ */
static inline void cmul_inplace(double* z, double c, double s) {
    double r = z[0] * c - z[1] * s;
    double i = z[0] * s + z[1] * c;
    z[0] = r;
    z[1] = i;
}

static void scale(size_t n_complex, double* a, double s) {
    for (size_t i = 0; i < 2 * n_complex; ++i) a[i] *= s;
}

/* Field::power(sample): sum over modes of |A|^2 (field.cpp:164-171) */
static double power_at(int modes, int samples, const double* a, int sample) {
    double p = 0;
    for (int m = 0; m < modes; ++m) {
        const double* z = a + 2 * ((size_t)sample + (size_t)m * samples);
        p += z[0] * z[0] + z[1] * z[1];
    }
    return p;
}

double ofc_average_power(int modes, int samples, const double* a) {
    double p = 0;
    for (size_t i = 0; i < (size_t)modes * samples; ++i)
        p += a[2 * i] * a[2 * i] + a[2 * i + 1] * a[2 * i + 1];
    return p / samples; /* field.cpp:181-187 */
}

double ofc_peak_power(int modes, int samples, const double* a) {
    double pk = 0; /* field.cpp:173-179 */
    for (int i = 0; i < samples; ++i) {
        double p = power_at(modes, samples, a, i);
        if (pk < p) pk = p;
    }
    return pk;
}

/* ------------------------------------------------------------------------ */
/* SSFM (ssfm.cpp)                                                           */
/* ------------------------------------------------------------------------ */
typedef struct {
    int modes, samples;
    const ofc_fiber* f;
    const double* disp;
    double max_phase, max_step;
} ssfm_ctx;

static void nofft_linear_step(const ssfm_ctx* c, double* a, double step) {
    /* ssfm.cpp:152-158 */
    scale((size_t)c->modes * c->samples, a, exp(-0.5 * c->f->alpha * step));
    double argument = 0.5 * c->f->beta2 * step;
    size_t size = (size_t)c->modes * c->samples;
    for (size_t i = 0; i < size; ++i) {
        double ph = argument * c->disp[i % c->samples];
        cmul_inplace(a + 2 * i, cos(ph), sin(ph));
    }
}

static void linear_step(const ssfm_ctx* c, double* a, double step) {
    /* ssfm.cpp:142-150 */
    scale((size_t)c->modes * c->samples, a, exp(-0.5 * c->f->alpha * step));
    ofc_field_fft(c->modes, c->samples, a);
    double argument = 0.5 * c->f->beta2 * step;
    size_t size = (size_t)c->modes * c->samples;
    for (size_t i = 0; i < size; ++i) {
        double ph = argument * c->disp[i % c->samples];
        cmul_inplace(a + 2 * i, cos(ph), sin(ph));
    }
    ofc_field_ifft(c->modes, c->samples, a);
}

static void nonlinear_step(const ssfm_ctx* c, double* a, double step) {
    /* ssfm.cpp:160-164 */
    double argument = c->f->kappa * c->f->gamma * step;
    size_t size = (size_t)c->modes * c->samples;
    for (size_t i = 0; i < size; ++i) {
        double ph = argument * power_at(c->modes, c->samples, a, (int)(i % c->samples));
        cmul_inplace(a + 2 * i, cos(ph), sin(ph));
    }
}

static void fft_nonlinear_step(const ssfm_ctx* c, double* a, double step) {
    /* ssfm.cpp:166-172 */
    ofc_field_ifft(c->modes, c->samples, a);
    nonlinear_step(c, a, step);
    ofc_field_fft(c->modes, c->samples, a);
}

static double next_adaptive_step(const ssfm_ctx* c, const double* a) {
    /* ssfm.cpp:136-140 */
    double argument = fabs(c->f->kappa * c->f->gamma);
    double phase_shift = argument * ofc_peak_power(c->modes, c->samples, a);
    double h = c->max_phase / phase_shift;
    return c->max_step < h ? c->max_step : h;
}

static int logarithmic_steps(const ssfm_ctx* c, const double* a) {
    /* ssfm.cpp:120-134 */
    double alpha = c->f->alpha;
    double L_nl = 1.0 / c->f->gamma / ofc_average_power(c->modes, c->samples, a);
    double CL_nl_kappa = c->max_phase * L_nl / c->f->kappa;
    double L_eff = (1.0 - exp(-alpha * c->f->length)) / alpha;
    double L_nl_eff = (1.0 - exp(-alpha * CL_nl_kappa)) / alpha;
    int estimated = (int)(L_eff / L_nl_eff);
    int minimum = (int)(c->f->length / c->max_step);
    return minimum > estimated ? minimum : estimated;
}

static double* dispersion_cache(int samples, double dt) {
    /* ssfm.cpp:39-60: dispersion cache omega_k^2 in FFT order */
    double freq_step = 2.0 * REF_PI / (dt * samples);
    double* disp = (double*)malloc(sizeof(double) * (size_t)samples);
    for (int i = 0; i <= samples / 2; ++i) disp[i] = (double)i * freq_step;
    for (int i = samples / 2 + 1; i < samples; ++i) disp[i] = (double)(i - samples) * freq_step;
    for (int i = 0; i < samples; ++i) disp[i] *= disp[i];
    return disp;
}

static void record_step(double* h_out, int h_cap, int i, double step) {
    if (h_out && i < h_cap) h_out[i] = step;
}

int ofc_ssfm_run(int modes, int samples, double dt, double* a,
                 const ofc_fiber* fiber, int grid, int total_steps,
                 double max_phase_shift, double max_step_size,
                 double direction) {
    return ofc_ssfm_run_rec(modes, samples, dt, a, fiber, grid, total_steps, max_phase_shift,
                            max_step_size, direction, NULL, 0);
}

int ofc_ssfm_run_steps(int modes, int samples, double dt, double* a,
                       const ofc_fiber* fiber, const double* h, int n_steps,
                       double direction) {
    /* The ADAPTIVE loop of ssfm.cpp:92-118 with its step sizes taken from h
     * instead of next_adaptive_step: the same operations in the same order, so
     * replaying an ADAPTIVE run's recorded steps reproduces it bit for bit. */
    double* disp = dispersion_cache(samples, dt);
    ssfm_ctx c = {modes, samples, fiber, disp, 0.0, 0.0};
    ofc_field_fft(modes, samples, a);
    for (int i = 0; i + 1 < n_steps; ++i) {
        double step = h[i];
        nofft_linear_step(&c, a, 0.5 * step * direction);
        ofc_field_ifft(modes, samples, a);
        nonlinear_step(&c, a, step * direction);
        ofc_field_fft(modes, samples, a);
        nofft_linear_step(&c, a, 0.5 * step * direction);
    }
    double step = h[n_steps - 1];
    nofft_linear_step(&c, a, 0.5 * step * direction);
    fft_nonlinear_step(&c, a, step * direction);
    nofft_linear_step(&c, a, 0.5 * step * direction);
    ofc_field_ifft(modes, samples, a);
    free(disp);
    return n_steps;
}

int ofc_ssfm_run_rec(int modes, int samples, double dt, double* a,
                     const ofc_fiber* fiber, int grid, int total_steps,
                     double max_phase_shift, double max_step_size,
                     double direction, double* h_out, int h_cap) {
    double* disp = dispersion_cache(samples, dt);
    ssfm_ctx c = {modes, samples, fiber, disp, max_phase_shift, max_step_size};
    int steps = 0;
    if (grid == OFC_UNIFORM) {
        /* ssfm.cpp:62-72 */
        double step = fiber->length / total_steps;
        step = direction * step;
        linear_step(&c, a, 0.5 * step);
        for (int i = 0; i < total_steps; ++i) {
            record_step(h_out, h_cap, i, fabs(step));
            nonlinear_step(&c, a, step);
            linear_step(&c, a, step);
        }
        linear_step(&c, a, -0.5 * step);
        steps = total_steps;
    } else if (grid == OFC_LOGARITHMIC) {
        /* ssfm.cpp:74-90 */
        int n_steps = logarithmic_steps(&c, a);
        double inv_alpha = -1.0 / fiber->alpha * direction;
        double inv_gain = exp(-fiber->alpha * fiber->length) - 1;
        inv_gain /= n_steps;
        ofc_field_fft(modes, samples, a);
        for (int i = 0; i < n_steps; ++i) {
            double step = inv_alpha * log(1 + inv_gain / (1 + inv_gain * i));
            record_step(h_out, h_cap, i, fabs(step));
            nofft_linear_step(&c, a, 0.5 * step);
            fft_nonlinear_step(&c, a, step);
            nofft_linear_step(&c, a, 0.5 * step);
        }
        ofc_field_ifft(modes, samples, a);
        steps = n_steps;
    } else {
        /* ssfm.cpp:92-118 */
        double distance = 0;
        double next_step = next_adaptive_step(&c, a);
        double step = next_step;
        int steps_done = 1;
        ofc_field_fft(modes, samples, a);
        while (distance + step < fiber->length) {
            record_step(h_out, h_cap, steps_done - 1, step);
            nofft_linear_step(&c, a, 0.5 * step * direction);
            ofc_field_ifft(modes, samples, a);
            nonlinear_step(&c, a, step * direction);
            next_step = next_adaptive_step(&c, a);
            ofc_field_fft(modes, samples, a);
            nofft_linear_step(&c, a, 0.5 * step * direction);
            distance += step;
            step = next_step;
            steps_done++;
        }
        step = fiber->length - distance;
        record_step(h_out, h_cap, steps_done - 1, step);
        nofft_linear_step(&c, a, 0.5 * step * direction);
        fft_nonlinear_step(&c, a, step * direction);
        nofft_linear_step(&c, a, 0.5 * step * direction);
        ofc_field_ifft(modes, samples, a);
        steps = steps_done;
    }
    free(disp);
    return steps;
}

ofc_fiber ofc_fiber_scale(ofc_fiber f, double length_factor) {
    /* fiber.cpp:32-45 */
    ofc_fiber g = f;
    if (length_factor >= 0) {
        g.length *= length_factor;
    } else {
        g.alpha = -f.alpha;
        g.beta2 = -f.beta2;
        g.gamma = -f.gamma;
        g.length *= -length_factor;
    }
    return g;
}

ofc_fiber ofc_fiber_dispersive(ofc_fiber f) {
    /* fiber.cpp:17-22 */
    f.alpha = 0;
    f.gamma = 0;
    return f;
}

void ofc_cd_compensation(int modes, int samples, double dt, double* a,
                         const ofc_fiber* fiber, int spans) {
    /* systems.cpp:63-71: SSFM(fiber.dispersive() * spans, 1).run(BACKWARD) */
    ofc_fiber f = ofc_fiber_scale(ofc_fiber_dispersive(*fiber), spans);
    ofc_ssfm_run(modes, samples, dt, a, &f, OFC_UNIFORM, 1, 0, 0, -1.0);
}

/* ------------------------------------------------------------------------ */
/* Counter-based noise: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel */
/* random numbers: as easy as 1, 2, 3", SC'11) + Box-Muller.                  */
/* ------------------------------------------------------------------------ */
void ofc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

void ofc_gaussian_pair(uint32_t x0, uint32_t x1, double* z0, double* z1) {
    /* u1 in (0, 1], u2 in [0, 1): 24-bit grids, exact in FP32 as well */
    double u1 = ((double)(x0 >> 8) + 0.5) * (1.0 / 16777216.0);
    double u2 = (double)(x1 >> 8) * (1.0 / 16777216.0);
    double r = sqrt(-2.0 * log(u1));
    double th = 2.0 * REF_PI * u2;
    *z0 = r * cos(th);
    *z1 = r * sin(th);
}

void ofc_add_noise(int modes, int samples, double dt, double f0, double* a,
                   double gain, double noise_factor, uint64_t seed,
                   uint64_t counter, int realization) {
    /* amplifier.cpp:20-28 */
    double variance = REF_PLANCK * f0;
    variance *= noise_factor * (gain - 1) / 2;
    variance *= 1.0 / dt;
    double sigma = sqrt(variance / 2);
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int m = 0; m < modes; ++m) {
        for (int s = 0; s < samples; ++s) {
            uint32_t ctr[4] = {(uint32_t)s, (uint32_t)(m + modes * realization),
                               (uint32_t)counter, (uint32_t)(counter >> 32)};
            uint32_t o[4];
            ofc_philox4x32_10(ctr, key, o);
            double z0, z1;
            ofc_gaussian_pair(o[0], o[1], &z0, &z1);
            double* z = a + 2 * ((size_t)s + (size_t)m * samples);
            z[0] += sigma * z0;
            z[1] += sigma * z1;
        }
    }
}

void ofc_amplify(int modes, int samples, double dt, double f0, double* a,
                 double gain, double noise_factor, uint64_t seed,
                 uint64_t counter, int realization) {
    /* amplifier.cpp:15-18 */
    scale((size_t)modes * samples, a, sqrt(gain));
    if (noise_factor != 0)
        ofc_add_noise(modes, samples, dt, f0, a, gain, noise_factor, seed, counter, realization);
}

void ofc_give_power(int modes, int samples, double* a, double gain) {
    scale((size_t)modes * samples, a, gain > 1 ? sqrt(gain) : sqrt(1 / gain)); /* :30-35 */
}

void ofc_drop_power(int modes, int samples, double* a, double gain) {
    scale((size_t)modes * samples, a, gain < 1 ? sqrt(gain) : sqrt(1 / gain)); /* :37-42 */
}

/* ------------------------------------------------------------------------ */
/* Modulation / DSP (modulation.cpp)                                         */
/* ------------------------------------------------------------------------ */
void ofc_gray16(double* t) {
    /* modulation.cpp:9-17: Gray-coded 16QAM, unit average power */
    static const int re[16] = {-3, -1, 3, 1, -3, -1, 3, 1, -3, -1, 3, 1, -3, -1, 3, 1};
    static const int im[16] = {-3, -3, -3, -3, -1, -1, -1, -1, 3, 3, 3, 3, 1, 1, 1, 1};
    double s = sqrt(10.0);
    for (int i = 0; i < 16; ++i) {
        t[2 * i] = (double)re[i] / s;
        t[2 * i + 1] = (double)im[i] / s;
    }
}

void ofc_qam16_map(int n, const int32_t* codes, double* out) {
    double t[32];
    ofc_gray16(t);
    for (int i = 0; i < n; ++i) {
        out[2 * i] = t[2 * (codes[i] & 15)];
        out[2 * i + 1] = t[2 * (codes[i] & 15) + 1];
    }
}

void ofc_rrc_pulse(int n_symbols, int osf, double roll_off, double* out) {
    /* modulation.cpp:47-74 */
    int len = n_symbols * osf;
    for (int i = 0; i < len; ++i) {
        double t = (double)i / osf - n_symbols / 2.0;
        double v = 0;
        if (t == 0) {
            v = 1 - roll_off + 4 * roll_off / REF_PI;
        } else if (fabs(t) == 1 / roll_off / 4) {
            v += (1 + 2 / REF_PI) * sin(REF_PI / roll_off / 4);
            v += (1 - 2 / REF_PI) * cos(REF_PI / roll_off / 4);
            v *= roll_off / sqrt(2.0);
        } else {
            v += cos(REF_PI * t * (1 + roll_off));
            v *= 4 * roll_off * t;
            v += sin(REF_PI * t * (1 - roll_off));
            v /= 1 - 16 * roll_off * roll_off * t * t;
            v /= REF_PI * t;
        }
        out[2 * i] = v;
        out[2 * i + 1] = 0;
    }
    double power = 0;
    for (int i = 0; i < len; ++i) power += out[2 * i] * out[2 * i] + out[2 * i + 1] * out[2 * i + 1];
    double g = (double)len / power;
    for (int i = 0; i < len; ++i) {
        out[2 * i] *= g;
        out[2 * i + 1] *= g;
    }
}

void ofc_filter_inplace(int modes, int samples, double* a, int h_len, const double* h) {
    /* field.cpp:358-372 */
    double* zp = (double*)calloc(2 * (size_t)samples, sizeof(double));
    int half = h_len / 2;
    int shift = samples - half;
    for (int i = 0; i < h_len / 2; ++i) {
        zp[2 * i] = h[2 * (i + half)];
        zp[2 * i + 1] = h[2 * (i + half) + 1];
        zp[2 * (shift + i)] = h[2 * i];
        zp[2 * (shift + i) + 1] = h[2 * i + 1];
    }
    ofc_field_fft(modes, samples, a);
    ofc_field_fft(1, samples, zp); /* focss::fft normalizes by size (functions.cpp:132-141) */
    for (int m = 0; m < modes; ++m)
        for (int s = 0; s < samples; ++s) {
            double* z = a + 2 * ((size_t)s + (size_t)m * samples);
            cmul_inplace(z, zp[2 * s], zp[2 * s + 1]);
        }
    ofc_field_ifft(modes, samples, a);
    free(zp);
}

void ofc_upsample(int modes, int samples, const double* a, int factor, double* out) {
    size_t size = (size_t)modes * samples;
    memset(out, 0, sizeof(double) * 2 * size * factor);
    for (size_t i = 0; i < size; ++i) {
        out[2 * factor * i] = a[2 * i];
        out[2 * factor * i + 1] = a[2 * i + 1];
    }
}

void ofc_downsample(int modes, int samples, const double* a, int factor, double* out) {
    size_t size = (size_t)modes * (samples / factor);
    for (size_t i = 0; i < size; ++i) {
        out[2 * i] = a[2 * i * factor];
        out[2 * i + 1] = a[2 * i * factor + 1];
    }
}

void ofc_decimate(int modes, int samples, const double* a, int factor, double* out) {
    int ds = samples / factor;
    double* spec = (double*)malloc(sizeof(double) * 2 * (size_t)modes * samples);
    memcpy(spec, a, sizeof(double) * 2 * (size_t)modes * samples);
    ofc_field_fft(modes, samples, spec);
    int cutoff = samples / factor / 2;
    int shift = samples - ds;
    for (int m = 0; m < modes; ++m) {
        for (int s = 0; s < cutoff; ++s) {
            out[2 * ((size_t)s + (size_t)m * ds)] = spec[2 * ((size_t)s + (size_t)m * samples)];
            out[2 * ((size_t)s + (size_t)m * ds) + 1] = spec[2 * ((size_t)s + (size_t)m * samples) + 1];
        }
        for (int s = cutoff; s < ds; ++s) {
            out[2 * ((size_t)s + (size_t)m * ds)] = spec[2 * ((size_t)s + shift + (size_t)m * samples)];
            out[2 * ((size_t)s + (size_t)m * ds) + 1] = spec[2 * ((size_t)s + shift + (size_t)m * samples) + 1];
        }
    }
    ofc_field_ifft(modes, ds, out);
    free(spec);
}

void ofc_rrc_shaping(int modes, int n_symbols, const double* symbols, int osf,
                     double roll_off, double gain, double* out) {
    /* modulation.cpp:85-90 with the roll-off as a parameter */
    int samples = n_symbols * osf;
    double* h = (double*)malloc(sizeof(double) * 2 * (size_t)samples);
    ofc_rrc_pulse(n_symbols, osf, roll_off, h);
    ofc_upsample(modes, n_symbols, symbols, osf, out);
    ofc_filter_inplace(modes, samples, out, samples, h);
    scale((size_t)modes * samples, out, sqrt(gain) * osf);
    free(h);
}

void ofc_rrc_sampling(int modes, int samples, const double* signal, int osf,
                      double roll_off, double gain, double* out) {
    /* modulation.cpp:92-96 */
    double* h = (double*)malloc(sizeof(double) * 2 * (size_t)samples);
    double* tmp = (double*)malloc(sizeof(double) * 2 * (size_t)modes * samples);
    ofc_rrc_pulse(samples / osf, osf, roll_off, h);
    memcpy(tmp, signal, sizeof(double) * 2 * (size_t)modes * samples);
    ofc_filter_inplace(modes, samples, tmp, samples, h);
    ofc_downsample(modes, samples, tmp, osf, out);
    scale((size_t)modes * (samples / osf), out, sqrt(gain));
    free(h);
    free(tmp);
}

uint32_t ofc_demodulate16(double re, double im) {
    /* modulation.cpp:98-110: argmin, ties to the lowest code */
    static double t[32];
    static int init = 0;
    if (!init) {
        ofc_gray16(t);
        init = 1;
    }
    uint32_t argmin = 0;
    double dr = re - t[0], di = im - t[1];
    double mn = dr * dr + di * di;
    for (uint32_t code = 1; code < 16; ++code) {
        dr = re - t[2 * code];
        di = im - t[2 * code + 1];
        double d = dr * dr + di * di;
        if (mn > d) {
            mn = d;
            argmin = code;
        }
    }
    return argmin;
}

void ofc_hd_sequence(int modes, int samples, const double* a, int32_t* codes) {
    /* modulation.cpp:148-156 */
    double sc = sqrt(modes / ofc_average_power(modes, samples, a));
    for (size_t i = 0; i < (size_t)modes * samples; ++i)
        codes[i] = (int32_t)ofc_demodulate16(sc * a[2 * i], sc * a[2 * i + 1]);
}

void ofc_hard_decision(int modes, int samples, const double* a, double* out) {
    /* modulation.cpp:112-120 */
    double t[32];
    ofc_gray16(t);
    double power = ofc_average_power(modes, samples, a) / modes;
    double sp = sqrt(power);
    for (size_t i = 0; i < (size_t)modes * samples; ++i) {
        uint32_t c = ofc_demodulate16(a[2 * i] / sp, a[2 * i + 1] / sp);
        out[2 * i] = sp * t[2 * c];
        out[2 * i + 1] = sp * t[2 * c + 1];
    }
}

void ofc_soft_decision(int modes, int samples, const double* a, double uncertainty, double* out) {
    /* modulation.cpp:122-146: hard decision per quadrature unless the received
     * value lies within sqrt(10)*uncertainty of a decision boundary (0, +-2/sqrt(10)),
     * in which case the received value is kept */
    double t[32];
    ofc_gray16(t);
    double power = ofc_average_power(modes, samples, a) / modes;
    double sp = sqrt(power);
    double pivot = 2.0 / sqrt(10);
    double threshold = sqrt(10) * uncertainty;
    for (size_t i = 0; i < (size_t)modes * samples; ++i) {
        double re = a[2 * i] / sp, im = a[2 * i + 1] / sp;
        uint32_t c = ofc_demodulate16(re, im);
        double gr = t[2 * c], gi = t[2 * c + 1];
        if (fabs(re) < threshold || fabs(re - pivot) < threshold || fabs(re + pivot) < threshold) gr = re;
        if (fabs(im) < threshold || fabs(im - pivot) < threshold || fabs(im + pivot) < threshold) gi = im;
        out[2 * i] = sp * gr;
        out[2 * i + 1] = sp * gi;
    }
}

/* Decisions of the WDM scoring task (src/tasks/wdm_scoring.cpp:105-156) on a
 * rows x cols matrix (rows = channel * modes + mode, row-major here).  The
 * amplitude scale is the matrix's RMS over all its elements (arma
 * norm(., "fro") / sqrt(n_elem)). */
static double fro2(size_t n, const double* a) {
    double p = 0;
    for (size_t i = 0; i < n; ++i) p += a[2 * i] * a[2 * i] + a[2 * i + 1] * a[2 * i + 1];
    return p;
}

double ofc_find_certainty(int rows, int cols, const double* tx, const double* rx) {
    /* wdm_scoring.cpp:105-126: the smallest distance from a wrongly decided
     * received sample to its decided point, capped at 1/sqrt(5), in units of
     * the transmitted RMS amplitude, times sqrt(5) */
    double t[32];
    ofc_gray16(t);
    const size_t n = (size_t)rows * cols;
    const double scale = sqrt((double)n) / sqrt(fro2(n, tx));
    double threshold = 1.0 / sqrt(5.0) / scale;
    for (size_t i = 0; i < n; ++i) {
        uint32_t tc = ofc_demodulate16(scale * tx[2 * i], scale * tx[2 * i + 1]);
        uint32_t rc = ofc_demodulate16(scale * rx[2 * i], scale * rx[2 * i + 1]);
        if (tc ^ rc) {
            double d = hypot(t[2 * rc] / scale - rx[2 * i], t[2 * rc + 1] / scale - rx[2 * i + 1]);
            if (threshold > d) threshold = d;
        }
    }
    return sqrt(5.0) * scale * threshold;
}

void ofc_certainty_decision(int rows, int cols, const double* a, double certainty, double* out) {
    /* wdm_scoring.cpp:128-144 ("sd"): a sample is replaced by its decided
     * point when it lies closer than certainty / sqrt(5) (RMS-normalized) */
    double t[32];
    ofc_gray16(t);
    const size_t n = (size_t)rows * cols;
    const double amp = sqrt(fro2(n, a)) / sqrt((double)n);
    const double threshold = certainty / sqrt(5.0);
    for (size_t i = 0; i < n; ++i) {
        double re = a[2 * i] / amp, im = a[2 * i + 1] / amp;
        uint32_t c = ofc_demodulate16(re, im);
        if (hypot(t[2 * c] - re, t[2 * c + 1] - im) < threshold) {
            re = t[2 * c];
            im = t[2 * c + 1];
        }
        out[2 * i] = amp * re;
        out[2 * i + 1] = amp * im;
    }
}

void ofc_hd_rms(int rows, int cols, const double* a, double* out) {
    /* wdm_scoring.cpp:146-156 ("hd"): hard decision at the RMS amplitude */
    double t[32];
    ofc_gray16(t);
    const size_t n = (size_t)rows * cols;
    const double amp = sqrt(fro2(n, a)) / sqrt((double)n);
    for (size_t i = 0; i < n; ++i) {
        uint32_t c = ofc_demodulate16(a[2 * i] / amp, a[2 * i + 1] / amp);
        out[2 * i] = amp * t[2 * c];
        out[2 * i + 1] = amp * t[2 * c + 1];
    }
}

static int popcount4(uint32_t d) {
    int n = 0;
    while (d) {
        d &= d - 1;
        n++;
    }
    return n;
}

void ofc_error_counts(int modes, int samples, const double* tx, const double* rx,
                      int cut, uint64_t* bit_errors, uint64_t* symbol_errors) {
    double sc = sqrt(modes / ofc_average_power(modes, samples, tx));
    uint64_t be = 0, se = 0;
    for (int m = 0; m < modes; ++m)
        for (int s = cut; s < samples - cut; ++s) {
            size_t i = (size_t)s + (size_t)m * samples;
            uint32_t tc = ofc_demodulate16(sc * tx[2 * i], sc * tx[2 * i + 1]);
            uint32_t rc = ofc_demodulate16(sc * rx[2 * i], sc * rx[2 * i + 1]);
            int d = popcount4(tc ^ rc);
            be += (uint64_t)d;
            se += d > 0;
        }
    *bit_errors = be;
    *symbol_errors = se;
}

double ofc_bit_error_rate(int modes, int samples, const double* tx, const double* rx, int cut) {
    uint64_t be, se;
    ofc_error_counts(modes, samples, tx, rx, cut, &be, &se);
    /* modulation.cpp:200-201: denominator 4*size - 8*cut */
    return (double)be / (double)(4 * modes * samples - 8 * cut);
}

double ofc_symbol_error_rate(int modes, int samples, const double* tx, const double* rx, int cut) {
    uint64_t be, se;
    ofc_error_counts(modes, samples, tx, rx, cut, &be, &se);
    /* modulation.cpp:221-222: denominator size - modes*cut */
    return (double)se / (double)(modes * samples - modes * cut);
}

double ofc_evm2(int modes, int samples, const double* tx, const double* rx, int cut) {
    /* functions.cpp:53-67 (cut = 0 reproduces the uncut overload :40-51) */
    double num = 0, den = 0;
    for (int m = 0; m < modes; ++m)
        for (int s = cut; s < samples - cut; ++s) {
            size_t i = (size_t)s + (size_t)m * samples;
            double dr = tx[2 * i] - rx[2 * i], di = tx[2 * i + 1] - rx[2 * i + 1];
            num += dr * dr + di * di;
            den += tx[2 * i] * tx[2 * i] + tx[2 * i + 1] * tx[2 * i + 1];
        }
    return num / den;
}

double ofc_q2(int modes, int samples, const double* tx, const double* rx, int cut) {
    return -10 * log10(ofc_evm2(modes, samples, tx, rx, cut));
}

void ofc_frequency_shift(int modes, int samples, double dt, double* a, double frequency) {
    /* modulation.cpp:255-264 */
    double wdt = 2 * REF_PI * frequency * dt;
    for (int m = 0; m < modes; ++m)
        for (int s = 0; s < samples; ++s) {
            double ph = wdt * s;
            cmul_inplace(a + 2 * ((size_t)s + (size_t)m * samples), cos(ph), sin(ph));
        }
}

void ofc_bandpass(int modes, int samples, double dt, double* a, double frequency) {
    /* modulation.cpp:266-277 */
    int cut = (int)(frequency * (samples * dt)) + 1;
    ofc_field_fft(modes, samples, a);
    for (int m = 0; m < modes; ++m)
        for (int s = cut; s <= samples - cut; ++s) {
            a[2 * ((size_t)s + (size_t)m * samples)] = 0;
            a[2 * ((size_t)s + (size_t)m * samples) + 1] = 0;
        }
    ofc_field_ifft(modes, samples, a);
}

void ofc_wdm_select(int modes, int samples, double dt, double* a, int channel_index,
                    double channel_bandwidth) {
    /* modulation.cpp:248-253 */
    ofc_frequency_shift(modes, samples, dt, a, -channel_bandwidth * channel_index);
    ofc_bandpass(modes, samples, dt, a, 0.5 * channel_bandwidth);
}

void ofc_wdm_mux(int n_channels, int modes, int samples, double dt, const double* channels,
                 double channel_bandwidth, double* out) {
    /* modulation.cpp:225-235 */
    size_t size = (size_t)modes * samples;
    double* tmp = (double*)malloc(sizeof(double) * 2 * size);
    memset(out, 0, sizeof(double) * 2 * size);
    for (int idx = 0; idx < n_channels; ++idx) {
        double frequency = (idx - n_channels / 2) * channel_bandwidth;
        memcpy(tmp, channels + 2 * size * idx, sizeof(double) * 2 * size);
        ofc_frequency_shift(modes, samples, dt, tmp, frequency);
        for (size_t i = 0; i < 2 * size; ++i) out[i] += tmp[i];
    }
    free(tmp);
}

/* ------------------------------------------------------------------------ */
/* Linear equalizers                                                          */
/* ------------------------------------------------------------------------ */
double ofc_pse_estimate(int modes, int samples, const double* desired,
                        const double* actual, int angle_steps) {
    /* phase_shift_equalizer.cpp:30-46 */
    size_t size = (size_t)modes * samples;
    double* rot = (double*)malloc(sizeof(double) * 2 * size);
    double argmax_angle = 0;
    double max_q2 = ofc_q2(modes, samples, desired, actual, 0);
    for (int i = 0; i < angle_steps; ++i) {
        double angle = 2 * REF_PI * (double)i / angle_steps;
        double c = cos(angle), s = sin(angle);
        for (size_t j = 0; j < size; ++j) {
            rot[2 * j] = actual[2 * j] * c - actual[2 * j + 1] * s;
            rot[2 * j + 1] = actual[2 * j] * s + actual[2 * j + 1] * c;
        }
        double q2 = ofc_q2(modes, samples, desired, rot, 0);
        if (max_q2 < q2) {
            max_q2 = q2;
            argmax_angle = angle;
        }
    }
    free(rot);
    return argmax_angle;
}

void ofc_rotate(int modes, int samples, double* a, double angle) {
    double c = cos(angle), s = sin(angle);
    for (size_t j = 0; j < (size_t)modes * samples; ++j) cmul_inplace(a + 2 * j, c, s);
}

void ofc_scalar_estimate(int modes, int samples, const double* desired,
                         const double* actual, double* scalar) {
    /* scalar_equalizer.cpp:22-33: sum conj(a) d / sum |a|^2 */
    double xx = 0, xyr = 0, xyi = 0;
    size_t size = (size_t)modes * samples;
    for (size_t i = 0; i < size; ++i) xx += actual[2 * i] * actual[2 * i] + actual[2 * i + 1] * actual[2 * i + 1];
    for (size_t i = 0; i < size; ++i) {
        double ar = actual[2 * i], ai = -actual[2 * i + 1];
        xyr += ar * desired[2 * i] - ai * desired[2 * i + 1];
        xyi += ar * desired[2 * i + 1] + ai * desired[2 * i];
    }
    scalar[0] = xyr / xx;
    scalar[1] = xyi / xx;
}

/* ------------------------------------------------------------------------ */
/* Triplet sum (sino.cpp:161-171, 203-220)                                   */
/* ------------------------------------------------------------------------ */
static inline void sino_term(int modes, int samples, const double* a, int mode,
                             int k, int m, int n, double* out) {
    double tr = 0, ti = 0;
    for (int p = 0; p < modes; ++p) {
        const double* x = a + 2 * ((size_t)(k + n) + (size_t)p * samples);
        const double* y = a + 2 * ((size_t)(k + m + n) + (size_t)p * samples);
        /* x * conj(y) */
        tr += x[0] * y[0] + x[1] * y[1];
        ti += x[1] * y[0] - x[0] * y[1];
    }
    const double* z = a + 2 * ((size_t)(k + m) + (size_t)mode * samples);
    out[0] = z[0] * tr - z[1] * ti;
    out[1] = z[0] * ti + z[1] * tr;
}

void ofc_sino_cubic(int modes, int samples, const double* a, int radius,
                    const double* weights, double* out) {
    int w = 2 * radius + 1;
    memset(out, 0, sizeof(double) * 2 * (size_t)modes * samples);
    for (int mode = 0; mode < modes; ++mode)
        for (int k = radius; k < samples - radius; ++k) {
            double sr = 0, si = 0;
            for (int m = -radius; m <= radius; ++m) {
                int borders = radius - abs(m);
                for (int n = -borders; n <= borders; ++n) {
                    double t[2];
                    sino_term(modes, samples, a, mode, k, m, n, t);
                    const double* c = weights + 2 * ((size_t)(m + radius) * w + (n + radius));
                    sr += c[0] * t[0] - c[1] * t[1];
                    si += c[0] * t[1] + c[1] * t[0];
                }
            }
            out[2 * ((size_t)k + (size_t)mode * samples)] = sr;
            out[2 * ((size_t)k + (size_t)mode * samples) + 1] = si;
        }
}

void ofc_triplet_sparse(int modes, int samples, const double* a, int radius,
                        int n_terms, const int32_t* m, const int32_t* n,
                        const double* c, double* out) {
    /* Terms may reach k + m + n outside [0, samples) (|m|,|n| <= R box sets):
     * such samples count as zero.  Diamond sets (|m|+|n| <= R, the
     * reference's SINO::cubic) never leave the range. */
    memset(out, 0, sizeof(double) * 2 * (size_t)modes * samples);
    for (int mode = 0; mode < modes; ++mode)
        for (int k = radius; k < samples - radius; ++k) {
            double sr = 0, si = 0;
            for (int i = 0; i < n_terms; ++i) {
                double t[2];
                int lo = k + (m[i] < 0 ? m[i] : 0) + (n[i] < 0 ? n[i] : 0);
                int hi = k + (m[i] > 0 ? m[i] : 0) + (n[i] > 0 ? n[i] : 0);
                if (lo < 0 || hi >= samples) {
                    /* evaluate with zero padding */
                    int km = k + m[i], kn = k + n[i], kmn = k + m[i] + n[i];
                    if (km < 0 || km >= samples || kn < 0 || kn >= samples || kmn < 0 || kmn >= samples)
                        continue;
                }
                sino_term(modes, samples, a, mode, k, m[i], n[i], t);
                sr += c[2 * i] * t[0] - c[2 * i + 1] * t[1];
                si += c[2 * i] * t[1] + c[2 * i + 1] * t[0];
            }
            out[2 * ((size_t)k + (size_t)mode * samples)] = sr;
            out[2 * ((size_t)k + (size_t)mode * samples) + 1] = si;
        }
}

/* ------------------------------------------------------------------------ */
/* Batched helpers for timing                                                */
/* ------------------------------------------------------------------------ */
int ofc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void ofc_ssfm_batch(int batch, int modes, int samples, double dt, double* a,
                    const ofc_fiber* fiber, int grid, int total_steps,
                    double max_phase_shift, double max_step_size,
                    double direction, int threads, int* steps) {
    for (int l = 0; l < 40; ++l)
        if ((1 << l) == samples) twiddles(l);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : 1)
#endif
    for (int b = 0; b < batch; ++b) {
        int s = ofc_ssfm_run(modes, samples, dt, a + 2 * (size_t)b * modes * samples, fiber,
                             grid, total_steps, max_phase_shift, max_step_size, direction);
        if (steps) steps[b] = s;
    }
    (void)threads;
}

void ofc_uniform_steps_batch(int batch, int modes, int samples, double dt,
                             double* a, const ofc_fiber* fiber, double step,
                             int n_steps, int threads) {
    for (int l = 0; l < 40; ++l)
        if ((1 << l) == samples) twiddles(l);
    double freq_step = 2.0 * REF_PI / (dt * samples);
    double* disp = (double*)malloc(sizeof(double) * (size_t)samples);
    for (int i = 0; i <= samples / 2; ++i) disp[i] = (double)i * freq_step;
    for (int i = samples / 2 + 1; i < samples; ++i) disp[i] = (double)(i - samples) * freq_step;
    for (int i = 0; i < samples; ++i) disp[i] *= disp[i];
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : 1)
#endif
    for (int b = 0; b < batch; ++b) {
        ssfm_ctx c = {modes, samples, fiber, disp, 0, 0};
        double* x = a + 2 * (size_t)b * modes * samples;
        for (int i = 0; i < n_steps; ++i) {
            nonlinear_step(&c, x, step);
            linear_step(&c, x, step);
        }
    }
    free(disp);
    (void)threads;
}
