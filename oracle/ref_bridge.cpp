/*
 * ref_bridge.cpp -- extern "C" entry points over the reference's OWN classes
 * (focss::Field, SSFM, Amplifier, modulation, linear equalizers), compiled
 * from the unmodified reference sources where they lie (oracle/build_ref.py).
 *
 * TEST INFRASTRUCTURE ONLY: used in this container to pin the FP64 oracle
 * restatement (oracle/focss_oracle.c) and to generate the golden vectors
 * committed under tests/golden/.  The product never links it.
 */
#include <cstring>
#include <string>
#include <random>

#include "focss/definitions.h"
#include "focss/equalizer/linear.h"
#include "focss/field.h"
#include "focss/functions.h"
#include "focss/module/amplifier.h"
#include "focss/module/fiber.h"
#include "focss/processing/modulation.h"
#include "focss/solver/ssfm.h"

using namespace focss;

// src/tasks/verification.cpp (compiled alongside)
Field sech_pulse(const int& points, const double& z);
Field dark_pulse(const int& points, const double& z);

namespace {
Field make_field(int modes, int samples, double dt, double f0, const double* data) {
    Domain d{modes, samples, dt, f0};
    Field f(d);
    for (int i = 0; i < f.size(); ++i) f[i] = complex_t(data[2 * i], data[2 * i + 1]);
    return f;
}
void store(const Field& f, double* out) {
    for (int i = 0; i < f.size(); ++i) {
        out[2 * i] = f[i].real();
        out[2 * i + 1] = f[i].imag();
    }
}
Fiber make_fiber(const double* p) { return Fiber{p[0], p[1], p[2], p[3], p[4], p[5]}; }
}  // namespace

extern "C" {

void ref_field_fft(int modes, int samples, double dt, double* data) {
    Field f = make_field(modes, samples, dt, 0, data);
    f.fft_inplace();
    store(f, data);
}

void ref_field_ifft(int modes, int samples, double dt, double* data) {
    Field f = make_field(modes, samples, dt, 0, data);
    f.ifft_inplace();
    store(f, data);
}

void ref_ssfm_run(int modes, int samples, double dt, double* data, const double* fiber6,
                  int grid, int total_steps, double max_phase, double max_step,
                  double direction) {
    Field f = make_field(modes, samples, dt, 0, data);
    SSFM s(make_fiber(fiber6));
    s.set_grid(grid);
    s.set_total_steps(total_steps);
    s.set_maximum_phase_shift(max_phase);
    s.set_maximum_step_size(max_step);
    s.run(f, direction);
    store(f, data);
}

void ref_fiber_scale(const double* fiber6, double factor, double* out6) {
    Fiber g = make_fiber(fiber6) * factor;
    double v[6] = {g.alpha, g.beta2, g.gamma, g.length, g.wavelength, g.kappa};
    std::memcpy(out6, v, sizeof(v));
}

void ref_fiber_dispersive(const double* fiber6, double* out6) {
    Fiber g = make_fiber(fiber6).dispersive();
    double v[6] = {g.alpha, g.beta2, g.gamma, g.length, g.wavelength, g.kappa};
    std::memcpy(out6, v, sizeof(v));
}

void ref_amplify(int modes, int samples, double dt, double f0, double* data, double gain,
                 double noise_factor, unsigned seed) {
    Field f = make_field(modes, samples, dt, f0, data);
    global_urng().seed(seed);
    Amplifier(gain, noise_factor).amplify(f);
    store(f, data);
}

/* Field::average_power / peak_power (field.cpp:164-187). */
void ref_field_power(int modes, int samples, const double* data, double* average, double* peak) {
    Field f = make_field(modes, samples, 1.0, 0, data);
    *average = f.average_power();
    *peak = f.peak_power();
}

void ref_drop_power(int modes, int samples, double* data, double gain) {
    Field f = make_field(modes, samples, 1.0, 0, data);
    Amplifier(gain).drop_power(f);
    store(f, data);
}

void ref_give_power(int modes, int samples, double* data, double gain) {
    Field f = make_field(modes, samples, 1.0, 0, data);
    Amplifier(gain).give_power(f);
    store(f, data);
}

double ref_db_to_linear(double x) { return db_to_linear(x); }
double ref_dbm_to_watts(double x) { return dbm_to_watts(x); }
double ref_db_to_natural(double x) { return db_to_natural(x); }
double ref_disp_to_beta2(double d, double wl) { return disp_to_beta2(d, wl); }

void ref_rrc_pulse(int n_symbols, int osf, double roll_off, double* out) {
    ComplexVector h = pulse::rrc(n_symbols, osf, roll_off);
    for (int i = 0; i < h.size(); ++i) {
        out[2 * i] = h[i].real();
        out[2 * i + 1] = h[i].imag();
    }
}

void ref_filter(int modes, int samples, double dt, double* data, int h_len, const double* h) {
    Field f = make_field(modes, samples, dt, 0, data);
    ComplexVector hv(h_len);
    for (int i = 0; i < h_len; ++i) hv[i] = complex_t(h[2 * i], h[2 * i + 1]);
    f.filter_inplace(hv);
    store(f, data);
}

void ref_upsample(int modes, int samples, double dt, const double* data, int factor, double* out) {
    store(make_field(modes, samples, dt, 0, data).upsample(factor), out);
}

void ref_downsample(int modes, int samples, double dt, const double* data, int factor, double* out) {
    store(make_field(modes, samples, dt, 0, data).downsample(factor), out);
}

void ref_decimate(int modes, int samples, double dt, const double* data, int factor, double* out) {
    store(make_field(modes, samples, dt, 0, data).decimate(factor), out);
}

/* The reference's own shaping/sampling (roll-off fixed at 0.01, modulation.cpp:85). */
void ref_rrc_shaping(int modes, int n_symbols, double dt, const double* symbols, int osf,
                     double gain, double* out) {
    store(rrc_shaping(make_field(modes, n_symbols, dt, 0, symbols), osf, gain), out);
}

void ref_rrc_sampling(int modes, int samples, double dt, const double* signal, int osf,
                      double gain, double* out) {
    store(rrc_sampling(make_field(modes, samples, dt, 0, signal), osf, gain), out);
}

/* The same three-line wrappers (modulation.cpp:86-96) with the roll-off the
 * benchmark configurations ask for, built from the reference's primitives. */
void ref_rrc_shaping_rolloff(int modes, int n_symbols, double dt, const double* symbols,
                             int osf, double roll_off, double gain, double* out) {
    Field sy = make_field(modes, n_symbols, dt, 0, symbols);
    auto rrc = pulse::rrc(sy.samples(), osf, roll_off);
    auto signal = sy.upsample(osf).filter_inplace(rrc);
    store((std::sqrt(gain) * osf) * signal, out);
}

void ref_rrc_sampling_rolloff(int modes, int samples, double dt, const double* signal, int osf,
                              double roll_off, double gain, double* out) {
    Field sg = make_field(modes, samples, dt, 0, signal);
    auto rrc = pulse::rrc(sg.samples() / osf, osf, roll_off);
    auto symbols = sg.filter(rrc).downsample(osf);
    store(std::sqrt(gain) * symbols, out);
}

unsigned ref_demodulate16(double re, double im) { return demodulate_16qam(complex_t(re, im)); }

void ref_hard_decision(int modes, int samples, const double* data, double* out) {
    store(hard_decision_16qam(make_field(modes, samples, 1.0, 0, data)), out);
}
void ref_save_transmission(int modes, int samples, const double* tx, const double* rx, const char* path) {
    save_transmission(std::string(path), make_field(modes, samples, 1.0, 0, tx), make_field(modes, samples, 1.0, 0, rx));
}

void ref_load_transmission(int modes, int samples, const char* path, double* tx, double* rx) {
    Field t(Domain{modes, samples, 1.0, 0}), r(Domain{modes, samples, 1.0, 0});
    load_transmission(std::string(path), &t, &r);
    store(t, tx);
    store(r, rx);
}

void ref_soft_decision(int modes, int samples, const double* data, double uncertainty, double* out) {
    store(soft_decision_16qam(make_field(modes, samples, 1.0, 0, data), uncertainty), out);
}

double ref_ber(int modes, int samples, const double* tx, const double* rx, int cut) {
    Field t = make_field(modes, samples, 1.0, 0, tx);
    Field r = make_field(modes, samples, 1.0, 0, rx);
    return cut < 0 ? bit_error_rate_16qam(t, r) : bit_error_rate_16qam(t, r, cut);
}

double ref_ser(int modes, int samples, const double* tx, const double* rx, int cut) {
    return symbol_error_rate_16qam(make_field(modes, samples, 1.0, 0, tx),
                                   make_field(modes, samples, 1.0, 0, rx), cut);
}

double ref_q2(int modes, int samples, const double* tx, const double* rx, int cut) {
    Field t = make_field(modes, samples, 1.0, 0, tx);
    Field r = make_field(modes, samples, 1.0, 0, rx);
    return cut < 0 ? q2_factor(t, r) : q2_factor(t, r, cut);
}

double ref_pse_angle(int modes, int samples, const double* desired, const double* actual,
                     int angle_steps) {
    PhaseShiftEqualizer pse(angle_steps);
    pse.train(make_field(modes, samples, 1.0, 0, desired),
              make_field(modes, samples, 1.0, 0, actual));
    return pse.get_angle();
}

void ref_scalar_estimate(int modes, int samples, const double* desired, const double* actual,
                         double* out2) {
    ScalarEqualizer se;
    se.train(make_field(modes, samples, 1.0, 0, desired),
             make_field(modes, samples, 1.0, 0, actual));
    out2[0] = se.get_scalar().real();
    out2[1] = se.get_scalar().imag();
}

void ref_frequency_shift(int modes, int samples, double dt, double* data, double frequency) {
    Field f = make_field(modes, samples, dt, 0, data);
    store(frequency_shift(f, frequency), data);
}

void ref_bandpass(int modes, int samples, double dt, double* data, double frequency) {
    Field f = make_field(modes, samples, dt, 0, data);
    store(bandpass_filter(f, frequency), data);
}

void ref_wdm_select(int modes, int samples, double dt, double* data, int channel_index,
                    double channel_bandwidth) {
    Field f = make_field(modes, samples, dt, 0, data);
    store(wdm_select(f, channel_index, channel_bandwidth), data);
}

void ref_wdm_mux(int n_channels, int modes, int samples, double dt, const double* channels,
                 double channel_bandwidth, double* out) {
    Vector<Field> ch(n_channels);
    for (int c = 0; c < n_channels; ++c)
        ch[c] = make_field(modes, samples, dt, 0, channels + 2 * (size_t)c * modes * samples);
    store(wdm_mux(ch, channel_bandwidth), out);
}

void ref_soliton(int dark, int points, double z, double* out) {
    store(dark ? dark_pulse(points, z) : sech_pulse(points, z), out);
}

}  // extern "C"
