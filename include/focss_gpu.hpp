/* focss_gpu.hpp -- C++ facade over the C ABI in focss_gpu.h.
 *
 * Mirrors the reference's C++ API for the split-step path with the same class
 * and function names in namespace focss:
 *   Domain, Field                    src/focss/field.h:20-162
 *   Fiber                            src/focss/module/fiber.h:5-21
 *   SSFM                             src/focss/solver/ssfm.h:8-54
 *   Amplifier                        src/focss/module/amplifier.h:7-22
 *   q2/evm2, dB helpers              src/focss/functions.h
 *   pulse::rrc, rrc_shaping/sampling, decisions, BER/SER, WDM helpers
 *                                    src/focss/processing/modulation.h:8-45
 *   PhaseShiftEqualizer, ScalarEqualizer
 *                                    src/focss/equalizer/linear.h
 *   save/load_transmission           src/focss/functions.cpp:174-221
 *   save_field / load_field          src/tasks/wdm_run.cpp:55-77, wdm_scoring.cpp:79-103
 *   find_certainty, sd, hd           src/tasks/wdm_scoring.cpp:105-156
 *   SINO                             src/focss/equalizer/sino.h:8-50
 *   WdmPPE                           src/focss/equalizer/wdm_sino.h:8-71
 * so that callers such as src/tasks/systems.cpp compile against it unchanged
 * (include/focss_compat/ maps the reference's header names onto this file).
 *
 * Differences from the reference, all forced by device residency:
 *  - A Field lives in GPU memory (complex64).  Element access (operator[],
 *    operator()) goes through a host mirror that is filled on demand and
 *    written back before the next device operation; a reference returned by
 *    the non-const accessors is valid until that operation.
 *  - A Field may hold a batch of independent realizations (extra `batch`
 *    argument, default 1); every operation applies to all of them.  Scalar
 *    results (powers, Q, BER, angles) refer to realization 0; the *_each
 *    variants return one value per realization.
 *  - Errors throw focss::gpu_error (the reference only asserts).
 *  - ASE noise comes from a counter-based generator: the process-wide seed
 *    (reseed_global_urng / set_global_seed) plus a call counter, so every
 *    add_noise call draws fresh noise as the reference's global engine does.
 *  - rrc_shaping / rrc_sampling keep the reference's fixed roll-off 0.01
 *    (modulation.cpp:85); overloads take the roll-off explicitly.
 * Header only; link with libfocss_gpu.so.
 */
#ifndef FOCSS_GPU_HPP_
#define FOCSS_GPU_HPP_

#include <atomic>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <istream>
#include <ostream>
#include <random>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "focss_gpu.h"

namespace focss {

typedef double real_t;
typedef std::complex<real_t> complex_t;
template <typename T>
using Vector = std::vector<T>;
typedef Vector<real_t> RealVector;
typedef Vector<complex_t> ComplexVector;

const real_t math_pi = 3.14159265358979323846264338;
const real_t planck = 6.62607004081818181818181e-34;  // [m^2 kg / s]
const real_t light_speed = 299792458;                 // [m / s]
const complex_t i_unit = complex_t(0, 1);

/* Error raised for any non-OK status of the C ABI. */
class gpu_error : public std::runtime_error {
  public:
    gpu_error(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
    int status() const { return status_; }

  private:
    int status_;
};

namespace detail {
inline void check(focss_status s, const focss_ctx* ctx = nullptr) {
    if (s == FOCSS_OK) return;
    std::string msg = std::string("focss: ") + focss_status_string(s);
    if (ctx) {
        const char* e = focss_ctx_last_error(ctx);
        if (e && *e) msg += std::string(": ") + e;
    }
    throw gpu_error(s, msg);
}
struct ContextHolder {
    focss_ctx* ctx = nullptr;
    ~ContextHolder() {
        if (ctx) focss_ctx_destroy(ctx);
    }
};
inline std::atomic<std::uint64_t>& urng_seed() {
    static std::atomic<std::uint64_t> s{0x5eed0f0c55ull};
    return s;
}
inline std::atomic<std::uint64_t>& urng_counter() {
    static std::atomic<std::uint64_t> c{0};
    return c;
}
}  // namespace detail

/* The calling thread's device context (one stream per host thread).  The
 * device is FOCSS_DEVICE from the environment, else 0. */
inline focss_ctx* gpu_context() {
    static thread_local detail::ContextHolder h;
    if (!h.ctx) {
        int dev = 0;
        if (const char* e = std::getenv("FOCSS_DEVICE")) dev = std::atoi(e);
        detail::check(focss_ctx_create(dev, &h.ctx));
    }
    return h.ctx;
}
inline void gpu_sync() { detail::check(focss_ctx_sync(gpu_context()), gpu_context()); }

/* ------------------------------------------------------------- functions */
/* src/focss/functions.cpp:11-25: the ASE generator's seed. */
inline void set_global_seed(std::uint64_t seed) {
    detail::urng_seed() = seed;
    detail::urng_counter() = 0;
}
inline void reseed_global_urng() {
    std::random_device rd;
    set_global_seed(((std::uint64_t)rd() << 32) ^ (std::uint64_t)rd());
}
inline void setup() { reseed_global_urng(); }

/* src/focss/functions.cpp:82-105 */
inline double db_to_linear(const double& db_value) { return std::pow(10, db_value / 10); }
inline double dbm_to_watts(const double& dbm_power) { return 1e-3 * std::pow(10, dbm_power / 10); }
inline double db_to_natural(const double& db_value) { return db_value * std::log(10) / 10; }
inline double disp_to_beta2(const double& dispersion, const double& wavelength) {
    return -wavelength * wavelength * dispersion / (2 * math_pi * light_speed);
}
inline double sinc(const double& x) { return x == 0 ? 1 : std::sin(math_pi * x) / math_pi / x; }
inline complex_t i_exp(const double& x) { return complex_t(std::cos(x), std::sin(x)); }

/* ---------------------------------------------------------------- Domain */
struct Domain {
    int modes;
    int samples;
    real_t time_step;
    real_t center_frequency;
    inline int size() const { return modes * samples; }
    inline bool operator==(const Domain& o) const {
        return modes == o.modes && samples == o.samples && time_step == o.time_step &&
               center_frequency == o.center_frequency;
    }
};

/* ----------------------------------------------------------------- Field */
class Field {
  public:
    Field() : h_(nullptr), dom_{0, 0, 0, 0}, batch_(0), where_(DEVICE) {}
    explicit Field(const Domain& domain, int batch = 1) : dom_(domain), batch_(batch), where_(DEVICE) {
        create();
    }
    /* data: batch * modes * samples values, realization-major then mode-major. */
    Field(const Domain& domain, const ComplexVector& data) : dom_(domain), where_(DEVICE) {
        const size_t n = (size_t)domain.size();
        if (n == 0 || data.size() % n) throw gpu_error(FOCSS_ERR_INVALID_ARG, "focss: data size is not a multiple of the domain size");
        batch_ = (int)(data.size() / n);
        create();
        host_ = data;
        where_ = HOST;
    }
    Field(const Field& o) : dom_(o.dom_), batch_(o.batch_), where_(DEVICE) {
        h_ = nullptr;
        if (!o.h_) return;
        create();
        o.push();
        detail::check(focss_field_copy(h_, o.h_), gpu_context());
    }
    Field(Field&& o) noexcept : h_(o.h_), dom_(o.dom_), batch_(o.batch_), host_(std::move(o.host_)), where_(o.where_) {
        o.h_ = nullptr;
        o.batch_ = 0;
    }
    Field& operator=(const Field& o) {
        if (this == &o) return *this;
        Field t(o);
        swap(t);
        return *this;
    }
    Field& operator=(Field&& o) noexcept {
        swap(o);
        return *this;
    }
    ~Field() {
        if (h_) focss_field_destroy(h_);
    }
    void swap(Field& o) noexcept {
        std::swap(h_, o.h_);
        std::swap(dom_, o.dom_);
        std::swap(batch_, o.batch_);
        host_.swap(o.host_);
        std::swap(where_, o.where_);
    }

    /* ---- element access through the host mirror (field.cpp:135-159) */
    complex_t operator[](const int& index) const { return pull()[(size_t)index]; }
    complex_t& operator[](const int& index) { return pull_mut()[(size_t)index]; }
    complex_t operator()(const int& mode, const int& sample) const {
        return pull()[(size_t)mode * dom_.samples + sample];
    }
    complex_t& operator()(const int& mode, const int& sample) {
        return pull_mut()[(size_t)mode * dom_.samples + sample];
    }
    ComplexVector operator()(const int& mode) const {
        const ComplexVector& h = pull();
        return ComplexVector(h.begin() + (size_t)mode * dom_.samples, h.begin() + (size_t)(mode + 1) * dom_.samples);
    }
    /* All realizations, realization-major. */
    const ComplexVector& data() const { return pull(); }

    /* ---- powers (field.cpp:164-195); realization 0, *_each per realization */
    real_t power(const int& sample) const {
        const ComplexVector& h = pull();
        real_t p = 0;
        for (int m = 0; m < dom_.modes; ++m) p += std::norm(h[(size_t)m * dom_.samples + sample]);
        return p;
    }
    RealVector peak_power_each() const {
        RealVector pk((size_t)batch_);
        detail::check(focss_field_power(handle(), nullptr, pk.data()), gpu_context());
        return pk;
    }
    RealVector average_power_each() const {
        RealVector av((size_t)batch_);
        detail::check(focss_field_power(handle(), av.data(), nullptr), gpu_context());
        return av;
    }
    real_t peak_power() const { return peak_power_each()[0]; }
    real_t average_power() const { return average_power_each()[0]; }
    Field& peak_normalize(const real_t& p = 1) { return (*this) *= std::sqrt(p / peak_power()); }
    Field& average_normalize(const real_t& p = 1) { return (*this) *= std::sqrt(p / average_power()); }

    /* ---- shape and grids (field.cpp:199-266) */
    int size() const { return dom_.size(); }
    int modes() const { return dom_.modes; }
    int samples() const { return dom_.samples; }
    int batch() const { return batch_; }
    real_t duration() const { return dom_.samples * dom_.time_step; }
    real_t bandwidth() const { return 1.0 / dom_.time_step; }
    real_t time_step() const { return dom_.time_step; }
    real_t sampling_rate() const { return 1.0 / dom_.time_step; }
    real_t center_frequency() const { return dom_.center_frequency; }
    real_t dt() const { return dom_.time_step; }
    real_t df() const { return 1.0 / (dom_.time_step * dom_.samples); }
    real_t dw() const { return 2.0 * math_pi / (dom_.time_step * dom_.samples); }
    real_t t(const int& sample) const { return static_cast<real_t>(sample) * dt(); }
    real_t f(const int& sample) const { return dom_.center_frequency + (sample - dom_.samples / 2) * df(); }
    real_t w(const int& sample) const { return 2 * math_pi * f(sample); }
    Domain domain() const { return dom_; }
    RealVector time_grid() const {
        RealVector g((size_t)dom_.samples);
        for (int s = 0; s < dom_.samples; ++s) g[(size_t)s] = t(s);
        return g;
    }
    RealVector frequency_grid() const {
        RealVector g((size_t)dom_.samples);
        for (int s = 0; s < dom_.samples; ++s) g[(size_t)s] = f(s);
        return g;
    }
    RealVector temporal_power() const {
        RealVector p((size_t)dom_.samples);
        for (int s = 0; s < dom_.samples; ++s) p[(size_t)s] = power(s);
        return p;
    }

    /* ---- resampling (field.cpp:272-320) */
    Field upsample(const int& factor) const {
        Field out(Domain{dom_.modes, dom_.samples * factor, dom_.time_step / factor, dom_.center_frequency}, batch_);
        detail::check(focss_upsample(gpu_context(), handle(), factor, out.h_), gpu_context());
        return out;
    }
    Field downsample(const int& factor) const {
        Field out(Domain{dom_.modes, dom_.samples / factor, dom_.time_step * factor, dom_.center_frequency}, batch_);
        detail::check(focss_downsample(gpu_context(), handle(), factor, out.h_), gpu_context());
        return out;
    }
    Field decimate(const int& factor) const {
        Field out(Domain{dom_.modes, dom_.samples / factor, dom_.time_step * factor, dom_.center_frequency}, batch_);
        detail::check(focss_decimate(gpu_context(), handle(), factor, out.h_), gpu_context());
        return out;
    }

    /* ---- Fourier methods (field.cpp:343-372) */
    Field& fft_inplace() {
        detail::check(focss_field_fft(mut()), gpu_context());
        return *this;
    }
    Field& ifft_inplace() {
        detail::check(focss_field_ifft(mut()), gpu_context());
        return *this;
    }
    Field fft() const { return Field(*this).fft_inplace(); }
    Field ifft() const { return Field(*this).ifft_inplace(); }
    Field& filter_inplace(const ComplexVector& impulse_response) {
        detail::check(focss_filter(gpu_context(), mut(), reinterpret_cast<const double*>(impulse_response.data()),
                                   (int)impulse_response.size()),
                      gpu_context());
        return *this;
    }
    Field filter(const ComplexVector& impulse_response) const { return Field(*this).filter_inplace(impulse_response); }

    /* ---- scalar arithmetic (field.cpp:376-400) */
    Field& operator*=(const real_t& a) { return (*this) *= complex_t(a, 0); }
    Field& operator*=(const complex_t& a) {
        detail::check(focss_field_scale(mut(), a.real(), a.imag()), gpu_context());
        return *this;
    }
    Field& operator/=(const real_t& a) { return (*this) *= complex_t(1.0 / a, 0); }
    Field& operator/=(const complex_t& a) { return (*this) *= (complex_t(1, 0) / a); }
    friend Field operator*(const Field& f, const real_t& a) { return Field(f) *= a; }
    friend Field operator*(const Field& f, const complex_t& a) { return Field(f) *= a; }
    friend Field operator*(const real_t& a, const Field& f) { return Field(f) *= a; }
    friend Field operator*(const complex_t& a, const Field& f) { return Field(f) *= a; }
    friend Field operator/(const Field& f, const real_t& a) { return Field(f) /= a; }
    friend Field operator/(const Field& f, const complex_t& a) { return Field(f) /= a; }

    /* ---- batch helpers */
    /* `count` realizations of `src` from src_first into this field from dst_first. */
    void copy_realizations(int dst_first, const Field& src, int src_first, int count) {
        detail::check(focss_field_copy_realizations(mut(), dst_first, src.handle(), src_first, count), gpu_context());
    }

    /* Device handle with host edits written back (read access). */
    focss_field* handle() const {
        push();
        return h_;
    }
    /* Device handle for an operation that modifies the field. */
    focss_field* mut() {
        push();
        where_ = DEVICE;
        return h_;
    }

  private:
    enum Where { DEVICE, HOST, BOTH };
    void create() {
        focss_domain d{dom_.modes, dom_.samples, dom_.time_step, dom_.center_frequency};
        detail::check(focss_field_create(gpu_context(), &d, batch_, &h_), gpu_context());
    }
    size_t count() const { return (size_t)batch_ * (size_t)dom_.size(); }
    void push() const {
        if (where_ != HOST) return;
        detail::check(focss_field_upload(h_, reinterpret_cast<const double*>(host_.data()), count()), gpu_context());
        where_ = BOTH;
    }
    const ComplexVector& pull() const {
        if (where_ == DEVICE) {
            host_.resize(count());
            detail::check(focss_field_download(h_, reinterpret_cast<double*>(host_.data()), count()), gpu_context());
            where_ = BOTH;
        }
        return host_;
    }
    ComplexVector& pull_mut() {
        pull();
        where_ = HOST;
        return host_;
    }

    focss_field* h_;
    Domain dom_;
    int batch_;
    mutable ComplexVector host_;
    mutable Where where_;
};

/* ----------------------------------------------------------------- Fiber */
/* src/focss/module/fiber.cpp:4-45 */
struct Fiber {
    double alpha;
    double beta2;
    double gamma;
    double length;
    double wavelength;
    double kappa;

    Fiber linear() const {
        Fiber f = *this;
        f.gamma = 0;
        return f;
    }
    Fiber nonlinear() const {
        Fiber f = *this;
        f.alpha = 0;
        f.beta2 = 0;
        return f;
    }
    Fiber dispersive() const {
        Fiber f = *this;
        f.alpha = 0;
        f.gamma = 0;
        return f;
    }
    Fiber operator-() const {
        Fiber f = *this;
        f.alpha = -alpha;
        f.beta2 = -beta2;
        f.gamma = -gamma;
        return f;
    }
    Fiber operator*(const double& length_factor) const {
        Fiber f = *this;
        if (length_factor >= 0) {
            f.length *= length_factor;
        } else {
            f.alpha = -alpha;
            f.beta2 = -beta2;
            f.gamma = -gamma;
            f.length *= -length_factor;
        }
        return f;
    }
    focss_fiber c() const { return focss_fiber{alpha, beta2, gamma, length, wavelength, kappa}; }
};

/* ------------------------------------------------------------------ SSFM */
/* src/focss/solver/ssfm.h:8-54.  The reference leaves the grid and limits
 * uninitialised unless set (ssfm.cpp:17-22); here they default to UNIFORM,
 * one step, 1e-3 rad and 1 km. */
class SSFM {
  public:
    typedef const int Grid;
    static constexpr int UNIFORM = FOCSS_UNIFORM;
    static constexpr int LOGARITHMIC = FOCSS_LOGARITHMIC;
    static constexpr int ADAPTIVE = FOCSS_ADAPTIVE;
    typedef const double Direction;
    static constexpr double FORWARD = FOCSS_FORWARD;
    static constexpr double BACKWARD = FOCSS_BACKWARD;

    SSFM() : fiber_{0, 0, 0, 0, 1.55e-6, 1}, opts_{FOCSS_UNIFORM, 1, 1e-3, 1e3} {}
    SSFM(const Fiber& fiber) : fiber_(fiber), opts_{FOCSS_UNIFORM, 1, 1e-3, 1e3} {}
    SSFM(const Fiber& fiber, const int& total_steps) : fiber_(fiber), opts_{FOCSS_UNIFORM, total_steps, 1e-3, 1e3} {}

    void set_fiber(const Fiber& fiber) { fiber_ = fiber; }
    void set_grid(const int& grid) { opts_.grid = grid; }
    void set_total_steps(const int& total_steps) { opts_.total_steps = total_steps; }
    void set_maximum_phase_shift(const double& v) { opts_.maximum_phase_shift = v; }
    void set_maximum_step_size(const double& v) { opts_.maximum_step_size = v; }

    /* Runs every realization of `field`; last_steps() gives the step counts. */
    void run(Field& field, const double& direction = FORWARD) {
        steps_.assign((size_t)field.batch(), 0);
        focss_fiber f = fiber_.c();
        detail::check(focss_ssfm_run(gpu_context(), field.mut(), &f, &opts_, direction, steps_.data()), gpu_context());
    }
    const Vector<int>& last_steps() const { return steps_; }

  private:
    Fiber fiber_;
    focss_ssfm_opts opts_;
    Vector<int> steps_;
};

/* ------------------------------------------------------------- Amplifier */
/* src/focss/module/amplifier.cpp:8-47 */
class Amplifier {
  public:
    Amplifier() : gain_(1), noise_factor_(0) {}
    Amplifier(const double& gain) : gain_(gain), noise_factor_(0) {}
    Amplifier(const double& gain, const double& noise_factor) : gain_(gain), noise_factor_(noise_factor) {}

    void amplify(Field& field) const { apply(field, FOCSS_AMP_AMPLIFY); }
    void add_noise(Field& field) const { apply(field, FOCSS_AMP_ADD_NOISE); }
    void give_power(Field& field) const { apply(field, FOCSS_AMP_GIVE_POWER); }
    void drop_power(Field& field) const { apply(field, FOCSS_AMP_DROP_POWER); }

  private:
    void apply(Field& field, int op) const {
        const std::uint64_t counter = detail::urng_counter().fetch_add(1);
        detail::check(focss_amplifier_apply(gpu_context(), field.mut(), gain_, noise_factor_, detail::urng_seed().load(),
                                            counter, op),
                      gpu_context());
    }
    double gain_;
    double noise_factor_;
};

/* -------------------------------------------------------------- metrics */
/* src/focss/functions.cpp:27-80 (FP64 sums on the device). */
inline double q2_factor(const Field& tx, const Field& rx, const int& cut) {
    Vector<double> q((size_t)tx.batch());
    detail::check(focss_q2_factor(gpu_context(), tx.handle(), rx.handle(), cut, q.data()), gpu_context());
    return q[0];
}
inline double q2_factor(const Field& tx, const Field& rx) { return q2_factor(tx, rx, -1); }
inline double evm2_factor(const Field& tx, const Field& rx, const int& cut) {
    return std::pow(10.0, -q2_factor(tx, rx, cut) / 10.0);
}
inline double evm2_factor(const Field& tx, const Field& rx) { return evm2_factor(tx, rx, -1); }
inline Vector<double> q2_factor_each(const Field& tx, const Field& rx, int cut = -1) {
    Vector<double> q((size_t)tx.batch());
    detail::check(focss_q2_factor(gpu_context(), tx.handle(), rx.handle(), cut, q.data()), gpu_context());
    return q;
}

/* ------------------------------------------------------------ modulation */
namespace pulse {
/* src/focss/processing/modulation.cpp:47-74, computed on the device in FP64. */
inline ComplexVector rrc(const int& n_symbols, const int& oversampling, const double& roll_off) {
    ComplexVector taps((size_t)n_symbols * oversampling);
    detail::check(focss_rrc_pulse(gpu_context(), n_symbols, oversampling, roll_off, reinterpret_cast<double*>(taps.data())),
                  gpu_context());
    return taps;
}
}  // namespace pulse

const double rrc_roll_off = 0.01;  // modulation.cpp:85

/* Gray 16QAM points of codes (modulation.cpp:9-17); codes in field order. */
inline Field qam16_symbols(const Vector<int>& codes, const Domain& domain) {
    const int batch = domain.size() ? (int)(codes.size() / (size_t)domain.size()) : 0;
    Field out(domain, batch);
    Vector<std::int32_t> c(codes.begin(), codes.end());
    detail::check(focss_qam16_map(gpu_context(), c.data(), c.size(), out.mut()), gpu_context());
    return out;
}

/* modulation.cpp:86-90 / :92-96 */
inline Field rrc_shaping(const Field& symbols, const int& osf, const double& gain, const double& roll_off) {
    const Domain d = symbols.domain();
    Field out(Domain{d.modes, d.samples * osf, d.time_step / osf, d.center_frequency}, symbols.batch());
    detail::check(focss_rrc_shaping(gpu_context(), symbols.handle(), osf, roll_off, gain, out.mut()), gpu_context());
    return out;
}
inline Field rrc_shaping(const Field& symbols, const int& osf, const double& gain = 1) {
    return rrc_shaping(symbols, osf, gain, rrc_roll_off);
}
inline Field rrc_sampling(const Field& signal, const int& osf, const double& gain, const double& roll_off) {
    const Domain d = signal.domain();
    Field out(Domain{d.modes, d.samples / osf, d.time_step * osf, d.center_frequency}, signal.batch());
    detail::check(focss_rrc_sampling(gpu_context(), signal.handle(), osf, roll_off, gain, out.mut()), gpu_context());
    return out;
}
inline Field rrc_sampling(const Field& signal, const int& osf, const double& gain = 1) {
    return rrc_sampling(signal, osf, gain, rrc_roll_off);
}

/* modulation.cpp:112-120, :148-156 */
inline Field hard_decision_16qam(const Field& signal) {
    Field out(signal.domain(), signal.batch());
    detail::check(focss_hard_decision(gpu_context(), signal.handle(), out.mut()), gpu_context());
    return out;
}
inline Field soft_decision_16qam(const Field& signal, const double& uncertainty) {
    Field out(signal.domain(), signal.batch());
    detail::check(focss_soft_decision(gpu_context(), signal.handle(), uncertainty, out.mut()), gpu_context());
    return out;
}
/* src/tasks/wdm_scoring.cpp:105-156 (file-local helpers of the WDM scoring
 * task): one matrix per realization, rows = modes (channel * modes + mode for
 * a loaded dataset field). */
inline double find_certainty(const Field& tx, const Field& rx) {
    Vector<double> v((size_t)tx.batch());
    detail::check(focss_find_certainty(gpu_context(), tx.handle(), rx.handle(), v.data()), gpu_context());
    return v[0];
}
inline Field sd(const Field& field, const double& certainty) {
    Field out(field.domain(), field.batch());
    detail::check(focss_certainty_decision(gpu_context(), field.handle(), certainty, out.mut()), gpu_context());
    return out;
}
inline Field hd(const Field& field) { return hard_decision_16qam(field); }
inline Vector<int> hd_sequence_16qam(const Field& signal) {
    Vector<std::int32_t> c((size_t)signal.batch() * signal.size());
    detail::check(focss_hd_codes(gpu_context(), signal.handle(), c.data()), gpu_context());
    return Vector<int>(c.begin(), c.end());
}

/* modulation.cpp:158-223 */
inline double bit_error_rate_16qam(const Field& tx, const Field& rx, const int& cut) {
    Vector<double> v((size_t)tx.batch());
    detail::check(focss_bit_error_rate(gpu_context(), tx.handle(), rx.handle(), cut, v.data()), gpu_context());
    return v[0];
}
inline double bit_error_rate_16qam(const Field& tx, const Field& rx) { return bit_error_rate_16qam(tx, rx, -1); }
inline double symbol_error_rate_16qam(const Field& tx, const Field& rx, const int& cut) {
    Vector<double> v((size_t)tx.batch());
    detail::check(focss_symbol_error_rate(gpu_context(), tx.handle(), rx.handle(), cut, v.data()), gpu_context());
    return v[0];
}

/* modulation.cpp:225-277 */
inline Field frequency_shift(const Field& field, const double& frequency) {
    Field out(field);
    detail::check(focss_frequency_shift(gpu_context(), out.mut(), frequency), gpu_context());
    return out;
}
inline Field bandpass_filter(const Field& field, const double& frequency) {
    Field out(field);
    detail::check(focss_bandpass(gpu_context(), out.mut(), frequency), gpu_context());
    return out;
}
inline Field wdm_select(const Field& field, const int& channel_index, const double& channel_bandwidth) {
    Field out(field.domain(), field.batch());
    detail::check(focss_wdm_select(gpu_context(), field.handle(), channel_index, channel_bandwidth, out.mut()),
                  gpu_context());
    return out;
}
inline Field wdm_mux(const Vector<Field>& channels, const double& channel_bandwidth) {
    if (channels.empty()) throw gpu_error(FOCSS_ERR_INVALID_ARG, "focss: wdm_mux of no channels");
    const Domain d = channels[0].domain();
    Field stacked(d, (int)channels.size());
    for (size_t c = 0; c < channels.size(); ++c) stacked.copy_realizations((int)c, channels[c], 0, 1);
    Field out(d, 1);
    detail::check(focss_wdm_mux(gpu_context(), stacked.handle(), channel_bandwidth, out.mut()), gpu_context());
    return out;
}
inline Vector<Field> wdm_demux(const Field& field, const int& n_channels, const double& channel_bandwidth) {
    Vector<Field> out;
    for (int ch = 0; ch < n_channels; ++ch) out.push_back(wdm_select(field, ch - n_channels / 2, channel_bandwidth));
    return out;
}

/* ------------------------------------------------------------- dataset I/O */
/* Transmission CSV of src/focss/functions.cpp:174-221: per sample the tx
 * modes then the rx modes as re,im pairs (realization 0 of each field). */
inline void save_transmission(std::ostream& output, const Field& tx, const Field& rx) {
    if (tx.modes() != rx.modes() || tx.samples() != rx.samples())
        throw gpu_error(FOCSS_ERR_INVALID_ARG, "focss: save_transmission of fields of different shapes");
    const int M = tx.modes();
    for (int i = 0; i < tx.samples(); ++i) {
        for (int m = 0; m < M; ++m) output << tx(m, i).real() << ',' << tx(m, i).imag() << ',';
        for (int m = 0; m < M; ++m) {
            output << rx(m, i).real() << ',' << rx(m, i).imag();
            output << (m + 1 < M ? ',' : '\n');
        }
    }
}
inline void load_transmission(std::istream& input, Field* tx, Field* rx) {
    if (tx->modes() != rx->modes() || tx->samples() != rx->samples())
        throw gpu_error(FOCSS_ERR_INVALID_ARG, "focss: load_transmission into fields of different shapes");
    double re, im;
    char delimiter = ',';
    for (int i = 0; i < tx->samples(); ++i) {
        for (int m = 0; m < tx->modes(); ++m) {
            if (m) input >> delimiter;
            input >> re >> delimiter >> im;
            (*tx)(m, i) = complex_t(re, im);
        }
        for (int m = 0; m < rx->modes(); ++m) {
            input >> delimiter >> re >> delimiter >> im;
            (*rx)(m, i) = complex_t(re, im);
        }
    }
}
inline void save_transmission(const std::string& filename, const Field& tx, const Field& rx) {
    std::ofstream file(filename);
    file.precision(15);
    save_transmission(file, tx, rx);
}
inline void load_transmission(const std::string& filename, Field* tx, Field* rx) {
    std::ifstream file(filename);
    load_transmission(file, tx, rx);
}

/* Field binary of src/tasks/wdm_run.cpp:55-77 (written) and
 * src/tasks/wdm_scoring.cpp:79-103 (read): ints n_ch, n_samples, n_modes,
 * flags = 0, then sample-major, channel, mode complex<double> values. */
inline void save_field(const Vector<Field>& data, const std::string& set, const std::string& tag,
                       const int& index) {
    std::ofstream file(set + "/" + tag + "/" + std::to_string(index) + ".bin", std::ios::binary);
    const int hdr[4] = {(int)data.size(), data.empty() ? 0 : data[0].samples(), data.empty() ? 0 : data[0].modes(), 0};
    file.write(reinterpret_cast<const char*>(hdr), sizeof hdr);
    for (int s = 0; s < hdr[1]; ++s)
        for (int ch = 0; ch < hdr[0]; ++ch)
            for (int m = 0; m < hdr[2]; ++m) {
                const complex_t v = data[(size_t)ch](m, s);
                file.write(reinterpret_cast<const char*>(&v), sizeof v);
            }
}
/* The channels back as fields of `domain` (modes and samples from the file). */
inline Vector<Field> load_field(const std::string& set, const std::string& tag, const int& index,
                                Domain domain) {
    std::ifstream file(set + "/" + tag + "/" + std::to_string(index) + ".bin", std::ios::binary);
    int hdr[4] = {0, 0, 0, 0};
    file.read(reinterpret_cast<char*>(hdr), sizeof hdr);
    if (!file) throw gpu_error(FOCSS_ERR_INVALID_ARG, "focss: cannot read field file header");
    domain.samples = hdr[1];
    domain.modes = hdr[2];
    Vector<ComplexVector> ch((size_t)hdr[0], ComplexVector((size_t)hdr[1] * hdr[2]));
    for (int s = 0; s < hdr[1]; ++s)
        for (int c = 0; c < hdr[0]; ++c)
            for (int m = 0; m < hdr[2]; ++m) {
                complex_t v;
                file.read(reinterpret_cast<char*>(&v), sizeof v);
                ch[(size_t)c][(size_t)m * hdr[1] + s] = v;
            }
    if (!file) throw gpu_error(FOCSS_ERR_INVALID_ARG, "focss: truncated field file");
    Vector<Field> out;
    for (auto& d : ch) out.emplace_back(domain, d);
    return out;
}

/* ------------------------------------------------------------ equalizers */
/* src/focss/equalizer/phase_shift_equalizer.cpp:1-46 */
class PhaseShiftEqualizer {
  public:
    PhaseShiftEqualizer() : angle_steps_(3600) {}
    explicit PhaseShiftEqualizer(const int& angle_steps) : angle_steps_(angle_steps) {}
    void set_angle_steps(const int& angle_steps) { angle_steps_ = angle_steps; }
    void train(const Field& desired, const Field& actual) { angles_ = estimate(desired, actual); }
    Field equalize(const Field& original) const {
        Field out(original);
        Vector<double> a = angles_;
        a.resize((size_t)original.batch(), angles_.empty() ? 0.0 : angles_.back());
        detail::check(focss_field_rotate(gpu_context(), out.mut(), a.data()), gpu_context());
        return out;
    }
    Field train_equalize(const Field& desired, const Field& actual) const {
        Field out(actual);
        Vector<double> a = estimate(desired, actual);
        detail::check(focss_field_rotate(gpu_context(), out.mut(), a.data()), gpu_context());
        return out;
    }
    double get_angle() const { return angles_.empty() ? 0.0 : angles_[0]; }
    const Vector<double>& get_angles() const { return angles_; }

  private:
    Vector<double> estimate(const Field& desired, const Field& actual) const {
        Vector<double> a((size_t)actual.batch());
        detail::check(focss_pse_estimate(gpu_context(), desired.handle(), actual.handle(), angle_steps_, a.data()),
                      gpu_context());
        return a;
    }
    int angle_steps_;
    Vector<double> angles_;
};

/* src/focss/equalizer/scalar_equalizer.cpp:1-33 */
class ScalarEqualizer {
  public:
    ScalarEqualizer() {}
    void train(const Field& desired, const Field& actual) { scalars_ = estimate(desired, actual); }
    Field equalize(const Field& original) const {
        Field out(original);
        Vector<double> s = scalars_;
        s.resize(2 * (size_t)original.batch(), 0.0);
        detail::check(focss_field_scale_each(gpu_context(), out.mut(), s.data()), gpu_context());
        return out;
    }
    Field train_equalize(const Field& desired, const Field& actual) const {
        Field out(actual);
        Vector<double> s = estimate(desired, actual);
        detail::check(focss_field_scale_each(gpu_context(), out.mut(), s.data()), gpu_context());
        return out;
    }
    complex_t get_scalar() const { return scalars_.size() >= 2 ? complex_t(scalars_[0], scalars_[1]) : complex_t(1, 0); }

  private:
    Vector<double> estimate(const Field& desired, const Field& actual) const {
        Vector<double> s(2 * (size_t)actual.batch());
        detail::check(focss_scalar_estimate(gpu_context(), desired.handle(), actual.handle(), s.data()), gpu_context());
        return s;
    }
    Vector<double> scalars_;
};

/* -------------------------------------------------- perturbation equalizers */
namespace detail {
/* x = G^-1 g for the fit's normal equations: gram is the (nf+1)^2 row-major
 * complex matrix [Z y]^H [Z y] (upper triangle valid), G its leading nf x nf
 * block, g its last column.  Right-looking Cholesky G = U^H U in FP64 on
 * the upper triangle (contiguous inner loops), then U^H w = g and U x = w;
 * with a residual function r(x) = Z^H (y - Z x) (evaluated in FP64 on the
 * GPU), `refinements` steps of iterative refinement x += G^-1 r(x). */
inline ComplexVector solve_normal_equations(const ComplexVector& gram, int nf,
                                            const std::function<ComplexVector(const ComplexVector&)>& residual = {},
                                            int refinements = 2) {
    const size_t n = (size_t)nf, w = n + 1;
    ComplexVector U(n * n);
    for (size_t i = 0; i < n; ++i)
        for (size_t j = i; j < n; ++j) U[i * n + j] = gram[i * w + j];
    for (size_t k = 0; k < n; ++k) {
        const double d = U[k * n + k].real();
        if (!(d > 0))
            throw gpu_error(FOCSS_ERR_INVALID_ARG, "focss: normal equations are not positive definite (rank-deficient design)");
        const double r = std::sqrt(d);
        U[k * n + k] = r;
        for (size_t j = k + 1; j < n; ++j) U[k * n + j] /= r;
        for (size_t i = k + 1; i < n; ++i) {
            const complex_t a = std::conj(U[k * n + i]);
            complex_t* row = &U[i * n];
            const complex_t* top = &U[k * n];
            for (size_t j = i; j < n; ++j) row[j] -= a * top[j];
        }
    }
    auto solve = [&](ComplexVector x) {
        for (size_t p = 0; p < n; ++p) {  // U^H w = b
            x[p] /= U[p * n + p].real();
            for (size_t i = p + 1; i < n; ++i) x[i] -= std::conj(U[p * n + i]) * x[p];
        }
        for (size_t i = n; i-- > 0;) {  // U x = w
            complex_t acc = x[i];
            for (size_t j = i + 1; j < n; ++j) acc -= U[i * n + j] * x[j];
            x[i] = acc / U[i * n + i].real();
        }
        return x;
    };
    ComplexVector g(n);
    for (size_t i = 0; i < n; ++i) g[i] = gram[i * w + n];
    ComplexVector x = solve(g);
    if (residual)
        for (int it = 0; it < refinements; ++it) {
            const ComplexVector d = solve(residual(x));
            for (size_t i = 0; i < n; ++i) x[i] += d[i];
        }
    return x;
}

/* The coefficient table of the symmetry-reduced triplet features
 * (src/focss/equalizer/sino.cpp:126-153, wdm_sino.cpp:105-128): R x R
 * diamond, C(m,n) = C(n,m) = C(-m,-n) = C(-n,-m); returns the next index. */
inline size_t fill_symmetric(ComplexVector& W, int R, const ComplexVector& raw, size_t index) {
    const size_t w = 2 * (size_t)R + 1;
    auto at = [&](int m, int n) -> complex_t& { return W[(size_t)(R + m) * w + (size_t)(R + n)]; };
    for (int m = -(R / 2); m <= R / 2; ++m)
        for (int n = std::abs(m); n <= R - std::abs(m); ++n) {
            const complex_t v = raw[index++];
            at(m, n) = v;
            if (m == n) {
                at(-m, -n) = v;
            } else if (m == -n) {
                at(n, m) = v;
            } else {
                at(n, m) = v;
                at(-m, -n) = v;
                at(-n, -m) = v;
            }
        }
    return index;
}

/* The 16-byte complex layout shared with the C ABI's interleaved doubles. */
inline double* cplx(ComplexVector& v) { return reinterpret_cast<double*>(v.data()); }
inline const double* cplx(const ComplexVector& v) { return reinterpret_cast<const double*>(v.data()); }
}  // namespace detail

/* src/focss/equalizer/sino.h:8-50.  train() forms the normal equations on
 * the GPU (focss_sino_gram) and solves them on the host in FP64: the
 * reference's least-squares solution for a full-rank design.  lambda is kept
 * for the interface; the reference's active solve does not use it either
 * (sino.cpp:114-118).  Unlike the reference, train() writes no
 * "data/mmm.csv": call save_matrix() for that file. */
enum SinoType { ORDINARY, FIXED, HOMOGENEOUS };

class SINO {
  public:
    SINO() : SINO(0) {}
    explicit SINO(const int& radius) : SINO(radius, 1.0, ORDINARY) {}
    SINO(const int& radius, const double& lambda) : SINO(radius, lambda, ORDINARY) {}
    SINO(const int& radius, const double& lambda, const SinoType& type)
        : radius_(radius), lambda_(lambda), type_(type), trained_(false) {}
    SINO& set_radius(const int& radius) { radius_ = radius; trained_ = false; return *this; }
    SINO& set_lambda(const double& lambda) { lambda_ = lambda; trained_ = false; return *this; }
    SINO& set_type(const SinoType& type) { type_ = type; trained_ = false; return *this; }
    SINO& set_linear_weight(const complex_t& w) { linear_weight_ = w; trained_ = false; return *this; }

    /* sino.cpp:42-159 */
    void train(const Field& transmitted, const Field& received) {
        const int nf = focss_sino_num_features(radius_, (int)type_);
        if (nf <= 0) throw gpu_error(FOCSS_ERR_INVALID_ARG, "focss: SINO radius must be >= 0");
        ComplexVector gram((size_t)(nf + 1) * (nf + 1)), mean((size_t)nf + 1);
        Vector<double> sd((size_t)nf);
        detail::check(focss_sino_gram(gpu_context(), transmitted.handle(), received.handle(), radius_, (int)type_,
                                      linear_weight_.real(), linear_weight_.imag(), detail::cplx(gram),
                                      detail::cplx(mean), sd.data()),
                      gpu_context());
        ComplexVector raw = detail::solve_normal_equations(gram, nf, [&](const ComplexVector& x) {
            ComplexVector r(x.size());
            detail::check(focss_sino_residual(gpu_context(), transmitted.handle(), received.handle(), radius_,
                                              (int)type_, linear_weight_.real(), linear_weight_.imag(),
                                              detail::cplx(x), detail::cplx(r)),
                          gpu_context());
            return r;
        });
        complex_t dot = 0;
        for (int i = 0; i < nf; ++i) {
            raw[(size_t)i] /= sd[(size_t)i];
            dot += raw[(size_t)i] * mean[(size_t)i];
        }
        intercept_ = mean[(size_t)nf] - dot;
        const size_t w = 2 * (size_t)radius_ + 1;
        weights_.assign(w * w, complex_t(0, 0));
        const size_t next = detail::fill_symmetric(weights_, radius_, raw, 0);
        if (type_ == ORDINARY) linear_weight_ = raw[next];
        else if (type_ == HOMOGENEOUS) linear_weight_ = 0.0;
        trained_ = true;
    }

    complex_t get_intercept() const { return intercept_; }
    complex_t get_linear_weight() const { return linear_weight_; }
    complex_t get_coo_weight() const { return weights_[(size_t)radius_ * (2 * radius_ + 1) + radius_]; }
    /* (2R+1)^2 row-major table W(m, n) = weights()[(R+m)(2R+1) + R+n]. */
    const ComplexVector& weights() const { return weights_; }

    /* sino.cpp:180-220 */
    Field linear(const Field& original) const { return linear_weight_ * original; }
    Field cubic(const Field& original) const {
        Terms t = terms();
        Field out(original.domain(), original.batch());
        detail::check(focss_triplet_apply(gpu_context(), original.handle(), radius_, (int)t.m.size(), t.m.data(),
                                          t.n.data(), detail::cplx(t.c), out.mut()),
                      gpu_context());
        return out;
    }
    /* (rx - cubic(tx)) / linear_weight (sino.cpp:188-191) */
    Field equalize(const Field& rx, const Field& tx) const { return equalize_with(rx, tx, linear_weight_); }
    /* linear + cubic (sino.cpp:183-186): (-a x - cubic(x)) / -1 */
    Field model(const Field& original) const {
        return equalize_with(original * (-linear_weight_), original, complex_t(-1, 0));
    }

    void save_matrix(const std::string& filename) const {
        std::ofstream f(filename);
        save_matrix(f);
    }
    /* sino.cpp:222-259: real, imaginary, modulus and argument tables */
    void save_matrix(std::ostream& output) const {
        const int w = 2 * radius_ + 1;
        for (int part = 0; part < 4; ++part) {
            if (part) output << "\n\n";
            for (int m = 0; m < w; ++m) {
                for (int n = 0; n < w; ++n) {
                    const complex_t v = weights_[(size_t)m * w + n];
                    output << (part == 0 ? v.real() : part == 1 ? v.imag() : part == 2 ? std::abs(v) : std::arg(v))
                           << ' ';
                }
                output << '\n';
            }
        }
    }

  private:
    struct Terms {
        Vector<std::int32_t> m, n;
        ComplexVector c;
    };
    /* the diamond |m| + |n| <= R of the table (sino.cpp:206-214) */
    Terms terms() const {
        if (!trained_) throw gpu_error(FOCSS_ERR_INVALID_ARG, "focss: SINO is not trained");
        Terms t;
        const int w = 2 * radius_ + 1;
        for (int m = -radius_; m <= radius_; ++m)
            for (int n = -(radius_ - std::abs(m)); n <= radius_ - std::abs(m); ++n) {
                t.m.push_back(m);
                t.n.push_back(n);
                t.c.push_back(weights_[(size_t)(m + radius_) * w + (n + radius_)]);
            }
        return t;
    }
    Field equalize_with(const Field& rx, const Field& tx, const complex_t& a) const {
        Terms t = terms();
        Field out(rx.domain(), rx.batch());
        detail::check(focss_sino_equalize(gpu_context(), rx.handle(), tx.handle(), radius_, (int)t.m.size(),
                                          t.m.data(), t.n.data(), detail::cplx(t.c), a.real(), a.imag(), out.mut()),
                      gpu_context());
        return out;
    }

    int radius_;
    double lambda_;
    SinoType type_;
    bool trained_;
    complex_t intercept_ = 0;
    complex_t linear_weight_ = 0;
    ComplexVector weights_;
};

/* src/focss/equalizer/wdm_sino.h:8-71 with Fields in place of arma::cx_mat:
 * inputs are 6-row Fields (rows channel * 2 + polarization: left neighbour
 * 0-1, centre 2-3, right neighbour 4-5, the layout load_field returns for
 * 3 channels x 2 modes); outputs are 2-row Fields (the centre channel).
 * train() forms the normal equations on the GPU (focss_wdm_ppe_gram) and
 * solves them on the host in FP64. */
class WdmPPE {
  public:
    WdmPPE() : WdmPPE(0, 0) {}
    explicit WdmPPE(const int& radii) : WdmPPE(radii, radii) {}
    WdmPPE(const int& c_radius, const int& d_radius) : c_(c_radius), d_(d_radius), trained_(false) {}
    WdmPPE& set_c_radius(const int& c_radius) { c_ = c_radius; trained_ = false; return *this; }
    WdmPPE& set_d_radius(const int& d_radius) { d_ = d_radius; trained_ = false; return *this; }

    /* wdm_sino.cpp:28-142 */
    void train(const Field& tx, const Field& rx) {
        const int nf = focss_wdm_ppe_num_features(c_, d_);
        ComplexVector gram((size_t)(nf + 1) * (nf + 1)), mean((size_t)nf + 1);
        Vector<double> sd((size_t)nf);
        detail::check(focss_wdm_ppe_gram(gpu_context(), tx.handle(), rx.handle(), c_, d_, detail::cplx(gram),
                                         detail::cplx(mean), sd.data()),
                      gpu_context());
        ComplexVector raw = detail::solve_normal_equations(gram, nf, [&](const ComplexVector& x) {
            ComplexVector r(x.size());
            detail::check(focss_wdm_ppe_residual(gpu_context(), tx.handle(), rx.handle(), c_, d_, detail::cplx(x),
                                                 detail::cplx(r)),
                          gpu_context());
            return r;
        });
        complex_t dot = 0;
        for (int i = 0; i < nf; ++i) {
            raw[(size_t)i] /= sd[(size_t)i];
            dot += raw[(size_t)i] * mean[(size_t)i];
        }
        intercept_ = mean[(size_t)nf] - dot;
        size_t index = 0;
        C_.assign(c_ >= 0 ? (size_t)(2 * c_ + 1) * (2 * c_ + 1) : 0, complex_t(0, 0));
        D_.assign(d_ >= 0 ? (size_t)(2 * d_ + 1) * (2 * d_ + 1) : 0, complex_t(0, 0));
        if (c_ >= 0) index = detail::fill_symmetric(C_, c_, raw, 0);
        for (int m = -d_; m <= d_; ++m)
            for (int n = -(d_ - std::abs(m)); n <= d_ - std::abs(m); ++n)
                D_[(size_t)(d_ + m) * (2 * d_ + 1) + (d_ + n)] = raw[index++];
        linear_weight_ = raw[index];
        trained_ = true;
    }

    complex_t get_intercept() const { return intercept_; }
    complex_t get_linear_weight() const { return linear_weight_; }
    complex_t get_coo_weight() const { return C_[(size_t)c_ * (2 * c_ + 1) + c_]; }
    /* (2c+1)^2 and (2d+1)^2 row-major tables, C(m, n) = C_table()[(c+m)(2c+1) + c+n] */
    const ComplexVector& C_table() const { return C_; }
    const ComplexVector& D_table() const { return D_; }

    /* wdm_sino.cpp:235-300 */
    Field linear(const Field& field) const { return apply(nullptr, nullptr, nullptr, &field); }
    Field spm(const Field& field) const { return apply(&field, nullptr, nullptr, nullptr); }
    Field xpm(const Field& field) const { return apply(nullptr, &field, nullptr, nullptr); }
    Field cubic(const Field& field) const {
        return apply(c_ >= 0 ? &field : nullptr, d_ >= 0 ? &field : nullptr, nullptr, nullptr);
    }
    Field model(const Field& field) const {
        return apply(c_ >= 0 ? &field : nullptr, d_ >= 0 ? &field : nullptr, nullptr, &field);
    }
    Field equalize(const Field& tx, const Field& rx) const { return equalize(tx, tx, rx); }
    Field equalize(const Field& tx_spm, const Field& tx_xpm, const Field& rx) const {
        return apply(c_ >= 0 ? &tx_spm : nullptr, d_ >= 0 ? &tx_xpm : nullptr, &rx, nullptr);
    }

  private:
    Field apply(const Field* spm_in, const Field* xpm_in, const Field* rx, const Field* lin_in) const {
        if (!trained_) throw gpu_error(FOCSS_ERR_INVALID_ARG, "focss: WdmPPE is not trained");
        const Field* ref = spm_in ? spm_in : xpm_in ? xpm_in : lin_in ? lin_in : rx;
        Domain dom = ref->domain();
        dom.modes = 2;
        Field out(dom, ref->batch());
        const complex_t zero[1] = {complex_t(0, 0)};
        detail::check(
            focss_wdm_ppe_apply(gpu_context(), spm_in ? spm_in->handle() : nullptr,
                                xpm_in ? xpm_in->handle() : nullptr, rx ? rx->handle() : nullptr,
                                lin_in ? lin_in->handle() : nullptr, c_,
                                C_.empty() ? reinterpret_cast<const double*>(zero) : detail::cplx(C_), d_,
                                D_.empty() ? reinterpret_cast<const double*>(zero) : detail::cplx(D_),
                                linear_weight_.real(), linear_weight_.imag(), out.mut()),
            gpu_context());
        return out;
    }

    int c_, d_;
    bool trained_;
    complex_t intercept_ = 0;
    complex_t linear_weight_ = 0;
    ComplexVector C_, D_;
};

}  // namespace focss

#endif  // FOCSS_GPU_HPP_
