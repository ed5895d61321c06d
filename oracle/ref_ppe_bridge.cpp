/*
 * ref_ppe_bridge.cpp -- extern "C" entry points over the reference's OWN
 * perturbation equalizers, focss::SINO (src/focss/equalizer/sino.cpp) and
 * focss::WdmPPE (src/focss/equalizer/wdm_sino.cpp), and over the decision
 * helpers of the WDM scoring task (find_certainty / sd / hd,
 * src/tasks/wdm_scoring.cpp:105-156).  Those unmodified sources are compiled
 * where they lie against the project's Armadillo stand-in
 * (oracle/arma_shim/armadillo), whose least-squares solve is Householder QR.
 *
 * TEST INFRASTRUCTURE ONLY: used in this container to pin the oracle
 * restatements and to write the golden vectors under tests/golden/.  The
 * product never links it.
 *
 * Matrices cross this boundary as row-major interleaved (re, im) doubles:
 * a field of `modes` x `samples`, a WdmPPE dataset of 6 x `samples`, and
 * weight tables of (2R+1) x (2R+1) indexed [R + m][R + n].
 */
#include <armadillo>
#include <complex>
#include <iostream>
#include <sstream>

#include "focss/definitions.h"
#include "focss/field.h"

// The trained tables have no accessor in the reference (only SINO::save_matrix
// prints them as text); this bridge reads and installs them directly.
#define private public
#include "focss/equalizer/sino.h"
#include "focss/equalizer/wdm_sino.h"
#undef private

using namespace focss;

// src/tasks/wdm_scoring.cpp (compiled alongside)
double find_certainty(const arma::cx_mat& tx, const arma::cx_mat& rx);
arma::cx_mat sd(const arma::cx_mat& field, const double& certainty);
arma::cx_mat hd(const arma::cx_mat& field);

namespace {
// The reference's training prints progress to std::cout; keep the test output clean.
struct Quiet {
    std::ostringstream sink;
    std::streambuf* old;
    Quiet() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~Quiet() { std::cout.rdbuf(old); }
};

Field make_field(int modes, int samples, const double* data) {
    Domain d{modes, samples, 1.0, 0.0};
    Field f(d);
    for (int m = 0; m < modes; ++m)
        for (int k = 0; k < samples; ++k) {
            const size_t i = (size_t)m * samples + k;
            f(m, k) = complex_t(data[2 * i], data[2 * i + 1]);
        }
    return f;
}
void store_field(const Field& f, double* out) {
    for (int m = 0; m < f.modes(); ++m)
        for (int k = 0; k < f.samples(); ++k) {
            const size_t i = (size_t)m * f.samples() + k;
            out[2 * i] = f(m, k).real();
            out[2 * i + 1] = f(m, k).imag();
        }
}
arma::cx_mat make_mat(int rows, int cols, const double* data) {
    arma::cx_mat a(rows, cols, arma::fill::zeros);
    for (int r = 0; r < rows; ++r)
        for (int c = 0; c < cols; ++c) {
            const size_t i = (size_t)r * cols + c;
            a(r, c) = complex_t(data[2 * i], data[2 * i + 1]);
        }
    return a;
}
void store_mat(const arma::cx_mat& a, double* out) {
    for (arma::uword r = 0; r < a.n_rows; ++r)
        for (arma::uword c = 0; c < a.n_cols; ++c) {
            const size_t i = (size_t)r * a.n_cols + c;
            out[2 * i] = a(r, c).real();
            out[2 * i + 1] = a(r, c).imag();
        }
}
void store_complex(complex_t v, double* out) {
    out[0] = v.real();
    out[1] = v.imag();
}
}  // namespace

extern "C" {

/* SINO::train (sino.cpp:42-159): weights (2R+1)^2, intercept, linear weight. */
void ref_sino_train(int modes, int samples, const double* tx, const double* rx, int radius, int type, double lw_re,
                    double lw_im, double* weights, double* intercept, double* linear_weight) {
    Quiet q;
    Field t = make_field(modes, samples, tx);
    Field r = make_field(modes, samples, rx);
    SINO s(radius, 1.0, static_cast<SinoType>(type));
    if (type == FIXED) s.set_linear_weight(complex_t(lw_re, lw_im));
    s.train(t, r);
    store_mat(s.weights_, weights);
    store_complex(s.get_intercept(), intercept);
    store_complex(s.get_linear_weight(), linear_weight);
}

/* SINO::cubic (sino.cpp:161-171, 203-220) with the given weight table. */
void ref_sino_cubic(int modes, int samples, const double* field, int radius, const double* weights, double* out) {
    SINO s(radius);
    s.weights_ = make_mat(2 * radius + 1, 2 * radius + 1, weights);
    s.trained_ = true;
    store_field(s.cubic(make_field(modes, samples, field)), out);
}

/* SINO::equalize (sino.cpp:193-196): (rx - cubic(tx)) / linear_weight. */
void ref_sino_equalize(int modes, int samples, const double* rx, const double* tx, int radius,
                       const double* weights, double lw_re, double lw_im, double* out) {
    SINO s(radius);
    s.weights_ = make_mat(2 * radius + 1, 2 * radius + 1, weights);
    s.linear_weight_ = complex_t(lw_re, lw_im);
    s.trained_ = true;
    store_field(s.equalize(make_field(modes, samples, rx), make_field(modes, samples, tx)), out);
}

/* WdmPPE::train (wdm_sino.cpp:28-142) on 6-row tx / rx datasets. */
void ref_wdm_ppe_train(int samples, const double* tx, const double* rx, int c_radius, int d_radius, double* C,
                       double* D, double* intercept, double* linear_weight) {
    Quiet q;
    WdmPPE p(c_radius, d_radius);
    p.train(make_mat(6, samples, tx), make_mat(6, samples, rx));
    store_mat(p.C_, C);
    store_mat(p.D_, D);
    store_complex(p.get_intercept(), intercept);
    store_complex(p.get_linear_weight(), linear_weight);
}

/* WdmPPE with the given tables: what = 0 spm, 1 xpm, 2 cubic, 3 model,
 * 4 equalize(tx, rx), 5 equalize(tx_spm, tx_xpm, rx) (wdm_sino.cpp:235-300);
 * inputs 6 x samples, output 2 x samples. */
void ref_wdm_ppe_apply(int samples, const double* a, const double* b, const double* rx, int c_radius,
                       const double* C, int d_radius, const double* D, double lw_re, double lw_im, int what,
                       double* out) {
    Quiet q;
    WdmPPE p(c_radius, d_radius);
    p.C_ = make_mat(2 * c_radius + 1, 2 * c_radius + 1, C);
    p.D_ = make_mat(2 * d_radius + 1, 2 * d_radius + 1, D);
    p.linear_weight_ = complex_t(lw_re, lw_im);
    p.trained_ = true;
    const arma::cx_mat A = make_mat(6, samples, a);
    arma::cx_mat y;
    switch (what) {
        case 0: y = p.spm(A); break;
        case 1: y = p.xpm(A); break;
        case 2: y = p.cubic(A); break;
        case 3: y = p.model(A); break;
        case 4: y = p.equalize(A, make_mat(6, samples, rx)); break;
        default: y = p.equalize(A, make_mat(6, samples, b), make_mat(6, samples, rx)); break;
    }
    store_mat(y, out);
}

/* find_certainty / sd / hd of the WDM scoring task (wdm_scoring.cpp:105-156). */
double ref_find_certainty(int rows, int cols, const double* tx, const double* rx) {
    return find_certainty(make_mat(rows, cols, tx), make_mat(rows, cols, rx));
}
void ref_certainty_sd(int rows, int cols, const double* field, double certainty, double* out) {
    store_mat(sd(make_mat(rows, cols, field), certainty), out);
}
void ref_hd_rms(int rows, int cols, const double* field, double* out) {
    store_mat(hd(make_mat(rows, cols, field)), out);
}

}  // extern "C"
