// Perturbation equalizers through the C++ facade (include/focss_gpu.hpp) in
// the reference's idiom (src/tasks/sp_scoring.cpp:29-50,
// src/tasks/wdm_scoring.cpp:168-175): WdmPPE(8, 2) trained on a 6-row
// transmitted / received pair, SINO(6) on its centre channel, then their
// tables, equalizer and model outputs, plus the decision certainty.
//
// usage: facade_ppe <tx6.c128> <rx6.c128> <samples> <out_prefix>
// writes <out_prefix>_wdm_C.c128, _wdm_D.c128, _wdm_eq.c128, _wdm_model.c128,
// _sino_W.c128, _sino_eq.c128, _sino_model.c128 and _scalars.txt
// ("wdm_lw.re wdm_lw.im wdm_b.re wdm_b.im sino_lw.re sino_lw.im sino_b.re sino_b.im certainty").
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "focss_gpu.hpp"

namespace {
focss::ComplexVector read_c128(const std::string& path, size_t n) {
    focss::ComplexVector v(n);
    std::ifstream f(path, std::ios::binary);
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(focss::complex_t)));
    if (!f) throw std::runtime_error("cannot read " + path);
    return v;
}
void write_c128(const std::string& path, const focss::ComplexVector& v) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(focss::complex_t)));
}
}  // namespace

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s tx6.c128 rx6.c128 samples out_prefix\n", argv[0]);
        return 2;
    }
    const int n = std::atoi(argv[3]);
    const std::string out = argv[4];
    try {
        const focss::Domain d6{6, n, 1.0 / 32e9, 0.0};
        const focss::ComplexVector t6 = read_c128(argv[1], 6 * (size_t)n);
        const focss::ComplexVector r6 = read_c128(argv[2], 6 * (size_t)n);
        focss::Field tx(d6, t6), rx(d6, r6);

        focss::WdmPPE ppe(8, 2);
        ppe.train(tx, rx);
        write_c128(out + "_wdm_C.c128", ppe.C_table());
        write_c128(out + "_wdm_D.c128", ppe.D_table());
        write_c128(out + "_wdm_eq.c128", ppe.equalize(tx, rx).data());
        write_c128(out + "_wdm_model.c128", ppe.model(tx).data());

        // the centre channel as a 2-mode field for SINO
        const focss::Domain d2{2, n, 1.0 / 32e9, 0.0};
        focss::ComplexVector tc(t6.begin() + 2 * n, t6.begin() + 4 * n), rc(r6.begin() + 2 * n, r6.begin() + 4 * n);
        focss::Field tcf(d2, tc), rcf(d2, rc);
        focss::SINO sino(6);
        sino.train(tcf, rcf);
        write_c128(out + "_sino_W.c128", sino.weights());
        write_c128(out + "_sino_eq.c128", sino.equalize(rcf, tcf).data());
        write_c128(out + "_sino_model.c128", sino.model(tcf).data());

        const double certainty = focss::find_certainty(tx, rx);
        std::ofstream s(out + "_scalars.txt");
        s.precision(17);
        const focss::complex_t v[4] = {ppe.get_linear_weight(), ppe.get_intercept(), sino.get_linear_weight(),
                                       sino.get_intercept()};
        for (const auto& x : v) s << x.real() << " " << x.imag() << " ";
        s << certainty << "\n";
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 3;
    }
    return 0;
}
