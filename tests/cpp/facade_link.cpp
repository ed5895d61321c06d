// Single-channel link written against the C++ facade (include/focss_gpu.hpp)
// in the reference's own idiom (src/tasks/sp_run.cpp:10-53,
// src/tasks/systems.cpp:26-71): 16QAM -> RRC shaping -> `spans` x 80 km SSMF,
// UNIFORM 1 km steps, lossless EDFA without noise -> CDC -> matched filter ->
// phase-shift equalizer -> Q, BER, decisions, decision certainty.
//
// usage: facade_link <codes.i32> <out_prefix> [spans]
// writes <out_prefix>_sym.c128 (symbols), _tx.c128 (transmitted field), _after.c128 (after the
// spans), _rx.c128 (equalized symbols), _codes.i32 (decisions) and
// _metrics.txt ("q ber certainty").
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "focss_gpu.hpp"

namespace {
template <class T>
void write_vec(const std::string& path, const std::vector<T>& v) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}
}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s codes.i32 out_prefix [spans]\n", argv[0]);
        return 2;
    }
    const int spans = argc > 3 ? std::atoi(argv[3]) : 10;
    std::ifstream in(argv[1], std::ios::binary | std::ios::ate);
    const size_t bytes = (size_t)in.tellg();
    in.seekg(0);
    std::vector<int> codes(bytes / sizeof(int));
    in.read(reinterpret_cast<char*>(codes.data()), (std::streamsize)bytes);
    const std::string out = argv[2];

    const int osf = 8;
    const double baud = 32e9, roll_off = 0.1;
    const focss::Fiber fiber = {focss::db_to_natural(2e-4), focss::disp_to_beta2(1.7e-5, 1.55e-6), 1.3e-3, 80e3,
                                1.55e-6, 1.0};
    try {
        const int n = (int)codes.size();
        focss::Field symbols = focss::qam16_symbols(codes, focss::Domain{1, n, 1.0 / baud, 0.0});
        symbols *= std::sqrt(focss::dbm_to_watts(2.0));
        write_vec(out + "_sym.c128", symbols.data());
        focss::Field signal = focss::rrc_shaping(symbols, osf, 1.0, roll_off);
        write_vec(out + "_tx.c128", signal.data());

        focss::SSFM ssfm(fiber);
        ssfm.set_grid(focss::SSFM::UNIFORM);
        ssfm.set_total_steps(80);
        focss::Amplifier amplifier(focss::db_to_linear(2e-4 * 80e3));
        for (int i = 0; i < spans; ++i) {
            ssfm.run(signal, focss::SSFM::FORWARD);
            amplifier.amplify(signal);
        }
        write_vec(out + "_after.c128", signal.data());

        focss::SSFM cdc(fiber.dispersive() * spans, 1);
        cdc.run(signal, focss::SSFM::BACKWARD);
        focss::Field rx = focss::rrc_sampling(signal, osf, 1.0, roll_off);
        rx = focss::PhaseShiftEqualizer(3600).train_equalize(symbols, rx);
        const double q = focss::q2_factor(symbols, rx, 100);
        const double ber = focss::bit_error_rate_16qam(symbols, rx, 100);
        const double certainty = focss::find_certainty(symbols, rx);
        const focss::Field snapped = focss::sd(rx, certainty);
        if (snapped.size() != rx.size() || focss::hd(rx).size() != rx.size()) return 4;
        write_vec(out + "_rx.c128", rx.data());
        write_vec(out + "_codes.i32", focss::hd_sequence_16qam(rx));
        std::ofstream m(out + "_metrics.txt");
        m.precision(17);
        m << q << " " << ber << " " << certainty << "\n";
        std::printf("Q %.4f dB  BER %.3e\n", q, ber);
    } catch (const focss::gpu_error& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 3;
    }
    return 0;
}
