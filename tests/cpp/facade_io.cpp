// Writes a transmission file through the C++ façade (focss::save_transmission,
// src/focss/functions.cpp:174-208) from two device fields, reads it back with
// focss::load_transmission and writes the round trip to <out>.back.
//
// usage: facade_io <in.c128: tx (2 x 40) then rx (2 x 40)> <out.csv>
#include <cstdio>
#include <fstream>
#include <vector>

#include "focss_gpu.hpp"

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const int modes = 2, samples = 40;
    std::vector<focss::complex_t> buf(2 * modes * samples);
    std::ifstream in(argv[1], std::ios::binary);
    in.read(reinterpret_cast<char*>(buf.data()), (std::streamsize)(buf.size() * sizeof(focss::complex_t)));
    try {
        const focss::Domain d{modes, samples, 1.0, 0.0};
        focss::Field tx(d, focss::ComplexVector(buf.begin(), buf.begin() + modes * samples));
        focss::Field rx(d, focss::ComplexVector(buf.begin() + modes * samples, buf.end()));
        focss::save_transmission(argv[2], tx, rx);
        focss::Field tx2(d), rx2(d);
        focss::load_transmission(argv[2], &tx2, &rx2);
        focss::save_transmission(std::string(argv[2]) + ".back", tx2, rx2);
    } catch (const focss::gpu_error& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 3;
    }
    return 0;
}
