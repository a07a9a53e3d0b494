// facade_check.cpp — drives include/pbf_simulation.hpp the way the reference's
// frame loop drives its Simulation (src/Runner.cpp:46-127): LoadParameters,
// InitBuffers, InitCells, LoadForceMasks, InitKernels, then Step() subSteps
// times per frame.
//
//   facade_check <scenario.par> <init_pos.bin> <frames> <out.bin>
//
// init_pos.bin holds particleCount float4 records; out.bin receives the final
// positions followed by the final velocities.  Exit codes: 0 ok, 2 usage or
// I/O error, 3 a library error (message on stderr).
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <vector>

#include "pbf_simulation.hpp"

int main(int argc, char** argv) {
    if (argc != 5) {
        std::cerr << "usage: facade_check <scenario.par> <init_pos.bin> <frames> <out.bin>\n";
        return 2;
    }
    std::ifstream par(argv[1]);
    std::stringstream text;
    text << par.rdbuf();
    try {
        LoadParameters(text.str());
        const size_t n = Params.particleCount;
        std::vector<float> pos(4 * n), vel(4 * n);
        std::ifstream in(argv[2], std::ios::binary);
        if (!in.read(reinterpret_cast<char*>(pos.data()), pos.size() * sizeof(float))) {
            std::cerr << "cannot read " << argv[2] << "\n";
            return 2;
        }
        Simulation simulation(0);
        simulation.InitBuffers(pos.data(), nullptr);
        simulation.InitCells();
        simulation.LoadForceMasks();
        if (!simulation.InitKernels()) {
            std::cerr << "InitKernels failed\n";
            return 3;
        }
        simulation.TrackPerformance(true);
        const int frames = std::atoi(argv[3]);
        for (int f = 0; f < frames; ++f)
            for (unsigned i = 0; i < Params.subSteps; ++i) simulation.Step();
        simulation.ReadState(pos.data(), vel.data());
        std::ofstream out(argv[4], std::ios::binary);
        out.write(reinterpret_cast<const char*>(pos.data()), pos.size() * sizeof(float));
        out.write(reinterpret_cast<const char*>(vel.data()), vel.size() * sizeof(float));
        for (const auto* t : simulation.PerfData.Trackers) std::cout << t->eventName << " " << t->total_time << "\n";
    } catch (const std::runtime_error& e) {
        std::cerr << "error: " << e.what() << "\n";
        return 3;
    }
    return 0;
}
