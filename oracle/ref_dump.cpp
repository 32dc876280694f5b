// ref_dump.cpp -- TEST INFRASTRUCTURE ONLY: a driver compiled against the reference's own
// simulator library (simlib/sim_lib.h, simlib/simulator.cpp) that writes the raw FP64
// activation times and ECG of one run, so the oracle can be pinned bit for bit.  The
// reference's CLI prints only 6 significant digits (simlib/simulator.h:197-240).
//
// usage: ref_dump <ini> <out.bin> <layer-k hex file> [du0 dv0 du1 dv1 ...]
//   <layer-k hex file>: nlayers lines of 9 hexadecimal doubles (%a), the layer APs.
//   displacements (optional): lead moves in the u/v basis (simlib/sim_lib.h:197-208).
// out.bin: int64 nz, ny, nx, nlead, steps; then nz*ny*nx doubles (activation times after
// calculateExcitationSequence), then nlead*steps doubles (ECG, lead-major).
#include "sim_lib.h"
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

int main(int argc, char** argv) {
    if (argc < 4) { std::fprintf(stderr, "usage: ref_dump ini out.bin layerk.txt [disp...]\n"); return 2; }
    try {
        SimLib::EkgSim sim;
        sim.loadSettings(argv[1]);
        sim.loadTransferMatrix();
        sim.loadMeasuringPoints();
        sim.loadShape();
        sim.simExcitationSequence();
        sim.applySettings();
        const SimLib::ShapeMatrix& shape = sim.getModelShape();
        std::vector<double> at;
        for (size_t z = 0; z < shape.size()[0]; ++z)
            for (size_t y = 0; y < shape.size()[1]; ++y)
                for (size_t x = 0; x < shape.size()[2]; ++x) at.push_back(shape[z][y][x].excitationDelay);
        // layer APs
        std::vector<SimLib::ActionPotential> aps;
        {
            std::ifstream kf(argv[3]);
            std::string tok;
            std::vector<double> ks;
            while (kf >> tok) ks.push_back(std::strtod(tok.c_str(), nullptr));
            for (size_t i = 0; i + 9 <= ks.size(); i += 9) {
                SimLib::ActionPotential ap;
                ap.init(&ks[i], 0);
                aps.push_back(ap);
            }
        }
        if (argc > 4) {
            std::vector<SimLib::EkgSim::PositionVec> disp(sim.numMeasurements());
            for (size_t i = 0; i < disp.size(); ++i) {
                disp[i][0] = (4 + 2 * i < (size_t)argc) ? std::strtod(argv[4 + 2 * i], nullptr) : 0.0;
                disp[i][1] = (5 + 2 * i < (size_t)argc) ? std::strtod(argv[5 + 2 * i], nullptr) : 0.0;
                disp[i][2] = 0;
            }
            sim.moveMeasuringPoints(disp);
        }
        sim.setApsDestructive(aps);
        sim.run();
        int64_t hdr[5] = {(int64_t)shape.size()[0], (int64_t)shape.size()[1], (int64_t)shape.size()[2],
                          (int64_t)sim.numMeasurements(),
                          (int64_t)(sim.numMeasurements() ? sim.getMeasurement(0).size() : 0)};
        std::FILE* f = std::fopen(argv[2], "wb");
        std::fwrite(hdr, sizeof(hdr), 1, f);
        std::fwrite(at.data(), sizeof(double), at.size(), f);
        for (size_t l = 0; l < sim.numMeasurements(); ++l)
            std::fwrite(sim.getMeasurement(l).data(), sizeof(double), sim.getMeasurement(l).size(), f);
        std::fclose(f);
    } catch (std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
