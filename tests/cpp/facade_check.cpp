// Drives the C++ façade the way the reference's Simulator does
// (Source/Simulator.cpp:33-63, 85-103): setupScene -> makeReady ->
// advanceFrame until the frame's 1/30 s accumulates, for `frames` frames.
// Writes the final positions and velocities (caller order, float32) to the
// output file.  Used by tests/test_facade.py.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>

#include "simplefluid/SPHSolver.hpp"

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s <scene> <frames> <out.bin>\n", argv[0]);
        return 2;
    }
    try {
        simplefluid::Simulator sim;
        auto params = sim.getSimParams();
        params->scene = std::atoi(argv[1]);
        const int frames = std::atoi(argv[2]);
        params->stopTime = 0.0333333333f * (float)frames - 1e-6f;
        int substeps = 0, nframes = 0;
        unsigned int nparticles = 0;
        sim.particleChanged = [&] { ++substeps; };
        sim.frameFinished = [&] { ++nframes; };
        sim.numParticleChanged = [&](unsigned int n) { nparticles = n; };
        sim.setupScene();
        substeps = 0;
        sim.startSimulation();
        sim.wait();
        const auto& pos = sim.solver().particles();
        const auto& vel = sim.solver().velocity();
        std::ofstream out(argv[3], std::ios::binary);
        const uint32_t n = (uint32_t)pos.size();
        out.write(reinterpret_cast<const char*>(&n), sizeof(n));
        out.write(reinterpret_cast<const char*>(&substeps), sizeof(substeps));
        out.write(reinterpret_cast<const char*>(&nframes), sizeof(nframes));
        out.write(reinterpret_cast<const char*>(pos.data()), n * sizeof(simplefluid::Vec3f));
        out.write(reinterpret_cast<const char*>(vel.data()), n * sizeof(simplefluid::Vec3f));
        std::printf("particles=%u substeps=%d frames=%d simtime=%.6f\n", nparticles, substeps, nframes, sim.simTime());
        // a healthy state after the run
        const sf_state_report rep = sim.solver().checkState();
        if (rep.n != n || rep.non_finite || rep.outside_box || rep.unsorted || rep.cell_table_mismatch ||
            rep.bad_ids) {
            std::fprintf(stderr, "state check failed\n");
            return 1;
        }
        // the same frames with no per-sub-step observer run on the device
        {
            simplefluid::Simulator sim2;
            *sim2.getSimParams() = *params;
            int frames2 = 0;
            sim2.frameFinished = [&] { ++frames2; };
            sim2.setupScene();
            sim2.startSimulation();
            sim2.wait();
            const auto& pos2 = sim2.solver().particles();
            if (frames2 != nframes || pos2.size() != pos.size() ||
                std::memcmp(pos2.data(), pos.data(), pos.size() * sizeof(simplefluid::Vec3f)) != 0) {
                std::fprintf(stderr, "device frame loop differs from the per-sub-step loop\n");
                return 1;
            }
        }
        // the error path: an invalid parameter throws simplefluid::Error
        try {
            params->kernelRadius = -1.f;
            params->updateParams();
            std::fprintf(stderr, "expected an error\n");
            return 1;
        } catch (const simplefluid::Error& e) {
            if (e.status != SF_ERR_INVALID_ARGUMENT) return 1;
        }
    } catch (const simplefluid::Error& e) {
        std::fprintf(stderr, "error %d: %s\n", e.status, e.what());
        return 1;
    }
    return 0;
}
