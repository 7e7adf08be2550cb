// C entry point around the reference's own frame loop (Simulator::doSimulation,
// compiled from the reference source by build_ref.sh with the shim in
// ref_shim/Simulator.h).  TEST INFRASTRUCTURE ONLY: it pins the frame
// accounting of the oracle and of the product against the reference.
#include <cstdint>
#include <memory>

#include "Simulator.h"

FrameScript* g_frame_script = nullptr;

namespace {
struct Runner : Simulator {
    using Simulator::Simulator;
    void run(float stop_time) {
        m_SimParams->stopTime = stop_time;
        startSimulation();
        m_SimulationFutureObj.wait();
    }
};
}  // namespace

// Runs doSimulation with a solver that returns dts[0..ndts) in turn, until the
// simulated time reaches stop_time.  Per frame, frame_substeps receives the
// sub-steps taken and sim_times the simulated time reported after the frame
// (float, as the reference keeps it).  Returns 0, 1 if more than cap frames
// ran, 2 if the loop asked for more sub-steps than given.
extern "C" int ref_frames(const float* dts, uint32_t ndts, float stop_time, uint32_t cap, uint32_t* frame_substeps,
                          float* sim_times, uint32_t* nframes) {
    FrameScript script;
    script.dts.assign(dts, dts + ndts);
    g_frame_script = &script;
    {
        Runner sim(std::make_shared<ParticleSystemData>());
        sim.run(stop_time);
    }
    g_frame_script = nullptr;
    const uint32_t nf = (uint32_t)script.frame_substeps.size();
    if (nframes) *nframes = nf;
    if (script.exhausted) return 2;
    if (nf > cap || script.sim_times.size() != nf) return 1;
    for (uint32_t f = 0; f < nf; ++f) {
        frame_substeps[f] = script.frame_substeps[f];
        sim_times[f] = script.sim_times[f];
    }
    return 0;
}
