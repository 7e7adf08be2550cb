// Build shim: the declarations that let the reference's own
// Source/Simulator.cpp compile here without Qt, TBB or the Banana library.
// It declares the interface of the reference's Include/Simulator.h (the
// members and methods Simulator.cpp uses).  Qt's signals become calls that
// record what the frame loop reports, and the solver returns a given sequence
// of sub-step sizes instead of simulating.  It contains no frame-loop logic:
// that comes from the reference's source.  Used only by build_ref.sh.
#pragma once
#include <cstdint>
#include <future>
#include <memory>
#include <vector>

#include "SceneManager.h"

#define emit
#define Q_ASSERT(cond) ((void)(cond))

namespace tbb {
class task_scheduler_init {
public:
    static const int automatic = -1;
    explicit task_scheduler_init(int) {}
};
}  // namespace tbb

// What the reference's frame loop sees and reports during one run.
struct FrameScript {
    std::vector<float> dts;                 // the sub-step sizes the solver returns, in order
    size_t next = 0;
    bool exhausted = false;                 // the loop asked for more sub-steps than given
    uint32_t in_frame = 0;                  // sub-steps since the last frameFinished
    std::vector<uint32_t> frame_substeps;   // per frameFinished
    std::vector<float> sim_times;           // per systemTimeChanged
};
extern FrameScript* g_frame_script;

class ParticleSystemData {
public:
    void setNumParticles(unsigned int) {}
    void setUInt(const char*, unsigned int) {}
    void setParticleRadius(float) {}
};

class QtSPHSolver {
public:
    void makeReady() {}
    float advanceFrame() {
        FrameScript* s = g_frame_script;
        ++s->in_frame;
        if (s->next < s->dts.size()) return s->dts[s->next++];
        s->exhausted = true;
        return 1.0f;  // ends the frame and the run
    }
    unsigned int getNumParticles() { return static_cast<unsigned int>(m_particles.size()); }
    Vec_Vec3<float>& getParticles() { return m_particles; }
    Vec_Vec3<float>& getVelocity() { return m_velocity; }

private:
    Vec_Vec3<float> m_particles, m_velocity;
};

class Simulator {
public:
    explicit Simulator(const std::shared_ptr<ParticleSystemData>& particleData) : m_ParticleData(particleData) {
        m_SPHSolver = std::make_unique<QtSPHSolver>();
        m_SceneManager = std::make_unique<SceneManager>(m_SimParams);
    }
    const std::shared_ptr<SPHParameters<float> >& getSimParams() { return m_SimParams; }
    bool isRunning() { return !m_bStop; }
    void stop();
    void reset();
    void startSimulation();
    void doSimulation();
    void changeScene(SimulationScenes::Scene scene);
    void setupScene();

    // the signals
    void simulationFinished() {}
    void systemTimeChanged(float time) { g_frame_script->sim_times.push_back(time); }
    void numParticleChanged(unsigned int) {}
    void particleChanged() {}
    void frameFinished() {
        g_frame_script->frame_substeps.push_back(g_frame_script->in_frame);
        g_frame_script->in_frame = 0;
    }

protected:
    std::unique_ptr<tbb::task_scheduler_init> m_ThreadInit = nullptr;
    volatile bool m_bStop = true;
    std::shared_ptr<ParticleSystemData> m_ParticleData = nullptr;
    float m_SimTime = 0;
    std::unique_ptr<SceneManager> m_SceneManager = nullptr;
    std::unique_ptr<QtSPHSolver> m_SPHSolver = nullptr;
    std::shared_ptr<SPHParameters<float> > m_SimParams = std::make_shared<SPHParameters<float> >();
    std::future<void> m_SimulationFutureObj;
};
