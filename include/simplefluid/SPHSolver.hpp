// simplefluid/SPHSolver.hpp — C++ host façade over the C ABI (sf_capi.h).
//
// Mirrors the solver-facing classes of the reference so that its call sites
// compile against this header:
//
//   SPHParameters<float>          fields of Source/Controller.cpp:54-61 (+ particleRadius,
//                                 scene: Source/SceneManager.cpp:23,45), updateParams() (:63)
//   SPHSolver / QtSPHSolver       makeReady() (Source/Simulator.cpp:42), advanceFrame() (:49),
//                                 getNumParticles/getParticles/getVelocity (Include/QtSPHSolver.h:33-35)
//   SceneManager                  setupScene(particles, velocity) (Source/SceneManager.cpp:21-38)
//   Simulator                     headless doSimulation/stop/reset/changeScene/setupScene
//                                 (Source/Simulator.cpp:22-103), Qt signals as std::function
//
// The particle state lives on the GPU.  getParticles()/getVelocity() return a
// host mirror (std::vector of 3-float vectors, the layout of Vec_Vec3<float>):
// fetched from the device when it is out of date, and — because the returned
// reference is writable, as in the reference where SceneManager fills it —
// uploaded again before the next makeReady()/advanceFrame().  Errors throw
// simplefluid::Error carrying the sf_status and sf_last_error().
#pragma once

#include <array>
#include <atomic>
#include <cstdint>
#include <functional>
#include <future>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../sf_capi.h"

namespace simplefluid {

class Error : public std::runtime_error {
public:
    Error(sf_status st, const std::string& what) : std::runtime_error(what), status(st) {}
    sf_status status;
};

inline void check(sf_status st) {
    if (st != SF_OK) throw Error(st, std::string("simplefluid: ") + sf_last_error());
}

using Vec3f = std::array<float, 3>;
using Vec_Vec3f = std::vector<Vec3f>;
static_assert(sizeof(Vec3f) == 3 * sizeof(float), "Vec3f must be three packed floats");

struct SimulationScenes {
    enum Scene { SphereDrop = SF_SCENE_SPHERE_DROP, CubeDrop, Dambreak, DoubleDambreak };
};

// SPHParameters<float>: the fields the reference GUI edits plus the constants
// its solver library keeps internally (fixed here by the workloads).
template <typename Real = float>
struct SPHParameters {
    int numThreads = 0;
    Real kernelRadius = Real(0.04);
    Real particleRadius = Real(0.01);
    Real pressureStiffness = Real(50);
    Real boundaryRestitution = Real(0.1);
    Real viscosity = Real(0.01);
    Real stopTime = Real(5);
    bool bUseAttractivePressure = false;
    int scene = SF_SCENE_DAMBREAK_16K;
    Real restDensity = Real(1000);
    std::array<Real, 3> gravity{Real(0), Real(-9.8), Real(0)};
    Real timeStep = Real(1e-4);
    std::array<Real, 3> boxMin{Real(0), Real(0), Real(0)};
    std::array<Real, 3> boxMax{Real(1), Real(1), Real(1)};
    int eos = SF_EOS_LINEAR;
    int cellsPerH = 2;
    bool adaptiveTimeStep = false;

    sf_params toC() const {
        sf_params p{};
        check(sf_params_default(&p));
        p.num_threads = numThreads;
        p.kernel_radius = (float)kernelRadius;
        p.particle_radius = (float)particleRadius;
        p.pressure_stiffness = (float)pressureStiffness;
        p.boundary_restitution = (float)boundaryRestitution;
        p.viscosity = (float)viscosity;
        p.stop_time = (float)stopTime;
        p.use_attractive_pressure = bUseAttractivePressure ? 1 : 0;
        p.scene = scene;
        p.rest_density = (float)restDensity;
        for (int a = 0; a < 3; ++a) {
            p.gravity[a] = (float)gravity[a];
            p.box_min[a] = (float)boxMin[a];
            p.box_max[a] = (float)boxMax[a];
        }
        p.time_step = (float)timeStep;
        p.eos = eos;
        p.cells_per_h = cellsPerH;
        p.adaptive_time_step = adaptiveTimeStep ? 1 : 0;
        return p;
    }

    // SPHParameters::updateParams(): validate (throws on a bad value).
    void updateParams() const {
        sf_params p = toC();
        check(sf_params_update(&p));
    }
};

// SPHSolver<float> (as used through QtSPHSolver) on one GB300.
class SPHSolver {
public:
    explicit SPHSolver(std::shared_ptr<SPHParameters<float>> params) : m_Params(std::move(params)) {
        const sf_params p = m_Params->toC();
        check(sf_create(&p, &m_Ctx));
    }
    ~SPHSolver() { sf_destroy(m_Ctx); }
    SPHSolver(const SPHSolver&) = delete;
    SPHSolver& operator=(const SPHSolver&) = delete;

    // Re-read the shared parameters (after the caller edited them).
    void updateParams() {
        const sf_params p = m_Params->toC();
        check(sf_set_params(m_Ctx, &p));
    }

    void makeReady() {
        upload_if_dirty();
        check(sf_make_ready(m_Ctx));
    }

    // One sub-step; returns the simulated time advanced.
    float advanceFrame() {
        upload_if_dirty();
        float dt = 0.f;
        check(sf_advance_frame(m_Ctx, &dt));
        m_HostStale = true;
        return dt;
    }

    // `n` sub-steps queued as graph replays (no host round trip).
    void advanceSteps(uint32_t n) {
        upload_if_dirty();
        check(sf_step(m_Ctx, n));
        m_HostStale = true;
    }

    // Whole frames on the device (sub-steps until frame_time, one graph
    // launch per frame); returns the simulated time advanced.
    double advanceFrames(uint32_t frames, double frame_time = 0.0333333333, uint32_t max_substeps = 100000,
                         uint32_t* substeps = nullptr) {
        upload_if_dirty();
        double t = 0.0;
        check(sf_advance_frames(m_Ctx, frames, frame_time, max_substeps, &t, substeps));
        m_HostStale = true;
        return t;
    }

    unsigned int getNumParticles() {
        if (m_HostDirty) return (unsigned int)m_Particles.size();
        uint32_t n = 0;
        check(sf_get_num_particles(m_Ctx, &n));
        return n;
    }

    Vec_Vec3f& getParticles() {
        download_if_stale();
        m_HostDirty = true;
        return m_Particles;
    }

    Vec_Vec3f& getVelocity() {
        download_if_stale();
        m_HostDirty = true;
        return m_Velocity;
    }

    // Read-only access that does not schedule a re-upload.
    const Vec_Vec3f& particles() {
        download_if_stale();
        return m_Particles;
    }
    const Vec_Vec3f& velocity() {
        download_if_stale();
        return m_Velocity;
    }

    void synchronize() { check(sf_synchronize(m_Ctx)); }

    // Invariants of the device state (sf_check_state): non-finite values,
    // particles outside the box, sort and particle-index consistency.
    sf_state_report checkState() {
        upload_if_dirty();
        sf_state_report r{};
        check(sf_check_state(m_Ctx, &r));
        return r;
    }

    sf_ctx* handle() { return m_Ctx; }
    const std::shared_ptr<SPHParameters<float>>& params() const { return m_Params; }

private:
    void upload_if_dirty() {
        if (!m_HostDirty) return;
        if (m_Velocity.size() != m_Particles.size()) m_Velocity.assign(m_Particles.size(), Vec3f{0.f, 0.f, 0.f});
        check(sf_set_state(m_Ctx, m_Particles.empty() ? nullptr : m_Particles.data()->data(),
                           m_Velocity.empty() ? nullptr : m_Velocity.data()->data(), (uint32_t)m_Particles.size()));
        m_HostDirty = false;
        m_HostStale = false;
    }

    void download_if_stale() {
        if (!m_HostStale) return;
        uint32_t n = 0;
        check(sf_get_num_particles(m_Ctx, &n));
        m_Particles.resize(n);
        m_Velocity.resize(n);
        if (n) check(sf_get_state(m_Ctx, m_Particles.data()->data(), m_Velocity.data()->data(), n));
        m_HostStale = false;
    }

    std::shared_ptr<SPHParameters<float>> m_Params;
    sf_ctx* m_Ctx = nullptr;
    Vec_Vec3f m_Particles, m_Velocity;
    bool m_HostDirty = false;  // host vectors may hold edits not yet on the device
    bool m_HostStale = false;  // the device holds a newer state than the host vectors
};

// SceneManager (Source/SceneManager.cpp:21-173).
class SceneManager {
public:
    explicit SceneManager(std::shared_ptr<SPHParameters<float>> params, uint64_t seed = 20171)
        : m_SimParams(std::move(params)), m_Seed(seed) {}

    void setupScene(Vec_Vec3f& particles, Vec_Vec3f& velocity) { make(m_SimParams->scene, particles, velocity); }
    void setupSceneCubeDrop(Vec_Vec3f& p, Vec_Vec3f& v) { make(SF_SCENE_CUBE_DROP, p, v); }
    void setupSceneSphereDrop(Vec_Vec3f& p, Vec_Vec3f& v) { make(SF_SCENE_SPHERE_DROP, p, v); }
    void setupSceneDambreak(Vec_Vec3f& p, Vec_Vec3f& v) { make(SF_SCENE_DAMBREAK, p, v); }
    void setupSceneDoubleDambreak(Vec_Vec3f& p, Vec_Vec3f& v) { make(SF_SCENE_DOUBLE_DAMBREAK, p, v); }

private:
    void make(int scene, Vec_Vec3f& particles, Vec_Vec3f& velocity) {
        const sf_params p = m_SimParams->toC();
        uint32_t n = 0;
        check(sf_scene_count(&p, scene, m_Seed, &n));
        particles.resize(n);
        velocity.assign(n, Vec3f{0.f, 0.f, 0.f});
        if (n) check(sf_setup_scene(&p, scene, m_Seed, particles.data()->data(), nullptr, n, &n));
    }

    std::shared_ptr<SPHParameters<float>> m_SimParams;
    uint64_t m_Seed;
};

// Headless Simulator (Source/Simulator.cpp:22-103).  The frame loop runs on a
// std::async worker; the Qt signals become optional callbacks.
class Simulator {
public:
    Simulator()
        : m_SimParams(std::make_shared<SPHParameters<float>>()),
          m_SPHSolver(std::make_unique<SPHSolver>(m_SimParams)),
          m_SceneManager(std::make_unique<SceneManager>(m_SimParams)) {}
    ~Simulator() {
        stop();
        if (m_Future.valid()) m_Future.wait();
    }

    std::function<void()> particleChanged, frameFinished, simulationFinished;
    std::function<void(float)> systemTimeChanged;
    std::function<void(unsigned int)> numParticleChanged;

    const std::shared_ptr<SPHParameters<float>>& getSimParams() { return m_SimParams; }
    SPHSolver& solver() { return *m_SPHSolver; }
    bool isRunning() const { return !m_bStop; }
    float simTime() const { return m_SimTime; }

    void startSimulation() {
        m_bStop = false;
        if (m_Future.valid()) m_Future.wait();
        m_Future = std::async(std::launch::async, [this] { doSimulation(); });
    }

    void wait() {
        if (m_Future.valid()) m_Future.get();
    }

    void doSimulation() {
        m_SPHSolver->updateParams();
        m_SPHSolver->makeReady();
        while (m_SimTime < m_SimParams->stopTime && !m_bStop) {
            float frameTime = 0;
            if (!particleChanged) {
                // no per-sub-step observer: the whole frame on the device
                frameTime = (float)m_SPHSolver->advanceFrames(1);
            } else {
                while (frameTime < 0.0333333333) {
                    frameTime += m_SPHSolver->advanceFrame();
                    particleChanged();
                }
            }
            m_SimTime += frameTime;
            if (systemTimeChanged) systemTimeChanged(m_SimTime);
            if (frameFinished) frameFinished();
        }
        m_SPHSolver->synchronize();
        if (!m_bStop) {
            m_bStop = true;
            if (simulationFinished) simulationFinished();
        }
    }

    void stop() { m_bStop = true; }

    void reset() {
        m_bStop = true;
        setupScene();
    }

    void changeScene(int scene) {
        m_SimParams->scene = scene;
        setupScene();
    }

    void setupScene() {
        m_SimTime = 0;
        if (systemTimeChanged) systemTimeChanged(m_SimTime);
        if (m_Future.valid()) m_Future.wait();
        m_SPHSolver->updateParams();
        m_SceneManager->setupScene(m_SPHSolver->getParticles(), m_SPHSolver->getVelocity());
        if (particleChanged) particleChanged();
        if (numParticleChanged) numParticleChanged(m_SPHSolver->getNumParticles());
    }

private:
    std::shared_ptr<SPHParameters<float>> m_SimParams;
    std::unique_ptr<SPHSolver> m_SPHSolver;
    std::unique_ptr<SceneManager> m_SceneManager;
    std::atomic<bool> m_bStop{true};
    float m_SimTime = 0;
    std::future<void> m_Future;
};

}  // namespace simplefluid
