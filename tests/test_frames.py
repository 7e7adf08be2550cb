"""Adaptive (CFL) sub-steps and whole frames on the device (a CUDA-graph
conditional while node per frame) against the oracle's frame loop."""
import numpy as np
import pytest

from helpers import params_16k
from simplefluid_gb300 import Simulator, SPHSolver, scene_positions, substeps_per_frame
from simplefluid_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def _start(prm, seed=1, scale=0.5):
    pos = scene_positions(prm, C.SF_SCENE_DAMBREAK_16K)
    vel = np.random.default_rng(seed).normal(scale=scale, size=pos.shape).astype(np.float32)
    return pos, vel


def test_adaptive_substeps_match_oracle(oracle):
    prm = params_16k(adaptiveTimeStep=True, timeStep=2e-3)
    pos, vel = _start(prm, scale=3.0)
    dts = []
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        for _ in range(30):
            dts.append(s.advanceFrame())
        s.step(30)
        gpos, gvel = s.getState()
    st = oracle.State(pos, vel)
    _, k, odts = st.frames(prm.to_c(), 1, frame_time=1.0, max_substeps=60, record_dts=60)
    assert k == 60
    assert np.array_equal(np.array(dts, np.float32).view(np.uint32), odts[:30].view(np.uint32))
    assert len(set(dts)) > 1 and max(dts) <= np.float32(2e-3) and min(dts) < np.float32(2e-3)  # it adapts
    st.sort(prm.to_c())
    opos, ovel = st.original_order()
    assert np.array_equal(gpos.view(np.uint32), opos.view(np.uint32))
    assert np.array_equal(gvel.view(np.uint32), ovel.view(np.uint32))


@pytest.mark.parametrize("adaptive", [False, True])
def test_frames_on_device_match_oracle(oracle, adaptive):
    prm = params_16k(adaptiveTimeStep=adaptive, timeStep=4e-4 if adaptive else 1e-4)
    pos, vel = _start(prm, seed=2)
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        t, k = s.advanceFrames(3)
        gpos, gvel = s.getState()
    st = oracle.State(pos, vel)
    ot, ok, _ = st.frames(prm.to_c(), 3)
    assert k == ok and t == ot
    if not adaptive:
        assert k == 3 * substeps_per_frame(1e-4)
    st.sort(prm.to_c())
    opos, ovel = st.original_order()
    assert np.array_equal(gpos.view(np.uint32), opos.view(np.uint32))
    assert np.array_equal(gvel.view(np.uint32), ovel.view(np.uint32))


def test_frame_respects_max_substeps():
    prm = params_16k()
    pos, vel = _start(prm)
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        t, k = s.advanceFrames(1, frame_time=1.0, max_substeps=7)
        assert k == 7 and t == pytest.approx(7e-4, rel=1e-6)
        t, k = s.advanceFrames(2, frame_time=1.0, max_substeps=3)
        assert k == 6


def test_simulator_frames_without_callbacks():
    """The headless Simulator advances whole frames on the device when no
    per-sub-step callback is set, and reaches stopTime like the reference loop."""
    prm = params_16k(stopTime=0.1)
    sim = Simulator(prm)
    frames = []
    sim.frameFinished = lambda: frames.append(1)
    sim.setupScene()
    sim.startSimulation()
    sim.wait()
    assert len(frames) == 3 and not sim.isRunning()
    assert float(sim.m_SimTime) >= 0.1


def test_adaptive_rejected_for_gradients_and_batches():
    from simplefluid_gb300 import SPHBatch
    prm = params_16k(adaptiveTimeStep=True)
    with SPHSolver(prm) as s:
        s.setParticles(np.zeros((8, 3), np.float32) + 0.5)
        with pytest.raises(C.SFError):
            s.forward(4, 2)
    with pytest.raises(C.SFError):
        SPHBatch([prm.to_c()])


def test_frame_loop_matches_the_reference_frame_loop():
    """On the adaptive 16,000-particle dambreak from rest, the device frame loop
    (one graph launch per frame) and the headless Simulator report the
    reference's own frame loop (Source/Simulator.cpp run on the same sub-step
    sizes, tests/golden/ref_frames.npz): sub-steps per 1/30 s frame and the float
    simulated time after each frame, bit for bit."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_frames.npz"))
    want_sub, want_t = g["adaptive16k_substeps"], g["adaptive16k_sim_times"]
    prm = params_16k(adaptiveTimeStep=True, timeStep=5e-3, stopTime=0.1)
    pos = scene_positions(prm, C.SF_SCENE_DAMBREAK_16K)
    subs, times = [], []
    with SPHSolver(prm) as s:
        s.setParticles(pos)
        sim_t = np.float32(0.0)
        while sim_t < np.float32(prm.stopTime):
            t, k = s.advanceFrames(1)
            sim_t = np.float32(sim_t + np.float32(t))
            subs.append(k)
            times.append(sim_t)
    assert np.array_equal(np.array(subs, np.uint32), want_sub)
    assert np.array_equal(np.array(times, np.float32).view(np.uint32), want_t.view(np.uint32))
    sim = Simulator(prm)
    reported = []
    sim.setupScene()
    sim.systemTimeChanged = lambda t: reported.append(np.float32(t))
    sim.startSimulation()
    sim.wait()
    assert np.array_equal(np.array(reported, np.float32).view(np.uint32), want_t.view(np.uint32))
