"""Seeded random configurations: the GPU path against the oracle, bit for bit.

Each case draws the whole parameter block from the valid ranges:
  * a non-cubic box;
  * the kernel and particle radii, stiffness, viscosity and restitution;
  * the EOS and the attractive-pressure flag;
  * the grid granularity K in {1, 2, 3};
  * a fixed or an adaptive sub-step.
It then builds a particle set from several parts:
  * a jittered lattice block;
  * a uniform cloud;
  * a dense cluster that overflows the neighbour lists;
  * particles on the box faces and corners, and some outside the box.
A few sub-steps run on both sides.  The caller-order positions and velocities
must match bit for bit, under every neighbour-list layout.  Batches of eight
such scenes (fixed time step, one grid granularity per batch, some with an
empty scene) run under the five-launch and the persistent batched step and
must match the oracle run on each scene alone.  The adjoint of each random
case (fixed time step) must match the oracle's FP32 adjoint, and whole
frames on the device must match the oracle's frame loop.
The generators themselves are checked on the CPU: every case passes
sf_params_update.
"""
import numpy as np
import pytest

from simplefluid_gb300 import SPHParameters, SPHSolver
from simplefluid_gb300 import _capi as C

CASES = 24
STEPS = 5


def make_case(seed: int):
    rng = np.random.default_rng(1000 + seed)
    lo = rng.uniform(-1.0, 0.2, size=3)
    ext = rng.uniform(0.4, 1.5, size=3)
    hi = lo + ext
    K = int(rng.integers(1, 4))
    h = float(rng.uniform(0.03, 0.1) * ext.min())
    h = max(h, float(K * ext.max() / 200.0))  # at most 200 cells per axis
    r = h / float(rng.uniform(2.5, 5.0))
    adaptive = bool(rng.integers(0, 2))
    prm = SPHParameters(
        particleRadius=r, kernelRadius=h, pressureStiffness=float(rng.uniform(10, 200)),
        viscosity=float(rng.choice([0.0, rng.uniform(0.001, 0.2)])),
        boundaryRestitution=float(rng.uniform(0, 1)), restDensity=float(rng.uniform(500, 1500)),
        timeStep=float(rng.uniform(2e-5, 2e-4)), boxMin=tuple(lo), boxMax=tuple(hi),
        eos=int(rng.integers(0, 2)), bUseAttractivePressure=bool(rng.integers(0, 2)), cellsPerH=K,
        adaptiveTimeStep=adaptive, gravity=(0.0, float(rng.uniform(-20, 0)), 0.0))
    parts = []
    # jittered lattice block at spacing 2r
    n_side = rng.integers(4, 14, size=3)
    corner = lo + rng.uniform(0.0, 0.5, size=3) * ext
    g = np.stack(np.meshgrid(*[np.arange(k) for k in n_side], indexing="ij"), -1).reshape(-1, 3)
    parts.append(corner + 2 * r * g + rng.uniform(-0.2, 0.2, size=g.shape) * 2 * r)
    # uniform cloud
    parts.append(rng.uniform(lo, hi, size=(int(rng.integers(0, 400)), 3)))
    # dense cluster (neighbour-list overflow)
    if rng.random() < 0.6:
        c = rng.uniform(lo + 0.2 * ext, hi - 0.2 * ext)
        parts.append(c + rng.normal(scale=0.15 * h, size=(int(rng.integers(70, 160)), 3)))
    # on faces and corners, and a few outside the box
    face = rng.uniform(lo, hi, size=(20, 3))
    axis = rng.integers(0, 3, size=20)
    side = rng.integers(0, 2, size=20)
    face[np.arange(20), axis] = np.where(side == 0, lo[axis], hi[axis])
    parts.append(face)
    parts.append(np.array([lo, hi, [lo[0], hi[1], lo[2]]]))
    parts.append(rng.uniform(lo - 0.1 * ext, hi + 0.1 * ext, size=(10, 3)))
    pos = np.concatenate(parts).astype(np.float32)
    vel = (rng.normal(size=pos.shape) * rng.uniform(0.0, 1.5)).astype(np.float32)
    return prm, pos, vel


@pytest.mark.parametrize("seed", range(CASES))
def test_generated_case_is_valid(seed, lib):
    import ctypes
    prm, pos, vel = make_case(seed)
    p = prm.to_c()
    assert lib.sf_params_update(ctypes.byref(p)) == C.SF_OK, C.load().sf_last_error()
    assert pos.shape == vel.shape and pos.shape[0] > 50


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(CASES))
def test_random_case_bit_identical(seed, oracle):
    prm, pos, vel = make_case(seed)
    st = oracle.State(pos, vel)
    st.step(prm.to_c(), STEPS)
    opos, ovel = st.original_order()
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        s.makeReady()
        s.step(STEPS)
        gpos, gvel = s.getState()
    assert np.array_equal(gpos.view(np.uint32), opos.view(np.uint32))
    assert np.array_equal(gvel.view(np.uint32), ovel.view(np.uint32))


def _with_list_mode(lib, s, mode):
    import ctypes
    t = C.sf_tuning()
    C.check(lib.sf_get_tuning(s.handle, ctypes.byref(t)))
    t.list_mode = mode
    C.check(lib.sf_set_tuning(s.handle, ctypes.byref(t)))


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(CASES))
def test_random_case_every_list_mode(seed, oracle, lib):
    """The same random cases with the other neighbour-list layouts (none,
    shared-memory staged, 16-bit warp tiles): every layout gives the
    oracle's bits."""
    prm, pos, vel = make_case(seed)
    st = oracle.State(pos, vel)
    st.step(prm.to_c(), STEPS)
    opos, ovel = st.original_order()
    for mode in (C.SF_LIST_NONE, C.SF_LIST_TILE_STAGED, C.SF_LIST_TILE16):
        with SPHSolver(prm) as s:
            s.setParticles(pos, vel)
            _with_list_mode(lib, s, mode)
            s.makeReady()
            s.step(STEPS)
            gpos, gvel = s.getState()
        assert np.array_equal(gpos.view(np.uint32), opos.view(np.uint32)), mode
        assert np.array_equal(gvel.view(np.uint32), ovel.view(np.uint32)), mode


def make_batch(index: int, K: int):
    """Eight random cases (fixed time step, all at grid granularity K) for one
    batch; every third batch has an empty scene."""
    params, poss, vels = [], [], []
    seed = 5000 + 100 * index
    while len(params) < 8:
        prm, pos, vel = make_case(seed)
        seed += 1
        if prm.cellsPerH < K:  # its grid was sized for a coarser K
            continue
        prm.adaptiveTimeStep = False
        prm.cellsPerH = K
        params.append(prm.to_c())
        poss.append(pos)
        vels.append(vel)
    if index % 3 == 0:
        poss[3], vels[3] = poss[3][:0], vels[3][:0]
    return params, poss, vels


@pytest.mark.gpu
@pytest.mark.parametrize("index", range(6))
def test_random_batch_every_step_form(index, oracle):
    """Batches of random scenes (their own boxes, radii, EOS and parameters)
    under the five-launch step with 32- and 16-bit lists and under the
    persistent cluster step: each scene gives the oracle's bits."""
    from simplefluid_gb300 import SPHBatch
    K = 2 if index % 2 == 0 else 1
    params, poss, vels = make_batch(index, K)
    counts = np.array([p.shape[0] for p in poss], np.uint32)
    pos = np.concatenate(poss).astype(np.float32)
    vel = np.concatenate(vels).astype(np.float32)
    refs = []
    for s in range(len(params)):
        if counts[s] == 0:
            refs.append((poss[s], vels[s]))
            continue
        st = oracle.State(poss[s], vels[s])
        st.step(params[s], STEPS)
        st.sort(params[s])
        refs.append(st.original_order())
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    tunings = [(C.SF_LIST_TILE, 128, 128, 2, 0, 0, 0), (C.SF_LIST_TILE16, 128, 128, 2, 0, 0, 0),
               (C.SF_LIST_TILE, 256, 128, 2, 0, 4, 256), (C.SF_LIST_TILE, 256, 128, 2, 0, 8, 1024),
               (C.SF_LIST_TILE, 256, 128, 2, 0, 2, 512)]
    for tune in tunings:
        with SPHBatch(params) as b:
            b.setState(counts, pos, vel)
            b.setTuning(C.sf_tuning(*tune))
            b.step(STEPS)
            gpos, gvel = b.getState()
        for s in range(len(params)):
            sl = slice(int(off[s]), int(off[s + 1]))
            assert np.array_equal(gpos[sl].view(np.uint32), refs[s][0].view(np.uint32)), (tune, s)
            assert np.array_equal(gvel[sl].view(np.uint32), refs[s][1].view(np.uint32)), (tune, s)


@pytest.mark.parametrize("index", range(6))
def test_random_batch_is_valid(index, lib):
    import ctypes
    K = 2 if index % 2 == 0 else 1
    params, poss, _ = make_batch(index, K)
    for p in params:
        assert p.cells_per_h == K and not p.adaptive_time_step
        assert lib.sf_params_update(ctypes.byref(p)) == C.SF_OK, C.load().sf_last_error()
    assert sum(x.shape[0] for x in poss) > 400


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(CASES))
def test_random_case_adjoint_matches_fp32_oracle(seed, oracle):
    """The adjoint (sf_forward + sf_adjoint) on the random cases, with a fixed
    time step, from a seeded final-state adjoint of positions and velocities:
    the GPU gradients of the initial state equal the FP32 oracle adjoint's bit
    for bit, and the viscosity and stiffness gradients agree to the rounding
    of their reductions."""
    prm, pos, vel = make_case(seed)
    prm.adaptiveTimeStep = False
    rng = np.random.default_rng(77 + seed)
    steps, ckpt = 6, 3
    sx = rng.normal(size=pos.shape).astype(np.float32)
    sv = rng.normal(size=pos.shape).astype(np.float32)
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        s.forward(steps, ckpt)
        pf = s.getState()[0]
        dx0, dv0, dmu, dk = s.adjoint(sx, sv)
    ox, ov, om, ok, opf = oracle.adjoint(prm.to_c(), pos, vel, steps, sx, sv, ckpt=ckpt, dtype=np.float32)
    assert np.array_equal(pf.view(np.uint32), opf.view(np.uint32))
    assert np.array_equal(dx0.view(np.uint32), ox.view(np.uint32))
    assert np.array_equal(dv0.view(np.uint32), ov.view(np.uint32))
    assert dmu == pytest.approx(om, rel=1e-5, abs=1e-30)
    assert dk == pytest.approx(ok, rel=1e-5, abs=1e-30)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(0, CASES, 2))
def test_random_case_frames_on_device(seed, oracle):
    """Whole frames on the device (the conditional-graph frame loop) on the
    random cases: sub-step count, simulated time and state equal the oracle's
    frame loop.  Frames of 1.5 ms hold a few to a few dozen sub-steps of the
    cases' fixed or adaptive step."""
    prm, pos, vel = make_case(seed)
    frame_time, frames, cap = 1.5e-3, 2, 200
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        t, k = s.advanceFrames(frames, frame_time, cap)
        gpos, gvel = s.getState()
    st = oracle.State(pos, vel)
    ot, ok, _ = st.frames(prm.to_c(), frames, frame_time=frame_time, max_substeps=cap)
    assert k == ok and t == ot and k >= frames
    st.sort(prm.to_c())
    opos, ovel = st.original_order()
    assert np.array_equal(gpos.view(np.uint32), opos.view(np.uint32))
    assert np.array_equal(gvel.view(np.uint32), ovel.view(np.uint32))
