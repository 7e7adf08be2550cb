"""Batches of independent scenes: the workload generator (CPU) and the batched
step (GPU) against the oracle and against per-scene contexts."""
import numpy as np
import pytest

from helpers import params_16k
from simplefluid_gb300 import SPHBatch, SPHParameters, SPHSolver, batch_cubes
from simplefluid_gb300 import _capi as C


def small_base(**kw):
    base = dict(particleRadius=0.01, kernelRadius=0.04)
    base.update(kw)
    return SPHParameters(**base)


def test_batch_cubes_workload_definition():
    params, counts, pos = batch_cubes(20171, 256, small_base())
    assert len(params) == 256 and counts.size == 256
    assert counts.min() >= 2000 and counts.max() <= 65536
    assert pos.shape[0] == int(counts.sum())
    assert 3.5e6 < counts.sum() < 6.5e6  # log-uniform mean ~ 18.2k per scene
    mus = np.array([p.viscosity for p in params])
    ks = np.array([p.pressure_stiffness for p in params])
    assert mus.min() >= 0.005 and mus.max() <= 0.05 and ks.min() >= 20 and ks.max() <= 100
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    for s in (0, 17, 255):
        blk = pos[off[s]:off[s + 1]]
        hi = params[s].box_max[0]
        assert np.all(blk > 0) and np.all(blk < hi)
    p2, c2, pos2 = batch_cubes(20171, 256, small_base())
    assert np.array_equal(c2, counts) and np.array_equal(pos2.view(np.uint32), pos.view(np.uint32))
    _, c3, _ = batch_cubes(7, 256, small_base())
    assert not np.array_equal(c3, counts)


def _scene_slices(counts):
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    return [slice(int(off[s]), int(off[s + 1])) for s in range(len(counts))]


@pytest.mark.gpu
@pytest.mark.parametrize("K", [1, 2])
def test_batch_matches_oracle_per_scene(oracle, K):
    params, counts, pos = batch_cubes(5, 6, small_base(cellsPerH=K))
    rng = np.random.default_rng(5)
    vel = rng.normal(scale=0.1, size=pos.shape).astype(np.float32)
    with SPHBatch(params) as b:
        b.setState(counts, pos, vel)
        b.step(15)
        gpos, gvel = b.getState()
        for s in range(len(params)):
            assert b.getParams(s).cells_per_h == K
    for s, sl in enumerate(_scene_slices(counts)):
        st = oracle.State(pos[sl], vel[sl])
        st.step(params[s], 15)
        st.sort(params[s])
        opos, ovel = st.original_order()
        assert np.array_equal(gpos[sl].view(np.uint32), opos.view(np.uint32)), s
        assert np.array_equal(gvel[sl].view(np.uint32), ovel.view(np.uint32)), s


@pytest.mark.gpu
def test_batch_equals_per_scene_contexts():
    params, counts, pos = batch_cubes(11, 5, small_base())
    with SPHBatch(params) as b:
        b.setState(counts, pos)
        b.step(25)
        gpos, _ = b.getState()
    for s, sl in enumerate(_scene_slices(counts)):
        with SPHSolver(SPHParameters.from_c(params[s])) as ctx:
            ctx.setParticles(pos[sl])
            ctx.step(25)
            spos = ctx.getParticles()
        assert np.array_equal(gpos[sl].view(np.uint32), spos.view(np.uint32)), s


@pytest.mark.gpu
def test_batch_autotune_restores_state_and_choice_is_valid(oracle):
    params, counts, pos = batch_cubes(3, 4, small_base())
    with SPHBatch(params) as b:
        b.setState(counts, pos)
        b.step(3)
        before = b.getState()
        t, K, ms = b.autotune(trial_steps=3)
        after = b.getState()
        assert K in (1, 2) and ms > 0
        assert t.list_mode in (C.SF_LIST_TILE_STAGED, C.SF_LIST_TILE, C.SF_LIST_TILE16) and t.prefetch == 2
        assert t.batch_cluster in (0, 4, 8)
        assert np.array_equal(before[0].view(np.uint32), after[0].view(np.uint32))
        got = b.getTuning()
        assert bytes(got) == bytes(t)
        b.step(5)
        gpos, _ = b.getState()
    # the chosen configuration still matches the oracle (with the chosen K)
    for s, sl in enumerate(_scene_slices(counts)):
        p = params[s]
        p.cells_per_h = K
        st = oracle.State(before[0][sl], before[1][sl])
        st.step(p, 5)
        st.sort(p)
        opos, _ = st.original_order()
        assert np.array_equal(gpos[sl].view(np.uint32), opos.view(np.uint32)), s


@pytest.mark.gpu
def test_batch_rejects_mixed_grids():
    a = small_base(cellsPerH=1).to_c()
    b = small_base(cellsPerH=2).to_c()
    with pytest.raises(C.SFError):
        SPHBatch([a, b])
    with pytest.raises(C.SFError):
        SPHBatch([small_base(cellsPerH=3).to_c()])


@pytest.mark.gpu
def test_batched_cubes_workload_500_steps(oracle):
    """The batched-cube workload as configured (256 scenes, counts log-uniform
    in [2000, 65536], 500 sub-steps): after the 500 sub-steps every sampled
    scene (every 16th, the smallest and the largest) equals the oracle run on
    that scene alone, bit for bit, and the whole batch passes the state checks."""
    from simplefluid_gb300 import configs
    cfg = configs.load("batched_cubes")
    assert cfg["scenes"] == 256 and cfg["steps"] == 500
    params, counts, pos = batch_cubes(cfg["seed"], cfg["scenes"], configs.params(cfg))
    with SPHBatch(params) as b:
        b.setState(counts, pos)
        b.step(cfg["steps"])
        gpos, gvel = b.getState()
        rep = b.checkState()
    assert all(rep[k] == 0 for k in ("non_finite", "outside_box", "unsorted", "cell_table_mismatch", "bad_ids"))
    slices = _scene_slices(counts)
    sample = sorted(set(range(0, len(params), 16)) | {int(np.argmin(counts)), int(np.argmax(counts))})
    for s in sample:
        sl = slices[s]
        st = oracle.State(pos[sl])
        st.step(params[s], cfg["steps"])
        st.sort(params[s])
        opos, ovel = st.original_order()
        assert np.array_equal(gpos[sl].view(np.uint32), opos.view(np.uint32)), s
        assert np.array_equal(gvel[sl].view(np.uint32), ovel.view(np.uint32)), s


@pytest.mark.gpu
@pytest.mark.parametrize("K,cluster,block", [(1, 2, 256), (2, 2, 512), (2, 4, 1024), (2, 8, 256), (1, 8, 1024)])
def test_persistent_batch_step_matches_oracle_and_five_launch_step(oracle, K, cluster, block):
    """The persistent batched step (one launch of thread-block clusters that
    take whole scenes, largest first) computes the bits of the five-launch
    step and of the oracle run on each scene alone; scenes of one and of zero
    particles included."""
    params, counts, pos = batch_cubes(9, 7, small_base(cellsPerH=K))
    # shrink two scenes to one particle and to none (positions of the others kept)
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    keep = np.ones(pos.shape[0], bool)
    keep[off[2] + 1:off[3]] = False
    keep[off[4]:off[5]] = False
    counts = counts.copy()
    counts[2], counts[4] = 1, 0
    pos = pos[keep]
    rng = np.random.default_rng(9)
    vel = rng.normal(scale=0.1, size=pos.shape).astype(np.float32)
    out = {}
    for c in (0, cluster):
        with SPHBatch(params) as b:
            b.setTuning(C.sf_tuning(C.SF_LIST_TILE, 256, 128, 2, 0, c, block if c else 0))
            b.setState(counts, pos, vel)
            b.step(12)
            out[c] = b.getState()
            assert b.getTuning().batch_cluster == c
            rep = b.checkState()
            assert all(rep[k] == 0 for k in ("non_finite", "outside_box", "unsorted", "cell_table_mismatch", "bad_ids"))
    for a, bb in zip(out[0], out[cluster]):
        assert np.array_equal(a.view(np.uint32), bb.view(np.uint32))
    gpos, gvel = out[cluster]
    for s, sl in enumerate(_scene_slices(counts)):
        if counts[s] == 0:
            continue
        st = oracle.State(pos[sl], vel[sl])
        st.step(params[s], 12)
        st.sort(params[s])
        opos, ovel = st.original_order()
        assert np.array_equal(gpos[sl].view(np.uint32), opos.view(np.uint32)), s
        assert np.array_equal(gvel[sl].view(np.uint32), ovel.view(np.uint32)), s


@pytest.mark.gpu
def test_persistent_batch_workload_500_steps(oracle):
    """The batched-cube workload's 500 sub-steps with the persistent step
    (clusters of 8 blocks of 1024 threads): sampled scenes equal the oracle."""
    from simplefluid_gb300 import configs
    cfg = configs.load("batched_cubes")
    params, counts, pos = batch_cubes(cfg["seed"], cfg["scenes"], configs.params(cfg))
    with SPHBatch(params) as b:
        b.setTuning(C.sf_tuning(C.SF_LIST_TILE, 256, 128, 2, 0, 8, 1024))
        b.setState(counts, pos)
        b.step(cfg["steps"])
        gpos, gvel = b.getState()
    slices = _scene_slices(counts)
    for s in (int(np.argmax(counts)), int(np.argmin(counts)), 100):
        sl = slices[s]
        st = oracle.State(pos[sl])
        st.step(params[s], cfg["steps"])
        st.sort(params[s])
        opos, ovel = st.original_order()
        assert np.array_equal(gpos[sl].view(np.uint32), opos.view(np.uint32)), s
        assert np.array_equal(gvel[sl].view(np.uint32), ovel.view(np.uint32)), s


@pytest.mark.gpu
def test_persistent_batch_step_rejections():
    import ctypes
    params, counts, pos = batch_cubes(3, 3, small_base())
    with SPHBatch(params) as b:
        for bad in (C.sf_tuning(C.SF_LIST_TILE, 256, 128, 2, 0, 3), C.sf_tuning(C.SF_LIST_TILE16, 256, 128, 2, 0, 4),
                    C.sf_tuning(C.SF_LIST_TILE, 256, 128, 2, 0, 4, 384)):
            with pytest.raises(C.SFError):
                b.setTuning(bad)
    with SPHSolver(SPHParameters.from_c(params[0])) as s:
        lib = C.load()
        assert lib.sf_set_tuning(s.handle, ctypes.byref(C.sf_tuning(C.SF_LIST_TILE, 256, 128, 2, 0, 4))) == \
            C.SF_ERR_INVALID_ARGUMENT
