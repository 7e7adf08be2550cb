"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Bars (fixed by the workload definition):
  * cell keys, sorted order, cell tables and neighbour sets: bit-exact;
  * single-pass density: within 1e-5 relative per particle (FP32);
  * single-pass acceleration: within 1e-5 of the field's max magnitude (FP32);
  * mass (particle count, identity of every particle) conserved exactly;
  * trajectories: kinetic energy and mean density error over 500 steps within
    a 1e-3 relative band of the oracle.
"""
import numpy as np
import pytest

from helpers import normwise_err, params_16k, params_1m, params_reference_box, rel_err
from simplefluid_gb300 import SPHSolver, scene_positions
from simplefluid_gb300 import _capi as C

pytestmark = pytest.mark.gpu

DENSITY_RTOL = 1e-5
ACCEL_NORMWISE = 1e-5
TRAJ_BAND = 1e-3


def solver_with(prm, pos, vel=None):
    s = SPHSolver(prm)
    s.setParticles(pos, vel)
    return s


def jittered_block(n_side=(16, 24, 16), spacing=0.02, seed=3, origin=0.05):
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(k) for k in n_side], indexing="ij"), -1).reshape(-1, 3)
    pos = origin + g * spacing + rng.uniform(-0.2, 0.2, size=g.shape) * spacing
    return pos.astype(np.float32)


def test_sort_and_cell_table_bit_exact(oracle):
    prm = params_16k()
    pos = scene_positions(prm, C.SF_SCENE_DAMBREAK_16K)
    rng = np.random.default_rng(0)
    pos = (pos + rng.uniform(-0.004, 0.004, size=pos.shape)).astype(np.float32)
    with solver_with(prm, pos) as s:
        gpos, _, gids, gkeys = s.sortedState()
        gcs = s.cellStart()
    st = oracle.State(pos)
    keys, cs = st.sort(prm.to_c(), want_cells=True)
    assert np.array_equal(gids, st.ids)
    assert np.array_equal(gkeys, keys)
    assert np.array_equal(gcs, cs)
    assert np.array_equal(gpos.view(np.uint32), st.pos.view(np.uint32))


def test_neighbour_sets_bit_exact(oracle):
    prm = params_16k()
    pos = jittered_block()
    with solver_with(prm, pos) as s:
        gcnt, ghash = s.neighbourStats()
    st = oracle.State(pos)
    st.sort(prm.to_c())
    cnt, hsh = st.neighbour_stats(prm.to_c())
    assert np.array_equal(gcnt, cnt)
    assert np.array_equal(ghash, hsh)
    assert cnt.mean() > 20


@pytest.mark.parametrize("eos,attr", [(C.SF_EOS_LINEAR, False), (C.SF_EOS_LINEAR, True), (C.SF_EOS_TAIT, False)])
def test_density_and_pressure(oracle, eos, attr):
    prm = params_16k(eos=eos, bUseAttractivePressure=attr)
    pos = jittered_block()
    with solver_with(prm, pos) as s:
        grho, gp = s.computeDensity()
    st = oracle.State(pos)
    st.sort(prm.to_c())
    rho, prs, _ = st.density(prm.to_c())
    assert rel_err(grho, rho) < DENSITY_RTOL
    assert normwise_err(gp, prs) < DENSITY_RTOL
    if not attr:
        assert np.all(gp >= 0)
    else:
        assert np.any(gp < 0)


def test_density_op_for_op_equal(oracle):
    """The kernel performs the oracle's operations in the oracle's order, so the
    density is not just within tolerance but bit-identical."""
    prm = params_16k()
    pos = jittered_block(seed=11)
    with solver_with(prm, pos) as s:
        grho, _ = s.computeDensity()
    st = oracle.State(pos)
    st.sort(prm.to_c())
    rho, _, _ = st.density(prm.to_c())
    assert np.array_equal(grho.view(np.uint32), rho.view(np.uint32))


def test_acceleration(oracle):
    prm = params_16k()
    pos = jittered_block(seed=5)
    vel = np.random.default_rng(5).normal(scale=0.3, size=pos.shape).astype(np.float32)
    with solver_with(prm, pos, vel) as s:
        gacc = s.computeAccel()
    st = oracle.State(pos, vel)
    st.sort(prm.to_c())
    acc = st.accel(prm.to_c())
    assert normwise_err(gacc, acc) < ACCEL_NORMWISE


def test_one_step_state(oracle):
    prm = params_16k()
    pos = jittered_block(seed=9)
    with solver_with(prm, pos) as s:
        dt = s.advanceFrame()
        gpos, gvel = s.getState()
    assert dt == np.float32(1e-4)
    st = oracle.State(pos)
    st.step(prm.to_c(), 1)
    opos, ovel = st.original_order()
    assert np.max(np.abs(gpos - opos)) <= 1e-6
    assert normwise_err(gvel, ovel) < 1e-5


def _ke_and_density_error(pos, vel, prm, oracle):
    ke = 0.5 * float(np.sum(vel.astype(np.float64) ** 2))
    st = oracle.State(pos, vel)
    st.sort(prm.to_c())
    rho, _, _ = st.density(prm.to_c())
    return ke, float(np.mean(np.abs(rho - prm.restDensity)) / prm.restDensity)


def test_trajectory_500_steps_16k(oracle):
    """500 steps of the 16,000-particle dambreak: kinetic energy and mean density
    error track the oracle within the stated band; mass is conserved exactly."""
    prm = params_16k()
    pos = scene_positions(prm, C.SF_SCENE_DAMBREAK_16K)
    st = oracle.State(pos)
    with solver_with(prm, pos) as s:
        for chunk in range(5):
            s.step(100)
            st.step(prm.to_c(), 100)
            gpos, gvel = s.getState()
            opos, ovel = st.original_order()
            gke, gde = _ke_and_density_error(gpos, gvel, prm, oracle)
            oke, ode = _ke_and_density_error(opos, ovel, prm, oracle)
            assert abs(gke - oke) <= TRAJ_BAND * max(oke, 1e-12), (chunk, gke, oke)
            assert abs(gde - ode) <= TRAJ_BAND * max(ode, 1e-12) + 1e-7, (chunk, gde, ode)
        _, _, ids, keys = s.sortedState()
        assert s.getNumParticles() == 16000
        assert np.array_equal(np.sort(ids), np.arange(16000, dtype=np.uint32))
        assert np.all(np.diff(keys.astype(np.int64)) >= 0)
        lo = np.float32(0.01)
        assert np.all(gpos >= lo) and np.all(gpos <= np.float32(0.99))
        assert np.isfinite(gpos).all() and np.isfinite(gvel).all()


def test_trajectory_bit_identical_200_steps(oracle):
    """Every kernel performs the oracle's floating-point operations in the
    oracle's order (explicit fmaf, IEEE sqrt and division, canonical neighbour
    order), so 200 sub-steps of the 16k dambreak agree bit for bit."""
    prm = params_16k()
    pos = scene_positions(prm, C.SF_SCENE_DAMBREAK_16K)
    with solver_with(prm, pos) as s:
        s.step(200)
        gpos, gvel = s.getState()
        _, _, ids, _ = s.sortedState()
    st = oracle.State(pos)
    st.step(prm.to_c(), 200)
    st.sort(prm.to_c())  # the solver leaves its state sorted after each step
    opos, ovel = st.original_order()
    assert np.array_equal(ids, st.ids)
    assert np.array_equal(gpos.view(np.uint32), opos.view(np.uint32))
    assert np.array_equal(gvel.view(np.uint32), ovel.view(np.uint32))


@pytest.mark.parametrize("scene", [C.SF_SCENE_SPHERE_DROP, C.SF_SCENE_CUBE_DROP, C.SF_SCENE_DAMBREAK,
                                   C.SF_SCENE_DOUBLE_DAMBREAK])
def test_reference_scenes_20_steps(oracle, scene):
    """The reference's four scenes in its [-1,1]^3 box at GUI resolution 24."""
    prm = params_reference_box(resolution=24, scene=scene)
    pos = scene_positions(prm, scene)
    with solver_with(prm, pos) as s:
        s.step(20)
        gpos, gvel = s.getState()
    st = oracle.State(pos)
    st.step(prm.to_c(), 20)
    opos, ovel = st.original_order()
    assert np.max(np.abs(gpos - opos)) <= 1e-5
    assert normwise_err(gvel, ovel) < 1e-4


def test_set_get_roundtrip_bits():
    prm = params_16k()
    pos = jittered_block(seed=2)
    vel = np.random.default_rng(2).normal(size=pos.shape).astype(np.float32)
    with solver_with(prm, pos, vel) as s:
        gpos, gvel = s.getState()
        assert s.getNumParticles() == pos.shape[0]
    assert np.array_equal(gpos.view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(gvel.view(np.uint32), vel.view(np.uint32))


def test_deterministic_repeat():
    prm = params_16k()
    pos = scene_positions(prm, C.SF_SCENE_DAMBREAK_16K)
    outs = []
    for _ in range(2):
        with solver_with(prm, pos) as s:
            s.step(50)
            outs.append(s.getState()[0])
    assert np.array_equal(outs[0].view(np.uint32), outs[1].view(np.uint32))


def test_edge_single_particle(oracle):
    prm = params_16k()
    pos = np.array([[0.5, 0.5, 0.5]], np.float32)
    with solver_with(prm, pos) as s:
        rho, _ = s.computeDensity()
        s.step(10)
        gpos, gvel = s.getState()
    st = oracle.State(pos)
    st.step(prm.to_c(), 10)
    assert rho[0] > 0
    assert np.array_equal(gpos.view(np.uint32), st.pos.view(np.uint32))


def test_edge_dense_cluster_one_cell(oracle):
    """Hundreds of particles in one cell (and coincident pairs): the per-cell
    ranking and the r = 0 pressure guard."""
    prm = params_16k()
    rng = np.random.default_rng(4)
    pos = (0.5 + rng.uniform(0, 0.03, size=(600, 3))).astype(np.float32)
    pos[300:310] = pos[0]
    with solver_with(prm, pos) as s:
        _, _, ids, keys = s.sortedState()
        s.step(3)
        gpos, gvel = s.getState()
    st = oracle.State(pos)
    okeys, _ = st.sort(prm.to_c())
    assert np.array_equal(ids, st.ids) and np.array_equal(keys, okeys)
    st2 = oracle.State(pos)
    st2.step(prm.to_c(), 3)
    opos, ovel = st2.original_order()
    assert np.isfinite(gpos).all()
    assert normwise_err(gpos, opos) < 1e-5


def test_edge_coincident_pairs_on_the_list_path(oracle):
    """Coincident distinct particles (r = 0, j != i) with short neighbour lists:
    the force pass's list path takes no pressure term for them, like the
    oracle, and the trajectory stays bit-identical."""
    prm = params_16k()
    pos = jittered_block(n_side=(10, 12, 10), seed=21)
    pos[[5, 117, 640, 999]] = pos[[6, 118, 641, 1000]]
    vel = np.random.default_rng(22).normal(scale=0.05, size=pos.shape).astype(np.float32)
    vel[[5, 117, 640, 999]] = vel[[6, 118, 641, 1000]]
    with solver_with(prm, pos, vel) as s:
        s.step(30)
        gpos, gvel = s.getState()
        rep = s.checkState()
    assert rep["list_overflow"] == 0 and rep["non_finite"] == 0  # the lists were read, not rescanned
    st = oracle.State(pos, vel)
    st.step(prm.to_c(), 30)
    st.sort(prm.to_c())
    opos, ovel = st.original_order()
    assert np.array_equal(gpos.view(np.uint32), opos.view(np.uint32))
    assert np.array_equal(gvel.view(np.uint32), ovel.view(np.uint32))
    assert np.array_equal(gpos[5], gpos[6]) and np.array_equal(gpos[999], gpos[1000])


def test_edge_particles_outside_box(oracle):
    """Particles given outside the box are binned into the edge cells and
    clamped back by the first step."""
    prm = params_16k()
    pos = jittered_block(n_side=(6, 6, 6))
    pos[:10] -= 0.5
    pos[10:20] += 2.0
    with solver_with(prm, pos) as s:
        s.step(1)
        gpos, _ = s.getState()
    st = oracle.State(pos)
    st.step(prm.to_c(), 1)
    opos, _ = st.original_order()
    assert np.all(gpos >= np.float32(0.01)) and np.all(gpos <= np.float32(0.99))
    assert np.max(np.abs(gpos - opos)) <= 1e-6


def test_errors_through_the_abi(lib):
    import ctypes
    prm = params_16k()
    s = SPHSolver(prm)
    with pytest.raises(C.SFError) as e:
        s.advanceFrame()
    assert e.value.status == C.SF_ERR_NOT_READY
    s.setParticles(jittered_block(n_side=(4, 4, 4)))
    out = np.zeros((3, 3), np.float32)
    st = lib.sf_get_state(s.handle, out.ctypes.data_as(ctypes.c_void_p), None, 3)
    assert st == C.SF_ERR_INVALID_ARGUMENT
    s.setParticles(np.zeros((0, 3), np.float32))
    assert s.getNumParticles() == 0
    with pytest.raises(C.SFError):
        s.makeReady()
    s.close()


def test_set_params_regrids(oracle):
    """Changing kernelRadius re-buckets the particles on the new grid."""
    prm = params_16k()
    pos = jittered_block(seed=6)
    with solver_with(prm, pos) as s:
        prm2 = params_16k(kernelRadius=0.05)
        s.setParams(prm2)
        d = oracle.derive(prm2.to_c())
        assert s.gridDims() == (int(d["nx"]), int(d["ny"]), int(d["nz"])) == (39, 39, 39)
        gcnt, ghash = s.neighbourStats()
        _, _, gids, _ = s.sortedState()
    # the solver re-sorts its current (old-grid) order stably on the new grid
    st = oracle.State(pos)
    st.sort(prm.to_c())
    st.sort(prm2.to_c())
    assert np.array_equal(gids, st.ids)
    cnt, hsh = st.neighbour_stats(prm2.to_c())
    assert np.array_equal(gcnt, cnt) and np.array_equal(ghash, hsh)


def test_full_size_1m_double_dambreak(oracle):
    """The 1,048,576-particle double dambreak: sort/cell table bit-exact and
    density within tolerance at full size; after 20 steps the size-independent
    properties hold (sorted keys, permutation of ids, cell table consistent
    with the keys, particles inside the box, finite state)."""
    prm = params_1m()
    pos = scene_positions(prm, C.SF_SCENE_DOUBLE_DAMBREAK_1M)
    n = pos.shape[0]
    assert n == 1048576
    st = oracle.State(pos)
    okeys, ocs = st.sort(prm.to_c(), want_cells=True)
    orho, _, _ = st.density(prm.to_c())
    with solver_with(prm, pos) as s:
        _, _, ids, keys = s.sortedState()
        assert np.array_equal(ids, st.ids) and np.array_equal(keys, okeys)
        assert np.array_equal(s.cellStart(), ocs)
        grho, _ = s.computeDensity()
        assert rel_err(grho, orho) < DENSITY_RTOL
        s.step(20)
        _, _, ids, keys = s.sortedState()
        cs = s.cellStart()
        gpos, gvel = s.getState()
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)
    assert np.array_equal(np.sort(ids), np.arange(n, dtype=np.uint32))
    counts = np.bincount(keys, minlength=cs.size - 1)
    assert cs[0] == 0 and cs[-1] == n and np.array_equal(np.diff(cs.astype(np.int64)), counts)
    assert np.isfinite(gpos).all() and np.isfinite(gvel).all()
    assert np.all(gpos >= np.float32(0.0025)) and np.all(gpos <= np.float32(0.9975))


def _assert_same_state_bits(s, st, what):
    """The solver's state equals the oracle's bit for bit, in the same sorted
    order (the solver re-sorts after every sub-step; the oracle is re-sorted
    here the same way)."""
    gpos, gvel = s.getState()
    _, _, gids, _ = s.sortedState()
    opos, ovel = st.original_order()
    assert np.array_equal(gids, st.ids), what
    assert np.array_equal(gpos.view(np.uint32), opos.view(np.uint32)), what
    assert np.array_equal(gvel.view(np.uint32), ovel.view(np.uint32)), what
    return gpos, gvel


def test_1m_double_dambreak_1000_steps_bit_identical(oracle):
    """The 1,048,576-particle double dambreak over its 1,000 sub-steps: after
    every 100 sub-steps the sorted order, positions and velocities equal the
    oracle's bit for bit, and kinetic energy and mean density error are
    inside the stated band of the oracle's (the band is implied by the bit
    equality; it is computed so that a tolerance failure names its size)."""
    prm = params_1m()
    pos = scene_positions(prm, C.SF_SCENE_DOUBLE_DAMBREAK_1M)
    assert pos.shape[0] == 1048576
    st = oracle.State(pos)
    cp = prm.to_c()
    with solver_with(prm, pos) as s:
        for chunk in range(10):
            s.step(100)
            st.step(cp, 100)
            st.sort(cp)
            gpos, gvel = _assert_same_state_bits(s, st, f"after {100 * (chunk + 1)} sub-steps")
            opos, ovel = st.original_order()
            gke, gde = _ke_and_density_error(gpos, gvel, prm, oracle)
            oke, ode = _ke_and_density_error(opos, ovel, prm, oracle)
            assert abs(gke - oke) <= TRAJ_BAND * max(oke, 1e-12), (chunk, gke, oke)
            assert abs(gde - ode) <= TRAJ_BAND * max(ode, 1e-12) + 1e-7, (chunk, gde, ode)
        assert oke > 0 and ode > 0  # the fluid moves and compresses
        rep = s.checkState()
        assert all(rep[k] == 0 for k in ("non_finite", "outside_box", "unsorted", "cell_table_mismatch", "bad_ids"))


def test_sphere_pool_50_steps_bit_identical(oracle):
    """Sphere drop into a pool (~3.35M particles) over 50 sub-steps: the state
    equals the oracle's bit for bit after 10 and after 50 sub-steps."""
    prm = params_1m(particleRadius=0.00227, kernelRadius=0.00908, scene=C.SF_SCENE_SPHERE_POOL)
    pos = scene_positions(prm, C.SF_SCENE_SPHERE_POOL)
    st = oracle.State(pos)
    cp = prm.to_c()
    with solver_with(prm, pos) as s:
        for chunk in (10, 40):
            s.step(chunk)
            st.step(cp, chunk)
            st.sort(cp)
            _assert_same_state_bits(s, st, f"after {chunk} more sub-steps")


def _tuned_run(prm, pos, tune, steps):
    import ctypes
    lib = C.load()
    with solver_with(prm, pos) as s:
        C.check(lib.sf_set_tuning(s.handle, ctypes.byref(tune)))
        got = C.sf_tuning()
        C.check(lib.sf_get_tuning(s.handle, ctypes.byref(got)))
        assert bytes(got) == bytes(tune)
        s.step(steps)
        return s.getState()


def test_tuning_variants_are_bit_identical(oracle):
    """Every kernel choice (neighbour-list layout, block sizes, gather batch)
    computes the same bits; a dense cluster forces the list-overflow path."""
    prm = params_16k()
    pos = jittered_block(n_side=(16, 20, 16), seed=12)
    rng = np.random.default_rng(12)
    cluster = (0.7 + rng.uniform(0, 0.03, size=(200, 3))).astype(np.float32)
    pos = np.concatenate([pos, cluster])
    st = oracle.State(pos)
    st.step(prm.to_c(), 8)
    st.sort(prm.to_c())
    ref_pos, ref_vel = st.original_order()
    combos = [(m, db, fb, pf, w) for m in (0, 1, 2, 3) for db in (128, 256) for fb in (128, 256) for pf in (2, 4)
              for w in (0, 1)
              if not (m == 0 and pf != 2) and not (m == 1 and db != 128) and not (w == 1 and (db, fb) != (256, 128))]
    for m, db, fb, pf, w in combos:
        t = C.sf_tuning(m, db, fb, pf, w)
        gpos, gvel = _tuned_run(prm, pos, t, 8)
        assert np.array_equal(gpos.view(np.uint32), ref_pos.view(np.uint32)), (m, db, fb, pf, w)
        assert np.array_equal(gvel.view(np.uint32), ref_vel.view(np.uint32)), (m, db, fb, pf, w)


def test_sixteen_bit_lists_with_wide_tiles(oracle):
    """SF_LIST_TILE16 on a scene whose candidate spans exceed 32767 sorted
    places in most warp tiles (a 160 x 120 x 100 lattice: one z-layer of cells
    holds 19,200 particles, so an inner particle's candidates reach ~38,000
    places back) but not near the lowest and highest layers: the wide tiles
    store 32-bit entries, the others 16-bit entries, and the state after 5
    steps equals the oracle's bit for bit."""
    r = 0.0025
    prm = params_16k(particleRadius=r, kernelRadius=4 * r)
    rng = np.random.default_rng(31)
    g = np.stack(np.meshgrid(np.arange(160), np.arange(120), np.arange(100), indexing="ij"), -1).reshape(-1, 3)
    pos = (0.05 + 2 * r * g + rng.uniform(-0.1, 0.1, size=g.shape) * 2 * r).astype(np.float32)
    gpos, gvel = _tuned_run(prm, pos, C.sf_tuning(C.SF_LIST_TILE16, 256, 128, 2), 5)
    st = oracle.State(pos)
    st.step(prm.to_c(), 5)
    st.sort(prm.to_c())
    opos, ovel = st.original_order()
    assert np.array_equal(gpos.view(np.uint32), opos.view(np.uint32))
    assert np.array_equal(gvel.view(np.uint32), ovel.view(np.uint32))


def test_tuning_rejects_bad_values(lib):
    import ctypes
    s = SPHSolver(params_16k())
    for bad in (C.sf_tuning(7, 128, 128, 2), C.sf_tuning(1, 64, 128, 2), C.sf_tuning(1, 128, 128, 3),
                C.sf_tuning(3, 128, 128, 2, 2), C.sf_tuning(2, 128, 128, 2, 0, 4)):
        assert lib.sf_set_tuning(s.handle, ctypes.byref(bad)) == C.SF_ERR_INVALID_ARGUMENT
    s.close()


def test_full_size_sphere_pool(oracle):
    """Sphere drop into a pool: a jittered pool of depth 0.3 over the unit
    footprint plus a jittered sphere of radius 0.15 at one particle spacing
    (r = 0.00227, h = 4r).  At one spacing the geometry holds ~3.35M
    particles (the pool ~3.19M, the sphere ~0.15M), the count recorded here.
    Sort, cell table and density are checked against the oracle at full size;
    after 10 steps the size-independent properties hold."""
    prm = params_1m(particleRadius=0.00227, kernelRadius=0.00908, scene=C.SF_SCENE_SPHERE_POOL)
    pos = scene_positions(prm, C.SF_SCENE_SPHERE_POOL)
    n = pos.shape[0]
    assert 3_300_000 < n < 3_400_000
    st = oracle.State(pos)
    okeys, ocs = st.sort(prm.to_c(), want_cells=True)
    orho, _, _ = st.density(prm.to_c())
    with solver_with(prm, pos) as s:
        _, _, ids, keys = s.sortedState()
        assert np.array_equal(ids, st.ids) and np.array_equal(keys, okeys)
        assert np.array_equal(s.cellStart(), ocs)
        grho, _ = s.computeDensity()
        assert np.array_equal(grho.view(np.uint32), orho.view(np.uint32))
        s.step(10)
        _, _, ids, keys = s.sortedState()
        gpos, gvel = s.getState()
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)
    assert np.array_equal(np.sort(ids), np.arange(n, dtype=np.uint32))
    assert np.isfinite(gpos).all() and np.isfinite(gvel).all()
    lo, hi = np.float32(0.00227), np.float32(1 - 0.00227)
    assert np.all(gpos >= lo) and np.all(gpos <= hi)


def _sampled_all_pairs_densities(spos, sample, h):
    """FP64 sum of (h^2 - r^2)^3 over all particles within h of each sampled
    particle, found by bucketing every particle into cells of edge h (numpy
    only): the neighbours of a particle lie in its own and the 26 adjacent
    cells."""
    p = spos.astype(np.float64)
    cell = np.floor(p / h).astype(np.int64) + 1  # >= 1, so the -1 neighbours stay >= 0
    dims = cell.max(0) + 2
    key = (cell[:, 2] * dims[1] + cell[:, 1]) * dims[0] + cell[:, 0]
    order = np.argsort(key, kind="stable")
    skey = key[order]
    out = []
    for i in sample:
        cx, cy, cz = cell[i]
        parts = []
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                k0 = ((cz + dz) * dims[1] + (cy + dy)) * dims[0] + (cx - 1)
                lo, hi = np.searchsorted(skey, [k0, k0 + 3])
                parts.append(order[lo:hi])
        nb = np.concatenate(parts)
        r2 = ((p[nb] - p[i]) ** 2).sum(1)
        out.append(((h * h - r2[r2 < h * h]) ** 3).sum())
    return np.array(out)


def test_large_scale_16m_lattice(oracle):
    """16,000,000 particles (a 200 x 400 x 200 jittered lattice, 72M grid
    cells): after 5 steps the state checks are clean (sorted, permutation,
    cell table, inside the box, finite), and the densities of 200 sampled
    particles equal all-pairs sums over their cell neighbourhoods (FP64,
    within the FP32 summation-order band)."""
    r = 0.0012
    prm = params_16k(particleRadius=r, kernelRadius=4 * r)
    rng = np.random.default_rng(16)
    g = np.stack(np.meshgrid(np.arange(200), np.arange(400), np.arange(200), indexing="ij"), -1).reshape(-1, 3)
    pos = (0.01 + 2 * r * g + rng.uniform(-0.2, 0.2, size=g.shape) * 2 * r).astype(np.float32)
    del g
    n = pos.shape[0]
    assert n == 16_000_000
    with solver_with(prm, pos) as s:
        s.makeReady()
        s.step(5)
        rep = s.checkState()
        assert all(rep[k] == 0 for k in ("non_finite", "outside_box", "unsorted", "cell_table_mismatch", "bad_ids"))
        assert rep["n"] == n
        rho, _ = s.computeDensity()
        spos, _, ids, _ = s.sortedState()
    h = np.float64(np.float32(4 * r))
    d = oracle.derive(prm.to_c())
    sample = rng.choice(n, 200, replace=False)
    w = _sampled_all_pairs_densities(spos, sample, h)
    assert np.all(np.abs(rho[sample] / (d["cd"] * w) - 1.0) < 2e-5)


def test_gather_depth_follows_scene_size_unless_set():
    """Small scenes gather four neighbours per batch, large ones two; an
    explicit sf_set_tuning is kept across uploads."""
    import ctypes
    lib = C.load()

    def prefetch(s):
        t = C.sf_tuning()
        C.check(lib.sf_get_tuning(s.handle, ctypes.byref(t)))
        return t.prefetch

    prm = params_16k()
    small = jittered_block()
    big = np.concatenate([jittered_block(n_side=(64, 64, 64), spacing=0.0125, seed=s, origin=0.05 + 0.1 * s)
                          for s in range(2)])
    assert small.shape[0] < 262144 <= big.shape[0]
    with solver_with(prm, small) as s:
        assert prefetch(s) == 4
        s.setParticles(big)
        assert prefetch(s) == 2
        C.check(lib.sf_set_tuning(s.handle, ctypes.byref(C.sf_tuning(2, 128, 128, 2))))
        s.setParticles(small)
        assert prefetch(s) == 2
