"""The CPU oracle against the reference's golden vectors and against the
mathematics it restates (CPU only)."""
import hashlib
import platform
import os

import numpy as np
import pytest

from helpers import normwise_err, params_16k, rel_err
from simplefluid_gb300 import _capi as C

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _ref_cases():
    d = np.load(os.path.join(GOLD, "ref_scenes.npz"))
    keys = sorted({k.rsplit("_", 1)[0] for k in d.files})
    return d, keys


def _cparams(r, box=(-1.0, 1.0)):
    p = C.sf_params()
    p.particle_radius = r
    p.kernel_radius = 4 * r
    p.rest_density = 1000.0
    p.time_step = 1e-4
    for a in range(3):
        p.box_min[a], p.box_max[a] = box
    return p


def test_oracle_scenes_match_reference_golden(oracle):
    """Scene generators restated from Source/SceneManager.cpp:41-173 reproduce the
    reference's own compiled generator bit for bit."""
    d, keys = _ref_cases()
    assert len(keys) >= 20
    for k in keys:
        s, r = int(d[k + "_scene"]), float(d[k + "_r"])
        pos = oracle.scene(_cparams(r), s)
        assert pos.shape[0] == int(d[k + "_n"]), k
        assert hashlib.sha256(pos.tobytes()).hexdigest() == str(d[k + "_sha"]), k
        if k + "_pos" in d.files:
            assert np.array_equal(pos.view(np.uint32), d[k + "_pos"].view(np.uint32)), k


def test_oracle_scenes_match_compiled_reference_live(oracle):
    """Where the reference's own scene generator was built (oracle/_ref, by
    the build entry point on a machine holding the reference tree), compare
    against it directly too."""
    if oracle.build_ref() is None:
        pytest.skip("the reference's scene generator is not built on this machine")
    for s in range(4):
        for r in (0.03, 0.011, 0.0075):
            a = oracle.scene(_cparams(r), s)
            b = oracle.ref_scene(s, r)
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (s, r)


def test_oracle_regression_fixture(oracle):
    """The oracle built on this host computes the bits recorded on x86-64."""
    g = np.load(os.path.join(GOLD, "oracle_regression.npz"))
    p = params_small()
    st = oracle.State(g["pos0"])
    keys, cs = st.sort(p, want_cells=True)
    assert np.array_equal(keys, g["keys"]) and np.array_equal(st.ids, g["ids"])
    assert np.array_equal(cs, g["cell_start"])
    rho, prs, inv = st.density(p)
    assert np.array_equal(rho.view(np.uint32), g["rho"].view(np.uint32))
    acc = st.accel(p, prs, inv)
    assert np.array_equal(acc.view(np.uint32), g["acc"].view(np.uint32))
    cnt, hsh = st.neighbour_stats(p)
    assert np.array_equal(cnt, g["nbr_count"]) and np.array_equal(hsh, g["nbr_hash"])
    st2 = oracle.State(g["pos0"])
    st2.step(p, 5)
    p5, v5 = st2.original_order()
    assert np.array_equal(p5.view(np.uint32), g["pos5"].view(np.uint32))
    assert np.array_equal(v5.view(np.uint32), g["vel5"].view(np.uint32))


def params_small():
    p = C.sf_params()
    p.particle_radius = 0.02
    p.kernel_radius = 0.08
    p.pressure_stiffness = 50.0
    p.boundary_restitution = 0.1
    p.viscosity = 0.01
    p.stop_time = 5.0
    p.rest_density = 1000.0
    p.gravity[1] = -9.8
    p.time_step = 1e-4
    for a in range(3):
        p.box_min[a] = 0.0
        p.box_max[a] = 1.0
    return p


def test_poly6_normalisation(oracle):
    """sum_j m W(r_ij) over a fine lattice of spacing s (mass = rho0 s^3) is rho0:
    the poly6 constant 315/(64 pi h^9) integrates to one."""
    h = 0.04
    s = h / 10
    m = np.arange(-12, 13) * s
    X, Y, Z = np.meshgrid(m, m, m, indexing="ij")
    r2 = X * X + Y * Y + Z * Z
    w = np.where(r2 < h * h, (h * h - r2) ** 3, 0.0) * 315.0 / (64 * np.pi * h ** 9)
    assert abs(w.sum() * s ** 3 - 1.0) < 2e-3


def test_rest_density_of_lattice(oracle):
    """A particle deep inside a lattice of spacing 2r (h = 4r) sits at ~rho0."""
    p = params_small()
    p.particle_radius = 0.01
    p.kernel_radius = 0.04
    pos = oracle.scene(p, C.SF_SCENE_DAMBREAK_16K)
    st = oracle.State(pos)
    st.sort(p)
    rho, _, _ = st.density(p)
    inner = np.all((st.pos > 0.06) & (st.pos < np.array([0.34, 0.74, 0.34])), axis=1)
    assert inner.sum() > 1000
    assert np.allclose(rho[inner], rho[inner][0], rtol=1e-5)
    assert abs(rho[inner].mean() / 1000.0 - 1.0) < 0.02


def test_pairwise_momentum_conservation(oracle):
    """Pressure and viscosity forces are pairwise antisymmetric once divided by
    rho_i: sum_i a_i = 0 without gravity and walls (FP64)."""
    p = params_small()
    p.gravity[1] = 0.0
    rng = np.random.default_rng(1)
    pos = rng.uniform(0.3, 0.7, size=(3000, 3))
    vel = rng.normal(size=(3000, 3))
    st = oracle.State(pos, vel, dtype=np.float64)
    st.sort(p)
    acc = st.accel(p)
    assert np.abs(acc.sum(0)).max() < 1e-9 * np.abs(acc).sum()


def test_fp32_tracks_fp64(oracle):
    """One step in FP32 stays within 1e-5 (density) of the FP64 oracle."""
    p = params_small()
    pos = oracle.scene(p, C.SF_SCENE_DAMBREAK_16K)[:4000]
    s32 = oracle.State(pos)
    s64 = oracle.State(pos, dtype=np.float64)
    s32.sort(p)
    s64.sort(p)
    assert np.array_equal(s32.ids, s64.ids)
    r32, _, _ = s32.density(p)
    r64, _, _ = s64.density(p)
    assert rel_err(r32, r64) < 1e-5
    a32 = s32.accel(p)
    a64 = s64.accel(p)
    assert normwise_err(a32, a64) < 1e-4


def test_sort_is_stable_and_grid_consistent(oracle):
    p = params_small()
    rng = np.random.default_rng(7)
    pos = rng.uniform(0, 1, size=(5000, 3)).astype(np.float32)
    pos[::7] = pos[0]  # many equal keys
    st = oracle.State(pos)
    keys, cs = st.sort(p, want_cells=True)
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)
    same = np.diff(keys.astype(np.int64)) == 0
    assert np.all(np.diff(st.ids.astype(np.int64))[same] > 0)  # stable: original order within a cell
    assert cs[0] == 0 and cs[-1] == st.n and np.all(np.diff(cs.astype(np.int64)) >= 0)
    assert np.array_equal(np.sort(st.ids), np.arange(st.n))


def test_oracle_step_deterministic_across_threads(oracle):
    p = params_small()
    pos = oracle.scene(p, C.SF_SCENE_DAMBREAK_16K)[:3000]
    a = oracle.State(pos)
    b = oracle.State(pos)
    a.step(p, 3, threads=1)
    b.step(p, 3, threads=4)
    assert np.array_equal(a.pos.view(np.uint32), b.pos.view(np.uint32))
    assert np.array_equal(a.ids, b.ids)


def test_boundary_clamp_and_restitution(oracle):
    p = params_small()
    p.boundary_restitution = 0.5
    pos = np.array([[0.5, 0.0201, 0.5]], np.float32)
    vel = np.array([[0.0, -10.0, 0.0]], np.float32)
    st = oracle.State(pos, vel)
    st.step(p, 1)
    lo = np.float32(0.0 + 0.02)
    assert st.pos[0, 1] == lo
    assert st.vel[0, 1] > 0 and abs(st.vel[0, 1] - 0.5 * (10.0 + 9.8e-4)) < 1e-4


def test_params_default_is_16k_workload():
    p = params_16k()
    assert p.kernelRadius == 4 * p.particleRadius


def test_frame_accounting_matches_the_reference_frame_loop(oracle):
    """The oracle's frame accounting (sub-steps summed in float to 1/30 s frames,
    frame times summed in float to the simulated time) reports what the
    reference's own frame loop (Source/Simulator.cpp, run on the same sub-step
    sizes; tests/golden/ref_frames.npz) reports: sub-steps per frame and the
    simulated time after each frame, bit for bit."""
    g = np.load(os.path.join(GOLD, "ref_frames.npz"))
    for case in ("fixed", "varied", "adaptive16k"):
        sub, times = oracle.frame_accounting(g[case + "_dts"], float(g[case + "_stop"]))
        assert np.array_equal(sub, g[case + "_substeps"]), case
        assert np.array_equal(times.view(np.uint32), g[case + "_sim_times"].view(np.uint32)), case


def test_frame_accounting_against_the_reference_live(oracle):
    """Where the reference's frame loop is built here, compare on fresh sizes too."""
    rng = np.random.default_rng(5)
    dts = rng.uniform(1e-5, 4e-3, size=20000).astype(np.float32)
    ref = oracle.ref_frames(dts, 1.0)
    if ref is None:
        pytest.skip("the reference's frame loop is not built on this machine")
    sub, times = oracle.frame_accounting(dts, 1.0)
    assert np.array_equal(sub, ref[0]) and np.array_equal(times.view(np.uint32), ref[1].view(np.uint32))


def test_oracle_adaptive_substeps_reproduce_the_frames_fixture(oracle):
    """The oracle's adaptive sub-steps on the 16,000-particle dambreak from rest
    are the sizes the frames fixture was made from (on this host's build)."""
    from simplefluid_gb300 import SPHParameters
    g = np.load(os.path.join(GOLD, "ref_frames.npz"))
    p = SPHParameters(particleRadius=0.01, kernelRadius=0.04, adaptiveTimeStep=True, timeStep=5e-3, stopTime=0.1,
                      scene=16).to_c()
    st = oracle.State(oracle.scene(p, 16))
    _, k, dts = st.frames(p, 4, record_dts=20000)
    n = g["adaptive16k_dts"].size
    assert k >= n and np.array_equal(dts[:n].view(np.uint32), g["adaptive16k_dts"].view(np.uint32))


def _shader_case(g, name):
    rp = C.sf_render_params.from_buffer_copy(g[name + "_rp"].tobytes())
    p = _cparams(float(g[name + "_radius"]))
    return rp, p


def _ulps(a, b):
    """Largest distance in units in the last place between equal-shaped float32 arrays."""
    ia = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    ib = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    return int(np.abs(ia - ib).max()) if ia.size else 0


# The fixture was written on x86-64; the fragment colours go through the C
# library's powf, which other hosts' libraries may round differently.
POW_ULPS = 0 if platform.machine() in ("x86_64", "AMD64") else 2


def test_oracle_shader_stages_match_the_reference_shaders(oracle):
    """The oracle's restatement of the particle shaders (vertex: eye-space
    centre, point size, clip position; fragment: discard test on the point
    coordinate and Blinn-Phong over the lights) reproduces the reference's own
    Shaders/particle.vs.glsl and particle.fs.glsl, compiled as C++ on seeded
    particles and fragments (tests/golden/ref_shader.npz), bit for bit; two
    settings (the viewer's, and eight lights with another camera) and both
    uniform and per-particle colours."""
    g = np.load(os.path.join(GOLD, "ref_shader.npz"))
    for name in ("viewer", "lights8"):
        rp, p = _shader_case(g, name)
        eye, size, clip = oracle.particle_vertex(p, rp, g[name + "_pos"])
        for got, key in ((eye, "_eye"), (size, "_size"), (clip, "_clip")):
            assert np.array_equal(got.view(np.uint32), g[name + key].view(np.uint32)), name + key
        fe, uv = eye[g[name + "_frag_idx"]], g[name + "_uv"]
        keep = ~g[name + "_discarded"]
        assert 0.1 < g[name + "_discarded"].mean() < 0.4 and keep[-8:].sum() == 6  # rim kept, corners not
        for color, key in ((None, "_rgba_uniform"), (g[name + "_color"], "_rgba_color")):
            rgba, disc = oracle.particle_fragment(p, rp, fe, uv, color)
            assert np.array_equal(disc, g[name + "_discarded"]), name + key
            assert _ulps(rgba[keep], g[name + key][keep]) <= POW_ULPS, name + key


def test_oracle_shader_stages_against_the_reference_live(oracle):
    """Where the reference's shaders are built here, compare on fresh inputs too."""
    from simplefluid_gb300 import render_params
    rp = render_params(width=800, height=600, eye=(-1.5, 2.0, 2.5), num_lights=3, mat_shininess=12.5)
    for l in range(3):
        rp.light_position[l][:] = [4.0 * l - 4.0, 6.0, 3.0 - l, 1.0]
        rp.light_diffuse[l][:] = [0.3 + 0.2 * l, 0.5, 0.9 - 0.2 * l, 1.0]
    p = _cparams(0.015)
    V, Pm, scale, rad = oracle.render_camera(p, rp)
    rng = np.random.default_rng(11)
    pos = rng.uniform(-1.2, 1.2, size=(300, 3)).astype(np.float32)
    ref = oracle.ref_particle_vertex(V, Pm, rad, scale, pos)
    if ref is None:
        pytest.skip("the reference's shaders are not built on this machine")
    got = oracle.particle_vertex(p, rp, pos)
    for a, b in zip(got, ref):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    idx = rng.integers(0, 300, 1500)
    uv = rng.uniform(-0.05, 1.05, size=(1500, 2)).astype(np.float32)
    color = rng.uniform(0.0, 1.0, size=(1500, 3)).astype(np.float32)
    rgba, disc = oracle.particle_fragment(p, rp, got[0][idx], uv, color)
    rrgba, rdisc = oracle.ref_particle_fragment(rp, rad, got[0][idx], uv, color)
    assert np.array_equal(disc, rdisc) and 0 < disc.sum() < disc.size
    assert np.array_equal(rgba[~disc].view(np.uint32), rrgba[~rdisc].view(np.uint32))
