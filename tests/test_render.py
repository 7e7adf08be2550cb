"""Headless sphere-impostor rendering (the reference's particle shaders as
CUDA kernels) against the CPU restatement."""
import numpy as np
import pytest

from helpers import params_16k, params_reference_box
from simplefluid_gb300 import SPHSolver, render_params, save_ppm, scene_positions
from simplefluid_gb300 import _capi as C


def test_render_params_defaults_follow_the_viewer(lib):
    rp = render_params()
    assert (rp.width, rp.height) == (1200, 1000)
    assert list(rp.eye) == pytest.approx([-3.0, 0.8, 0.0]) and list(rp.focus) == pytest.approx([0.0, -0.2, 0.0])
    assert rp.fovy_deg == 55.0 and rp.num_lights == 1 and rp.mat_shininess == 250.0
    assert list(rp.mat_diffuse) == pytest.approx([1.0, 0.63, 0.3, 1.0])


def test_oracle_single_sprite_geometry(oracle):
    """One particle at the camera focus lands in the image centre as a disc of
    diameter radius * (h / tan(fovy/2)) / distance pixels, lit from the light."""
    prm = params_16k(particleRadius=0.2, kernelRadius=0.8)
    rp = render_params(width=200, height=160)
    focus = np.array([[0.0, -0.2, 0.0]], np.float32)
    rgba, depth, owner = oracle.render(prm.to_c(), rp, focus)
    covered = owner == 0
    dist = np.linalg.norm(np.array([-3.0, 0.8, 0.0]) - focus[0])
    diameter = 0.2 * (160 / np.tan(np.radians(27.5))) / dist
    assert abs(covered.sum() - np.pi * (diameter / 2) ** 2) < 0.05 * covered.sum()
    ys, xs = np.nonzero(covered)
    assert abs(xs.mean() + 0.5 - 100) < 1.0 and abs(ys.mean() + 0.5 - 80) < 1.0
    assert np.all(rgba[covered][:, 3] == 1.0) and np.all(rgba[~covered] == 0.0)
    assert np.all(rgba[covered][:, :3] > 0.03)  # at least the ambient term


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [C.SF_COLOR_UNIFORM, C.SF_COLOR_RANDOM, C.SF_COLOR_RAMP])
def test_render_matches_oracle(oracle, tmp_path, mode):
    prm = params_reference_box(resolution=24, scene=C.SF_SCENE_DAMBREAK)
    pos = scene_positions(prm, C.SF_SCENE_DAMBREAK)
    rp = render_params(width=320, height=240, color_mode=mode)
    with SPHSolver(prm) as s:
        s.setParticles(pos)
        s.step(30)
        state, _ = s.getState()
        rgba, depth, owner = s.render(rp)
    orgba, odepth, oowner = oracle.render(prm.to_c(), rp, state)
    assert (owner != 0xffffffff).sum() > 1000
    assert np.array_equal(owner, oowner)
    assert np.array_equal(depth.view(np.uint32), odepth.view(np.uint32))
    assert np.max(np.abs(rgba - orgba)) < 1e-4
    save_ppm(str(tmp_path / "frame.ppm"), rgba)
    assert (tmp_path / "frame.ppm").stat().st_size == 320 * 240 * 3 + len(b"P6\n320 240\n255\n")


@pytest.mark.gpu
def test_render_rejects_bad_parameters():
    with SPHSolver(params_16k()) as s:
        s.setParticles(np.zeros((4, 3), np.float32) + 0.5)
        for kw in (dict(width=0), dict(num_lights=9), dict(color_mode=5), dict(fovy_deg=0.0)):
            with pytest.raises(C.SFError):
                s.render(render_params(**kw))


def _random_view(seed: int):
    """A seeded camera, light set, material and colour mode around the unit box."""
    rng = np.random.default_rng(300 + seed)
    d = rng.normal(size=3)
    eye = 0.5 + d / np.linalg.norm(d) * rng.uniform(1.2, 4.0)
    rp = render_params(width=int(rng.integers(64, 400)), height=int(rng.integers(64, 300)),
                       eye=tuple(eye), focus=tuple(rng.uniform(0.3, 0.7, 3)), fovy_deg=float(rng.uniform(30, 80)),
                       point_radius=float(rng.choice([0.0, rng.uniform(0.005, 0.05)])),
                       num_lights=int(rng.integers(1, 9)), mat_shininess=float(rng.uniform(1, 300)),
                       color_mode=int(rng.integers(0, 3)), color_seed=int(rng.integers(0, 2 ** 32)))
    for l in range(8):
        rp.light_position[l][:] = [*rng.uniform(-10, 10, 3), 1.0]
        rp.light_ambient[l][:] = [*rng.uniform(0, 0.2, 3), 1.0]
        rp.light_diffuse[l][:] = [*rng.uniform(0, 1, 3), 1.0]
        rp.light_specular[l][:] = [*rng.uniform(0, 1, 3), 1.0]
    rp.mat_ambient[:] = [*rng.uniform(0, 1, 3), 1.0]
    rp.mat_diffuse[:] = [*rng.uniform(0, 1, 3), 1.0]
    rp.mat_specular[:] = [*rng.uniform(0, 1, 3), 1.0]
    return rp


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(12))
def test_render_random_views_match_oracle(oracle, seed):
    """Seeded cameras, lights, materials, point radii and colour modes over a
    random particle set: visibility and depth bit-identical to the oracle,
    colours within 1e-4 relative."""
    rng = np.random.default_rng(seed)
    prm = params_16k()
    pos = np.concatenate([rng.uniform(0.0, 1.0, size=(3000, 3)),
                          0.5 + rng.normal(scale=0.05, size=(1000, 3))]).astype(np.float32)
    rp = _random_view(seed)
    with SPHSolver(prm) as s:
        s.setParticles(pos)
        state, _ = s.getState()
        rgba, depth, owner = s.render(rp)
    orgba, odepth, oowner = oracle.render(prm.to_c(), rp, state)
    assert np.array_equal(owner, oowner)
    assert np.array_equal(depth.view(np.uint32), odepth.view(np.uint32))
    assert np.all(np.abs(rgba - orgba) <= 1e-4 * np.maximum(1.0, np.abs(orgba)))


def test_random_views_are_valid():
    modes = set()
    for seed in range(12):
        rp = _random_view(seed)
        assert 1 <= rp.num_lights <= 8 and rp.width >= 64 and rp.height >= 64
        assert 30.0 <= rp.fovy_deg <= 80.0 and rp.znear > 0.0 and rp.zfar > rp.znear
        modes.add(rp.color_mode)
    assert modes == {C.SF_COLOR_UNIFORM, C.SF_COLOR_RANDOM, C.SF_COLOR_RAMP}
