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
