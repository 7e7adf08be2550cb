"""Workload configuration files: every file loads and validates, the scene
configurations generate the particle counts their descriptions state, and the
bench reads its workloads from them."""
import json
import os
import sys

import pytest

from simplefluid_gb300 import configs, scene_positions

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_every_configuration_loads():
    names = configs.available()
    assert {"double_dambreak_1m", "dambreak_16k", "dambreak_64k", "sphere_pool", "batched_cubes",
            "adjoint_64k"} <= set(names)
    for n in names:
        cfg = configs.load(n)
        assert cfg["name"] == n and cfg["description"]
        prm = configs.params(cfg)
        assert prm.kernelRadius > prm.particleRadius > 0


@pytest.mark.parametrize("name,count", [("dambreak_16k", 16000), ("dambreak_64k", 65536),
                                        ("double_dambreak_1m", 1048576), ("sphere_pool", 3345599)])
def test_scene_configurations_generate_their_particles(name, count):
    cfg = configs.load(name)
    prm = configs.params(cfg)
    pos = scene_positions(prm, prm.scene, cfg["seed"])
    assert pos.shape == (count, 3)
    assert (pos >= 0).all() and (pos <= 1).all()


def test_headline_parameters():
    prm = configs.params("double_dambreak_1m")
    assert (prm.particleRadius, prm.kernelRadius, prm.pressureStiffness, prm.viscosity) == (0.0025, 0.01, 50.0, 0.01)
    assert (prm.restDensity, prm.timeStep, prm.gravity) == (1000.0, 1e-4, (0.0, -9.8, 0.0))


def test_bench_reads_the_configurations():
    sys.path.insert(0, ROOT)
    import bench
    assert sorted(bench.WORKLOADS) == configs.available("scene")
    for wl in bench.WORKLOADS:
        assert bench.make_params(wl) == configs.params(wl)


@pytest.mark.parametrize("bad,match", [
    ({"kind": "scene", "params": {"particleRadius": 0.01}, "extra": 1}, "unknown keys"),
    ({"kind": "scene", "params": {"particleRadiuss": 0.01}}, "unknown SPHParameters fields"),
    ({"kind": "scene", "params": {"scene": "no_such_scene"}}, "unknown scene"),
    ({"kind": "movie", "params": {}}, "kind must be"),
    ({"kind": "batch", "params": {}}, "unknown keys"),
])
def test_invalid_configurations_are_rejected(tmp_path, monkeypatch, bad, match):
    monkeypatch.setattr(configs, "CONFIG_DIR", str(tmp_path))
    cfg = {"name": "bad", "description": "x", "seed": 1, "steps": 1, **bad}
    (tmp_path / "bad.json").write_text(json.dumps(cfg))
    with pytest.raises(ValueError, match=match):
        configs.load("bad")


def test_missing_configuration(tmp_path, monkeypatch):
    monkeypatch.setattr(configs, "CONFIG_DIR", str(tmp_path))
    with pytest.raises(ValueError, match="no workload configuration"):
        configs.load("absent")
