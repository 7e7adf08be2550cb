"""The C-ABI library on the host: it loads, exports every declared entry point,
validates parameters and generates the reference scenes (CPU only; no compute
call reaches a GPU)."""
import ctypes
import glob
import hashlib
import os
import re

import numpy as np
import pytest

from helpers import params_16k, params_1m
from simplefluid_gb300 import SPHParameters, SceneManager, scene_positions, substeps_per_frame
from simplefluid_gb300 import _capi as C

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        names |= set(re.findall(r"SF_API\s+[\w\s\*]+?\b(sf\w+)\s*\(", src))
    return sorted(names)


def test_library_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 26
    for n in names:
        assert hasattr(lib, n), n
    # and the Python binding covers each of them
    assert set(names) <= set(C.PROTOTYPES), set(names) - set(C.PROTOTYPES)


def test_params_default_and_update(lib):
    p = C.sf_params()
    C.check(lib.sf_params_default(ctypes.byref(p)))
    assert p.kernel_radius == pytest.approx(0.04) and p.particle_radius == pytest.approx(0.01)
    assert p.rest_density == 1000.0 and p.time_step == pytest.approx(1e-4)
    C.check(lib.sf_params_update(ctypes.byref(p)))
    # the Python mirror has the same defaults
    q = SPHParameters().to_c()
    assert bytes(q) == bytes(p)


@pytest.mark.parametrize("field,value", [
    ("kernel_radius", 0.0), ("kernel_radius", float("nan")), ("particle_radius", -1.0),
    ("time_step", 0.0), ("rest_density", 0.0), ("boundary_restitution", 1.5), ("viscosity", -0.1),
    ("pressure_stiffness", -1.0), ("eos", 7), ("num_threads", -2)])
def test_params_update_rejects(lib, field, value):
    p = C.sf_params()
    lib.sf_params_default(ctypes.byref(p))
    setattr(p, field, value)
    st = lib.sf_params_update(ctypes.byref(p))
    assert st == C.SF_ERR_INVALID_ARGUMENT
    assert lib.sf_last_error()


def test_params_update_rejects_huge_grid(lib):
    p = C.sf_params()
    lib.sf_params_default(ctypes.byref(p))
    p.kernel_radius = 1e-4
    p.particle_radius = 2.5e-5
    assert lib.sf_params_update(ctypes.byref(p)) == C.SF_ERR_GRID_TOO_LARGE


def test_python_updateParams_raises():
    with pytest.raises(C.SFError):
        SPHParameters(kernelRadius=-1.0).updateParams()


def test_scenes_match_reference_golden(lib):
    """The product's SceneManager reproduces the reference's own generator."""
    d = np.load(os.path.join(GOLD, "ref_scenes.npz"))
    keys = sorted({k.rsplit("_", 1)[0] for k in d.files})
    for k in keys:
        s, r = int(d[k + "_scene"]), float(d[k + "_r"])
        prm = SPHParameters(particleRadius=r, kernelRadius=4 * r, boxMin=(-1, -1, -1), boxMax=(1, 1, 1))
        pos = scene_positions(prm, s)
        assert pos.shape[0] == int(d[k + "_n"]), k
        assert hashlib.sha256(pos.tobytes()).hexdigest() == str(d[k + "_sha"]), k


def test_scene_manager_dispatch():
    prm = SPHParameters(particleRadius=0.05, kernelRadius=0.2, scene=C.SF_SCENE_CUBE_DROP)
    pos, vel = SceneManager(prm).setupScene()
    assert pos.shape == (1000, 3) and not vel.any()
    pos2, _ = SceneManager(prm).setupSceneCubeDrop()
    assert np.array_equal(pos, pos2)


def test_workload_scenes_match_oracle(oracle):
    for prm, scene, n in ((params_16k(), C.SF_SCENE_DAMBREAK_16K, 16000),
                          (params_1m(), C.SF_SCENE_DOUBLE_DAMBREAK_1M, 1048576)):
        a = scene_positions(prm, scene, 20171)
        assert a.shape == (n, 3)
        b = oracle.scene(prm.to_c(), scene, 20171)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        assert np.all(a >= 0.0) and np.all(a <= 1.0)


def test_scene_capacity_error(lib):
    p = params_16k().to_c()
    out = np.zeros((10, 3), np.float32)
    n = ctypes.c_uint32()
    st = lib.sf_setup_scene(ctypes.byref(p), C.SF_SCENE_DAMBREAK_16K, 0, out.ctypes.data_as(ctypes.c_void_p), None,
                            10, ctypes.byref(n))
    assert st == C.SF_ERR_CAPACITY and n.value == 16000


def test_unknown_scene(lib):
    p = params_16k().to_c()
    n = ctypes.c_uint32()
    assert lib.sf_scene_count(ctypes.byref(p), 99, 0, ctypes.byref(n)) == C.SF_ERR_INVALID_ARGUMENT


def test_substeps_per_frame_matches_float_accumulation():
    # float32 accumulation of 1e-4 reaches 1/30 after 334 sub-steps
    assert substeps_per_frame(1e-4) == 334
    assert substeps_per_frame(1.0 / 30.0 + 1e-6) == 1


def test_null_arguments(lib):
    assert lib.sf_create(None, None) == C.SF_ERR_INVALID_ARGUMENT
    assert lib.sf_destroy(None) == C.SF_OK
    assert lib.sf_make_ready(None) == C.SF_ERR_INVALID_ARGUMENT
