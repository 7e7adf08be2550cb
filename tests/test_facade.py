"""The C++ façade (include/simplefluid/SPHSolver.hpp): it compiles on the host
(CPU) and, on a GPU, a program written like the reference's Simulator gives
exactly the state of the same sub-steps driven from Python."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from helpers import params_16k
from simplefluid_gb300 import SPHSolver, scene_positions, substeps_per_frame
from simplefluid_gb300 import _capi as C

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_check.cpp")


def _cxx():
    return shutil.which("g++") or shutil.which("c++")


def test_facade_header_compiles():
    cxx = _cxx()
    if cxx is None:
        pytest.skip("no C++ compiler")
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
                        SRC], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_facade_simulator_matches_python(lib, tmp_path):
    cxx = _cxx()
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "facade_check")
    libdir = os.path.dirname(C.LIB_PATH)
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-L", libdir,
                        "-lsimplefluid_gb300", f"-Wl,-rpath,{libdir}", "-lpthread", "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = str(tmp_path / "state.bin")
    r = subprocess.run([exe, str(C.SF_SCENE_DAMBREAK_16K), "2", out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(out, dtype=np.uint32, count=3)
    n, substeps, frames = (int(x) for x in raw)
    data = np.fromfile(out, dtype=np.float32, offset=12).reshape(2, n, 3)
    k = substeps_per_frame(1e-4)
    assert n == 16000 and frames == 2 and substeps == 2 * k
    prm = params_16k()
    with SPHSolver(prm) as s:
        s.setParticles(scene_positions(prm, C.SF_SCENE_DAMBREAK_16K))
        s.step(2 * k)
        pos, vel = s.getState()
    assert np.array_equal(data[0].view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(data[1].view(np.uint32), vel.view(np.uint32))
