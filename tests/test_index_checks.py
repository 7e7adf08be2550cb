"""The checked build: kernels compiled with SF_DEVICE_CHECKS=1 check every
cell-table range end and neighbour-list entry before use and count bad ones.

* CPU: the release library reports that it has no checks and counts nothing.
* GPU: the checked library, run through the candidate walks, the list and
  rescan paths of the force pass under every list layout, a batch under the
  five-launch and the persistent step, whole frames with the adaptive
  sub-step and the adjoint, counts no bad index and gives the release
  library's bits.
"""
import json
import os
import subprocess
import sys

import pytest

from simplefluid_gb300 import _capi as C

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# Run in a subprocess: the library a process uses is chosen when it loads.
SCRIPT = r"""
import hashlib, json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from simplefluid_gb300 import SPHBatch, SPHParameters, SPHSolver, batch_cubes, scene_positions
from simplefluid_gb300 import _capi as C
C.index_checks(reset=True)
h = hashlib.sha1()
prm = SPHParameters(particleRadius=0.01, kernelRadius=0.04, scene=16)
pos = scene_positions(prm, 16)
with SPHSolver(prm) as s:
    s.setParticles(pos)
    s.step(40)
    p, v = s.getState()
    cnt, hsh = s.neighbourStats()
    h.update(p.tobytes()); h.update(v.tobytes()); h.update(cnt.tobytes()); h.update(hsh.tobytes())
# a dense cluster: lists overflow, the force pass rescans the candidate cells
rng = np.random.default_rng(4)
cl = (0.5 + rng.uniform(0, 0.03, size=(600, 3))).astype(np.float32)
with SPHSolver(prm) as s:
    s.setParticles(cl)
    s.step(3)
    p, v = s.getState()
    h.update(p.tobytes()); h.update(v.tobytes())
# a batch of three scenes
params, counts, bpos = batch_cubes(7, 3, SPHParameters(particleRadius=0.02, kernelRadius=0.08))
with SPHBatch(params) as b:
    b.setState(counts, bpos)
    b.step(5)
    bp, bv = b.getState()
    h.update(bp.tobytes()); h.update(bv.tobytes())
# the other neighbour-list layouts (none, staged, 16-bit warp tiles), on the
# scene and on the overflowing cluster
for mode in (0, 1, 3):
    for pts in (pos, cl):
        with SPHSolver(prm) as s:
            s.setParticles(pts)
            t = s.getTuning()
            t.list_mode = mode
            s.setTuning(t)
            s.step(4)
            p, v = s.getState()
            h.update(p.tobytes()); h.update(v.tobytes())
# the persistent batched step
with SPHBatch(params) as b:
    b.setState(counts, bpos)
    b.setTuning(C.sf_tuning(C.SF_LIST_TILE, 256, 128, 2, 0, 4, 256))
    b.step(5)
    bp, bv = b.getState()
    h.update(bp.tobytes()); h.update(bv.tobytes())
# whole frames with the adaptive sub-step
aprm = SPHParameters(particleRadius=0.01, kernelRadius=0.04, scene=16, adaptiveTimeStep=True, timeStep=2e-3)
with SPHSolver(aprm) as s:
    s.setParticles(pos)
    t_sim, k = s.advanceFrames(1, 4e-3, 60)
    p, v = s.getState()
    h.update(p.tobytes()); h.update(v.tobytes()); h.update(np.array([t_sim, k]).tobytes())
# the adjoint (recorded lists, rescans, reverse sweep)
sub = pos[:4000]
vel = np.random.default_rng(5).normal(scale=0.05, size=sub.shape).astype(np.float32)
target = np.random.default_rng(6).uniform(size=8 ** 3).astype(np.float32)
target /= target.sum()
with SPHSolver(prm) as s:
    s.setParticles(sub, vel)
    s.forward(20, 10)
    L, g = s.lossHistogram(target)
    dx0, dv0, dmu, dk = s.adjoint(g)
    h.update(dx0.tobytes()); h.update(dv0.tobytes())
failures, compiled = C.index_checks()
print(json.dumps({"hash": h.hexdigest(), "failures": failures, "compiled": compiled}))
"""


def _run(checked: bool) -> dict:
    env = dict(os.environ, SIMPLEFLUID_GB300_CHECKED="1" if checked else "0")
    out = subprocess.run([sys.executable, "-c", SCRIPT, ROOT], env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-3000:]
    return json.loads(out.stdout.strip().splitlines()[-1])


def test_release_build_has_no_checks(lib):
    failures, compiled = C.index_checks(reset=True)
    assert (failures, compiled) == (0, False)


@pytest.mark.gpu
def test_checked_build_counts_no_bad_index_and_matches_release():
    from simplefluid_gb300 import build as B
    B.build(checked=True)
    checked = _run(True)
    release = _run(False)
    assert checked["compiled"] is True and release["compiled"] is False
    assert checked["failures"] == 0
    assert checked["hash"] == release["hash"]
