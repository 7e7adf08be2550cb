"""Failure detection without a GPU fault: sf_check_state counts violated
invariants of the solver state on the GPU.

The faults are planted on the host side or through the in-bounds device views:
  * a NaN or out-of-box particle in the uploaded state;
  * a dense cluster that overflows the neighbour lists;
  * a duplicated caller index and two swapped positions, written into the
    cell-sorted arrays through sf_device_state.
Every access of the checking kernels stays inside the state's arrays, so no
planted fault can fault the GPU.
"""
import ctypes

import numpy as np
import pytest

from helpers import params_16k
from simplefluid_gb300 import SPHBatch, SPHSolver, batch_cubes, scene_positions
from simplefluid_gb300 import _capi as C

pytestmark = pytest.mark.gpu

CLEAN = ("non_finite", "outside_box", "unsorted", "cell_table_mismatch", "bad_ids")


def _block(seed=3):
    prm = params_16k()
    pos = scene_positions(prm, C.SF_SCENE_DAMBREAK_16K)
    vel = np.random.default_rng(seed).normal(scale=0.2, size=pos.shape).astype(np.float32)
    return prm, pos, vel


def test_healthy_state_reports_nothing():
    prm, pos, vel = _block()
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        r0 = s.checkState()
        s.makeReady()
        s.step(50)
        r = s.checkState()
        _, v = s.getState()
    assert r0["n"] == pos.shape[0] and all(r0[k] == 0 for k in CLEAN)
    assert all(r[k] == 0 for k in CLEAN), r
    assert r["list_overflow"] == 0
    assert r["max_speed"] == pytest.approx(float(np.sqrt((v.astype(np.float64) ** 2).sum(1)).max()), rel=1e-6)


def test_nan_and_outside_box_are_counted():
    prm, pos, vel = _block()
    pos = pos.copy()
    pos[7] = np.nan
    pos[100] = (1.5, 0.5, 0.5)
    pos[200] = (0.5, -0.25, 0.5)
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        r = s.checkState()
    assert r["non_finite"] == 1
    assert r["outside_box"] == 2
    assert r["unsorted"] == 0 and r["cell_table_mismatch"] == 0 and r["bad_ids"] == 0


def test_out_of_box_particles_are_clamped_by_a_step():
    prm, pos, vel = _block()
    pos = pos.copy()
    pos[100] = (1.5, 0.5, 0.5)
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        assert s.checkState()["outside_box"] == 1
        s.makeReady()
        s.step(1)
        assert s.checkState()["outside_box"] == 0


def test_list_overflow_is_counted():
    prm, pos, vel = _block()
    rng = np.random.default_rng(5)
    cluster = (0.6 + rng.normal(scale=0.004, size=(150, 3))).astype(np.float32)
    pos = np.concatenate([pos, cluster])
    vel = np.concatenate([vel, np.zeros_like(cluster)])
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        s.makeReady()
        s.step(1)
        r = s.checkState()
    assert r["list_overflow"] >= 100
    assert all(r[k] == 0 for k in CLEAN)


def test_corrupted_ids_and_order_are_detected():
    torch = pytest.importorskip("torch")
    prm, pos, vel = _block()
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        s.makeReady()
        s.step(3)
        s.synchronize()
        v = s.deviceState()
        n = v.n

        class _View:
            def __init__(self, ptr, shape):
                self.__cuda_array_interface__ = dict(shape=shape, typestr="<f4", data=(int(ptr), False),
                                                     strides=None, version=2)

        p4 = torch.as_tensor(_View(v.pos4, (n, 4)), device="cuda")
        # duplicate one caller index (one other index is then missing)
        orig = p4[10, 3].clone()
        p4[10, 3] = p4[11, 3]
        torch.cuda.synchronize()
        r = s.checkState()
        assert r["bad_ids"] == 2 and r["unsorted"] == 0 and r["cell_table_mismatch"] == 0
        p4[10, 3] = orig
        # swap two far-apart particles' positions: both leave their cells' ranges
        a, b = 5, n - 5
        tmp = p4[a, :3].clone()
        p4[a, :3] = p4[b, :3]
        p4[b, :3] = tmp
        torch.cuda.synchronize()
        r = s.checkState()
        assert r["cell_table_mismatch"] == 2
        assert r["unsorted"] >= 1


def test_batch_check_state():
    from simplefluid_gb300 import SPHParameters
    base = SPHParameters(particleRadius=0.005, kernelRadius=0.02)
    params, counts, pos = batch_cubes(7, 6, base)
    with SPHBatch(params) as b:
        b.setState(counts, pos)
        b.step(5)
        r = b.checkState()
    assert r["n"] == int(counts.sum())
    assert all(r[k] == 0 for k in CLEAN), r
