"""State transfer through device memory (sf_set_state_device,
sf_get_state_device, sf_device_state).

The device transfers must give exactly the state the host transfers give:
the same cell-sorted order and bits after the upload, and the same
caller-order arrays after stepping.  The device views must alias the arrays
that the inspection calls copy out.  Pointers that are not device memory of
the context's GPU are rejected.  Uploads from page-locked host arrays (which
overlap the velocity copy with the sort) must match pageable uploads.
"""
import ctypes

import numpy as np
import pytest

from helpers import params_16k
from simplefluid_gb300 import SPHSolver, scene_positions
from simplefluid_gb300 import _capi as C
from simplefluid_gb300.solver import _cuda_array, _stream_handle


class _Cai:
    """A bare __cuda_array_interface__ (version 2) over a raw pointer."""

    def __init__(self, ptr, shape, typestr="<f4", strides=None):
        self.__cuda_array_interface__ = dict(shape=tuple(shape), typestr=typestr, data=(int(ptr), False),
                                             strides=strides, version=2)


# ---------------------------------------------------------------- host side

def test_cuda_array_validation():
    assert _cuda_array(_Cai(4096, (10, 3)), "x")[1] == 10
    assert _cuda_array(_Cai(0, (0, 3)), "x") == (None, 0)
    with pytest.raises(ValueError):
        _cuda_array(_Cai(4096, (10, 4)), "x")
    with pytest.raises(ValueError):
        _cuda_array(_Cai(4096, (10, 3), typestr="<f8"), "x")
    with pytest.raises(ValueError):
        _cuda_array(_Cai(4096, (10, 3), strides=(4, 40)), "x")
    with pytest.raises(TypeError):
        _cuda_array(np.zeros((10, 3), np.float32), "x")


def test_stream_handle_mapping():
    class S:
        cuda_stream = 1234
    assert _stream_handle(None) is None
    assert _stream_handle(S()).value == 1234
    assert _stream_handle(0).value == 1  # the default stream as cudaStreamLegacy
    a = _Cai(4096, (1, 3))
    a.__cuda_array_interface__["stream"] = 77
    assert _stream_handle(None, a).value == 77


# ---------------------------------------------------------------- on the GPU

def _scene():
    prm = params_16k()
    pos = scene_positions(prm, C.SF_SCENE_DAMBREAK_16K)
    rng = np.random.default_rng(11)
    vel = rng.uniform(-0.3, 0.3, size=pos.shape).astype(np.float32)
    return prm, pos, vel


@pytest.mark.gpu
def test_device_upload_matches_host_upload():
    torch = pytest.importorskip("torch")
    prm, pos, vel = _scene()
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        dpos = torch.from_numpy(pos).cuda()
        dvel = torch.from_numpy(vel).cuda()
    with SPHSolver(prm) as a, SPHSolver(prm) as b:
        a.setParticles(pos, vel)
        b.setParticlesDevice(dpos, dvel, stream=stream)
        assert b.getNumParticles() == pos.shape[0]
        for x, y in zip(a.sortedState(), b.sortedState()):
            assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32))
        a.makeReady()
        b.makeReady()
        a.step(25)
        b.step(25)
        hp, hv = a.getState()
        out_p = torch.empty_like(dpos)
        out_v = torch.full_like(dvel, float("nan"))
        b.getStateDevice(out_p, out_v, stream=torch.cuda.current_stream())
        torch.cuda.current_stream().synchronize()
        assert np.array_equal(out_p.cpu().numpy().view(np.uint32), hp.view(np.uint32))
        assert np.array_equal(out_v.cpu().numpy().view(np.uint32), hv.view(np.uint32))


@pytest.mark.gpu
def test_device_upload_without_velocity_is_at_rest():
    torch = pytest.importorskip("torch")
    prm, pos, _ = _scene()
    dpos = torch.from_numpy(pos).cuda()
    torch.cuda.synchronize()
    with SPHSolver(prm) as s:
        s.setParticlesDevice(dpos)
        p, v = s.getState()
    assert np.array_equal(p, pos)
    assert not v.any()


@pytest.mark.gpu
def test_device_view_aliases_working_arrays():
    torch = pytest.importorskip("torch")
    prm, pos, vel = _scene()
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        s.makeReady()
        s.step(5)
        rho, p = s.computeDensity()
        spos, svel, ids, _ = s.sortedState()
        cs = s.cellStart()
        v = s.deviceState()
        n = v.n
        assert n == pos.shape[0] and v.ncells + 1 == cs.size
        pos4 = torch.as_tensor(_Cai(v.pos4, (n, 4)), device="cuda").cpu().numpy()
        vel4 = torch.as_tensor(_Cai(v.vel4, (n, 4)), device="cuda").cpu().numpy()
        drho = torch.as_tensor(_Cai(v.rho, (n,)), device="cuda").cpu().numpy()
        dpr = torch.as_tensor(_Cai(v.p_inv_rho, (n, 2)), device="cuda").cpu().numpy()
        dcs = torch.as_tensor(_Cai(v.cell_start, (v.ncells + 1,), typestr="<i4"), device="cuda").cpu().numpy()
    assert np.array_equal(pos4[:, :3], spos)
    assert np.array_equal(pos4[:, 3].view(np.uint32), ids)
    assert np.array_equal(vel4[:, :3], svel)
    assert np.array_equal(drho, rho)
    assert np.array_equal(dpr[:, 0], p)
    assert np.array_equal(dcs.view(np.uint32), cs)


@pytest.mark.gpu
def test_device_transfers_reject_host_memory():
    prm, pos, _ = _scene()
    host = np.ascontiguousarray(pos)
    fake = _Cai(host.ctypes.data, host.shape)
    with SPHSolver(prm) as s:
        with pytest.raises(C.SFError) as e:
            s.setParticlesDevice(fake)
        assert e.value.status == C.SF_ERR_INVALID_ARGUMENT
        s.setParticles(pos)
        with pytest.raises(C.SFError) as e:
            s.getStateDevice(fake)
        assert e.value.status == C.SF_ERR_INVALID_ARGUMENT
        # the state is untouched by the rejected calls
        assert np.array_equal(s.getParticles(), pos)


@pytest.mark.gpu
def test_device_upload_empty():
    prm, pos, _ = _scene()
    with SPHSolver(prm) as s:
        s.setParticles(pos)
        s.setParticlesDevice(_Cai(0, (0, 3)))
        assert s.getNumParticles() == 0


@pytest.mark.gpu
def test_pinned_host_upload_matches_pageable(lib):
    """Page-locked host arrays take the overlapped upload (velocities copied
    while positions are sorted); it must give the pageable path's state."""
    prm, pos, vel = _scene()
    n = pos.shape[0]
    nbytes = n * 12
    hp, hv = ctypes.c_void_p(), ctypes.c_void_p()
    C.check(lib.sf_host_alloc(nbytes, ctypes.byref(hp)))
    C.check(lib.sf_host_alloc(nbytes, ctypes.byref(hv)))
    try:
        P = np.ctypeslib.as_array((ctypes.c_float * (3 * n)).from_address(hp.value)).reshape(n, 3)
        V = np.ctypeslib.as_array((ctypes.c_float * (3 * n)).from_address(hv.value)).reshape(n, 3)
        P[:] = pos
        V[:] = vel
        with SPHSolver(prm) as a, SPHSolver(prm) as b:
            a.setParticles(pos, vel)
            C.check(lib.sf_set_state(b.handle, hp, hv, n))
            for x, y in zip(a.sortedState(), b.sortedState()):
                assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32))
            a.makeReady()
            b.makeReady()
            for _ in range(3):  # repeated round trips through the same pinned arrays
                a.step(10)
                b.step(10)
                pa, va = a.getState()
                C.check(lib.sf_get_state(b.handle, hp, hv, n))
                assert np.array_equal(P.view(np.uint32), pa.view(np.uint32))
                assert np.array_equal(V.view(np.uint32), va.view(np.uint32))
                a.setParticles(pa, va)
                C.check(lib.sf_set_state(b.handle, hp, hv, n))
    finally:
        lib.sf_host_free(hp)
        lib.sf_host_free(hv)


@pytest.mark.gpu
def test_pinned_upload_returns_before_its_sort_finishes(lib):
    """sf_set_state from page-locked arrays returns once the copies are done and
    leaves the sort queued.  What comes next must still see the sorted upload:
    an immediate page-locked read (stores split over two streams) returns the
    arrays unchanged, the caller may overwrite its arrays at once, and a larger
    upload (which reallocates the buffers the queued sort uses) gives the same
    state as a fresh context."""
    prm, pos, vel = _scene()
    n = pos.shape[0]
    hp, hv = ctypes.c_void_p(), ctypes.c_void_p()
    C.check(lib.sf_host_alloc(n * 12, ctypes.byref(hp)))
    C.check(lib.sf_host_alloc(n * 12, ctypes.byref(hv)))
    try:
        P = np.ctypeslib.as_array((ctypes.c_float * (3 * n)).from_address(hp.value)).reshape(n, 3)
        V = np.ctypeslib.as_array((ctypes.c_float * (3 * n)).from_address(hv.value)).reshape(n, 3)
        with SPHSolver(prm) as s:
            for _ in range(3):
                P[:] = pos
                V[:] = vel
                C.check(lib.sf_set_state(s.handle, hp, hv, n))
                P[:] = np.nan  # the upload has been read: overwriting is allowed
                V[:] = np.nan
                C.check(lib.sf_get_state(s.handle, hp, hv, n))
                assert np.array_equal(P.view(np.uint32), pos.view(np.uint32))
                assert np.array_equal(V.view(np.uint32), vel.view(np.uint32))
            P[:] = pos
            V[:] = vel
            C.check(lib.sf_set_state(s.handle, hp, hv, n))
            big_p = np.concatenate([pos, pos[: n // 2] * np.float32(0.5) + np.float32(0.25)])
            big_v = np.concatenate([vel, vel[: n // 2]])
            s.setParticles(big_p, big_v)  # grows the buffers right behind the queued sort
            s.makeReady()
            s.step(5)
            got = s.getState()
        with SPHSolver(prm) as f:
            f.setParticles(big_p, big_v)
            f.makeReady()
            f.step(5)
            ref = f.getState()
        for x, y in zip(got, ref):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    finally:
        lib.sf_host_free(hp)
        lib.sf_host_free(hv)


@pytest.mark.gpu
def test_pinned_download_after_each_kind_of_state_change(lib):
    """A page-locked sf_get_state (stores and copies split over two streams)
    gives the pageable read's bits after every kind of change of the state:
    steps, a parameter change that re-buckets the state, whole frames, a
    write through the device view and a forward/adjoint pair."""
    torch = pytest.importorskip("torch")
    prm, pos, vel = _scene()
    n = pos.shape[0]
    hp, hv = ctypes.c_void_p(), ctypes.c_void_p()
    C.check(lib.sf_host_alloc(n * 12, ctypes.byref(hp)))
    C.check(lib.sf_host_alloc(n * 12, ctypes.byref(hv)))
    try:
        P = np.ctypeslib.as_array((ctypes.c_float * (3 * n)).from_address(hp.value)).reshape(n, 3)
        V = np.ctypeslib.as_array((ctypes.c_float * (3 * n)).from_address(hv.value)).reshape(n, 3)

        def pinned_equals_pageable(s):
            P[:] = np.nan
            V[:] = np.nan
            C.check(lib.sf_get_state(s.handle, hp, hv, n))
            p2, v2 = s.getState()
            assert np.array_equal(P.view(np.uint32), p2.view(np.uint32))
            assert np.array_equal(V.view(np.uint32), v2.view(np.uint32))
            return p2

        with SPHSolver(prm) as s:
            s.setParticles(pos, vel)
            s.makeReady()
            for k in (1, 7):
                s.step(k)
                pinned_equals_pageable(s)
            s.setParams(params_16k(viscosity=0.02, kernelRadius=0.05))  # a new grid: the state is re-bucketed
            pinned_equals_pageable(s)
            s.step(3)
            s.advanceFrames(1, 2e-3, 40)
            pinned_equals_pageable(s)
            s.step(2)
            before = pinned_equals_pageable(s)
            v = s.deviceState()  # shift every x by 1e-3 through the view
            pos4 = torch.as_tensor(_Cai(v.pos4, (v.n, 4)), device="cuda")
            torch.cuda.synchronize()
            pos4[:, 0] += 1e-3
            torch.cuda.synchronize()
            after = pinned_equals_pageable(s)
            assert np.array_equal(after[:, 0], before[:, 0] + np.float32(1e-3))
            s.step(1)
            pinned_equals_pageable(s)
            s.forward(4, 2)
            pinned_equals_pageable(s)
            s.adjoint(np.ones((n, 3), np.float32))
            pinned_equals_pageable(s)
    finally:
        lib.sf_host_free(hp)
        lib.sf_host_free(hv)
