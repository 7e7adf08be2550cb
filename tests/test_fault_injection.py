"""Allocation failures injected on the host (sf_test_fail_allocation).

The hook makes the k-th device allocation from now fail as out of memory, for
every k that the API sequence below reaches.  The sequence is: create,
upload, step, check, forward with checkpoints, loss, adjoint and render.
Each time:
  * the call that hits the failure returns SF_ERR_OUT_OF_MEMORY;
  * no later call runs a kernel on a released buffer;
  * the context stays usable: after disarming the hook, a new upload and
    three steps give the clean run's bits.
The failure is a fake of the failing call, made on the host.  No kernel runs
on a missing buffer, so nothing here can fault the GPU.
"""
import ctypes
from ctypes import byref, c_double, c_float, c_void_p

import numpy as np
import pytest

from helpers import params_16k
from simplefluid_gb300 import _capi as C

pytestmark = pytest.mark.gpu

MAX_K = 120


def _vp(a):
    return None if a is None else a.ctypes.data_as(c_void_p)


def _scene():
    rng = np.random.default_rng(4)
    g = np.stack(np.meshgrid(*[np.arange(k) for k in (10, 12, 10)], indexing="ij"), -1).reshape(-1, 3)
    pos = (0.1 + 0.02 * g + rng.uniform(-0.004, 0.004, size=g.shape)).astype(np.float32)
    vel = rng.normal(scale=0.05, size=pos.shape).astype(np.float32)
    return params_16k(viscosity=1.0), pos, vel


def _sequence(lib, ctx, pos, vel):
    """The API calls in order; yields (name, status) until one fails."""
    n = pos.shape[0]
    target = np.full(8 ** 3, 1.0 / 8 ** 3, np.float32)
    dldx = np.zeros((n, 3), np.float32)
    dx0 = np.zeros((n, 3), np.float32)
    dv0 = np.zeros((n, 3), np.float32)
    L, dmu, dk = c_double(), c_float(), c_float()
    rp = C.sf_render_params()
    lib.sf_render_params_default(byref(rp))
    rp.width, rp.height = 64, 48
    rep = C.sf_state_report()
    calls = [
        ("set_state", lambda: lib.sf_set_state(ctx, _vp(pos), _vp(vel), n)),
        ("make_ready", lambda: lib.sf_make_ready(ctx)),
        ("step", lambda: lib.sf_step(ctx, 3)),
        ("check_state", lambda: lib.sf_check_state(ctx, byref(rep))),
        ("forward", lambda: lib.sf_forward(ctx, 6, 3)),
        ("loss", lambda: lib.sf_loss_histogram(ctx, _vp(target), 8, byref(L), _vp(dldx))),
        ("adjoint", lambda: lib.sf_adjoint(ctx, _vp(dldx), None, _vp(dx0), _vp(dv0), byref(dmu), byref(dk))),
        ("render", lambda: lib.sf_render(ctx, byref(rp), None, None, None)),
        ("synchronize", lambda: lib.sf_synchronize(ctx)),
    ]
    for name, call in calls:
        st = call()
        yield name, st
        if st != C.SF_OK:
            return


def _three_steps(lib, ctx, pos, vel):
    n = pos.shape[0]
    assert lib.sf_set_state(ctx, _vp(pos), _vp(vel), n) == C.SF_OK
    assert lib.sf_make_ready(ctx) == C.SF_OK
    assert lib.sf_step(ctx, 3) == C.SF_OK
    p = np.empty_like(pos)
    v = np.empty_like(vel)
    assert lib.sf_get_state(ctx, _vp(p), _vp(v), n) == C.SF_OK
    return p, v


def test_every_allocation_failure_is_reported_and_recoverable(lib):
    prm, pos, vel = _scene()
    cp = prm.to_c()
    lib.sf_test_fail_allocation(-1)
    ctx = c_void_p()
    assert lib.sf_create(byref(cp), byref(ctx)) == C.SF_OK
    clean_p, clean_v = _three_steps(lib, ctx, pos, vel)
    assert all(st == C.SF_OK for _, st in _sequence(lib, ctx, pos, vel))
    lib.sf_destroy(ctx)

    failures = {}
    try:
        for k in range(MAX_K):
            lib.sf_test_fail_allocation(k)
            ctx = c_void_p()
            st = lib.sf_create(byref(cp), byref(ctx))
            if st != C.SF_OK:
                assert st == C.SF_ERR_OUT_OF_MEMORY, lib.sf_last_error()
                assert not ctx.value
                failures[k] = "create"
                continue
            results = list(_sequence(lib, ctx, pos, vel))
            lib.sf_test_fail_allocation(-1)
            name, st = results[-1]
            if st == C.SF_OK:
                lib.sf_destroy(ctx)
                break  # the whole sequence allocated fewer than k + 1 times
            assert st == C.SF_ERR_OUT_OF_MEMORY, (k, name, st, lib.sf_last_error())
            failures[k] = name
            p, v = _three_steps(lib, ctx, pos, vel)
            assert np.array_equal(p.view(np.uint32), clean_p.view(np.uint32)), (k, name)
            assert np.array_equal(v.view(np.uint32), clean_v.view(np.uint32)), (k, name)
            lib.sf_destroy(ctx)
        else:
            pytest.fail(f"the sequence still allocated after {MAX_K} allocations")
    finally:
        lib.sf_test_fail_allocation(-1)
    # every stage that allocates was reached by some k
    assert {"create", "set_state", "check_state", "forward", "loss", "adjoint", "render"} <= set(failures.values())
