"""Several host threads at once: the C ABI's contract is one context per
thread at a time, separate contexts independent, and a per-thread last-error
message.  ctypes releases the GIL during each call, so the calls overlap."""
import ctypes
import threading

import numpy as np
import pytest

from helpers import params_16k
from simplefluid_gb300 import SPHSolver, scene_positions
from simplefluid_gb300 import _capi as C


def _run_threads(fns):
    """Run each function on its own thread; re-raise the first failure."""
    errors = [None] * len(fns)
    results = [None] * len(fns)

    def wrap(k):
        try:
            results[k] = fns[k]()
        except BaseException as e:  # noqa: BLE001 - re-raised on the main thread
            errors[k] = e

    threads = [threading.Thread(target=wrap, args=(k,)) for k in range(len(fns))]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
        assert not t.is_alive(), "a worker thread did not finish"
    for e in errors:
        if e is not None:
            raise e
    return results


def test_last_error_is_per_thread(lib):
    """Two threads fail different calls at the same time; each reads its own
    message afterwards."""
    barrier = threading.Barrier(2, timeout=30)

    def failing(field, value, expect):
        def fn():
            p = params_16k().to_c()
            setattr(p, field, value)
            st = lib.sf_params_update(ctypes.byref(p))
            barrier.wait()  # both calls have failed before either reads
            msg = lib.sf_last_error().decode()
            barrier.wait()
            return st, msg, expect
        return fn

    for _ in range(20):
        res = _run_threads([failing("viscosity", -1.0, "viscosity"),
                            failing("time_step", 0.0, "time_step")])
        for st, msg, expect in res:
            assert st == C.SF_ERR_INVALID_ARGUMENT and expect in msg, msg


def _scene(k):
    prm = params_16k(viscosity=0.005 * (k + 1), pressureStiffness=30.0 + 10 * k)
    pos = scene_positions(prm, C.SF_SCENE_DAMBREAK_16K)
    rng = np.random.default_rng(k)
    pos = (pos + rng.uniform(-0.002, 0.002, size=pos.shape)).astype(np.float32)
    vel = rng.normal(scale=0.3, size=pos.shape).astype(np.float32)
    return prm, pos, vel


def _cycle_run(k):
    """Three upload / step / download cycles of scene k on one context."""
    prm, pos, vel = _scene(k)
    with SPHSolver(prm) as s:
        for _ in range(3):
            s.setParticles(pos, vel)
            s.makeReady()
            s.step(20)
            pos, vel = s.getState()
    return pos, vel


@pytest.mark.gpu
def test_contexts_on_separate_host_threads_match_serial_runs():
    """Four contexts, each created, stepped and read on its own host thread at
    the same time, give the bits of the same runs done one after another."""
    serial = [_cycle_run(k) for k in range(4)]
    for _ in range(2):
        threaded = _run_threads([lambda k=k: _cycle_run(k) for k in range(4)])
        for (sp, sv), (tp, tv) in zip(serial, threaded):
            assert np.array_equal(sp.view(np.uint32), tp.view(np.uint32))
            assert np.array_equal(sv.view(np.uint32), tv.view(np.uint32))
