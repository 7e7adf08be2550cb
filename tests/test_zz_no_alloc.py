"""sf_density_noalloc: the allocation-free density entry point.

Some callers cannot allocate device memory while they run (an application or
plugin that owns a fixed device-memory budget, a real-time loop where an
allocation may block or fail).  For them the library offers one entry point
that computes density and pressure of caller-owned device positions with the
grid-sort scratch in a fixed static device array instead of cudaMalloc.

This file checks, through the C ABI, that two calls in a row (different inputs,
so the shared scratch is reused) give the same density and pressure as the
allocating entry point sf_compute_density, within the density tolerance of the
parity tests, and that requests beyond the fixed limits are refused.  It is
named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from helpers import params_16k, rel_err, normwise_err
from simplefluid_gb300 import SPHSolver, scene_positions
from simplefluid_gb300 import _capi as C

pytestmark = pytest.mark.gpu

DENSITY_RTOL = 1e-5
MAX_PARTICLES = 65536


def _existing(prm, pos):
    """Density and pressure from the allocating entry point, in caller order."""
    with SPHSolver(prm) as s:
        s.setParticles(pos)
        rho, prs = s.computeDensity()
        _, _, ids, _ = s.sortedState()
    out_rho = np.empty_like(rho)
    out_p = np.empty_like(prs)
    out_rho[ids] = rho
    out_p[ids] = prs
    return out_rho, out_p


def _noalloc(lib, torch, prm, pos):
    n = pos.shape[0]
    d_pos = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).cuda()
    d_rho = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
    d_p = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    cp = prm.to_c()
    C.check(lib.sf_density_noalloc(ctypes.byref(cp), ctypes.c_void_p(d_pos.data_ptr()), n,
                                   ctypes.c_void_p(d_rho.data_ptr()), ctypes.c_void_p(d_p.data_ptr()), None))
    torch.cuda.synchronize()
    return d_rho.cpu().numpy(), d_p.cpu().numpy()


def _inputs():
    prm = params_16k()
    a = scene_positions(prm, C.SF_SCENE_DAMBREAK_16K)
    rng = np.random.default_rng(21)
    a = (a + rng.uniform(-0.003, 0.003, size=a.shape)).astype(np.float32)
    b = (0.3 + rng.uniform(0.0, 0.25, size=(9000, 3))).astype(np.float32)
    return prm, a, b


def test_noalloc_matches_allocating_entry_point_two_calls(lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    prm, a, b = _inputs()
    rho_a, p_a = _noalloc(lib, torch, prm, a)   # first call
    rho_b, p_b = _noalloc(lib, torch, prm, b)   # second call reuses the scratch
    ref_a = _existing(prm, a)
    ref_b = _existing(prm, b)
    for (rho, prs), (rrho, rprs) in (((rho_a, p_a), ref_a), ((rho_b, p_b), ref_b)):
        assert np.isfinite(rho).all()
        assert rel_err(rho, rrho) < DENSITY_RTOL
        assert normwise_err(prs, rprs) < DENSITY_RTOL
    # a third call on the first input reproduces the first call
    rho_a2, p_a2 = _noalloc(lib, torch, prm, a)
    assert np.array_equal(rho_a2.view(np.uint32), rho_a.view(np.uint32))
    assert np.array_equal(p_a2.view(np.uint32), p_a.view(np.uint32))


def test_noalloc_rejects_requests_beyond_the_scratch(lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    prm = params_16k()
    cp = prm.to_c()
    d = torch.zeros(16, dtype=torch.float32, device="cuda")
    ptr = ctypes.c_void_p(d.data_ptr())
    # too many particles: refused before any GPU work touches the buffers
    st = lib.sf_density_noalloc(ctypes.byref(cp), ptr, MAX_PARTICLES + 1, ptr, None, None)
    assert st == C.SF_ERR_CAPACITY and b"65536" in lib.sf_last_error()
    # too many grid cells (h = 1/100 in the unit box: 10^6 cells)
    small_h = params_16k(kernelRadius=0.01, particleRadius=0.0025).to_c()
    st = lib.sf_density_noalloc(ctypes.byref(small_h), ptr, 4, ptr, None, None)
    assert st == C.SF_ERR_CAPACITY and b"262144" in lib.sf_last_error()


def test_noalloc_at_the_limits_on_a_caller_stream_without_allocating(lib):
    """Exactly 65,536 particles on a 64^3 = 262,144-cell grid, queued on the
    caller's own stream, with the library's allocation hook set to fail the
    next device allocation: the call still succeeds (it allocates nothing)
    and matches the allocating entry point."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    h = 0.031  # K = 2 cells per kernel radius: floor(2 / 0.031) = 64 cells per axis
    prm = params_16k(kernelRadius=h, particleRadius=h / 4)
    rng = np.random.default_rng(7)
    g = np.stack(np.meshgrid(np.arange(64), np.arange(32), np.arange(32), indexing="ij"), -1).reshape(-1, 3)
    sp = 2 * prm.particleRadius
    pos = (0.005 + g * sp + rng.uniform(-0.1, 0.1, size=g.shape) * sp).astype(np.float32)
    n = pos.shape[0]
    assert n == MAX_PARTICLES
    ref_rho, ref_p = _existing(prm, pos)
    d_pos = torch.from_numpy(pos).cuda()
    d_rho = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
    d_p = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    cp = prm.to_c()
    lib.sf_test_fail_allocation(0)
    try:
        with torch.cuda.stream(stream):
            st = lib.sf_density_noalloc(ctypes.byref(cp), ctypes.c_void_p(d_pos.data_ptr()), n,
                                        ctypes.c_void_p(d_rho.data_ptr()), ctypes.c_void_p(d_p.data_ptr()),
                                        ctypes.c_void_p(stream.cuda_stream))
    finally:
        lib.sf_test_fail_allocation(-1)
    assert st == C.SF_OK, lib.sf_last_error()
    stream.synchronize()
    rho, prs = d_rho.cpu().numpy(), d_p.cpu().numpy()
    assert np.isfinite(rho).all()
    assert rel_err(rho, ref_rho) < DENSITY_RTOL
    assert normwise_err(prs, ref_p) < DENSITY_RTOL
