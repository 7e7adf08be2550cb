"""GPU adjoint (sf_forward / sf_adjoint / sf_loss_histogram) against the
oracle's FP32 and FP64 adjoints and central finite differences; the
torch.autograd.Function wrapper lives here, in the test harness only."""
import numpy as np
import pytest

from helpers import normwise_err
from simplefluid_gb300 import SPHParameters, SPHSolver, scene_positions
from simplefluid_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def case(seed=0, shape=(12, 16, 12)):
    prm = SPHParameters(particleRadius=0.01, kernelRadius=0.04, viscosity=0.01, pressureStiffness=50.0)
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(k) for k in shape], indexing="ij"), -1).reshape(-1, 3)
    pos = (0.1 + g * 0.02 + rng.uniform(-0.002, 0.002, size=g.shape)).astype(np.float32)
    vel = rng.normal(scale=0.2, size=pos.shape).astype(np.float32)
    res = 32
    target = rng.uniform(size=res ** 3)
    target = (target / target.sum()).astype(np.float32)
    return prm, pos, vel, target


def gpu_grad(prm, pos, vel, target, steps, ckpt):
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        s.forward(steps, ckpt)
        before = s.getState()
        L, dldx = s.lossHistogram(target)
        dx0, dv0, dmu, dk = s.adjoint(dldx)
        after = s.getState()
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    return L, dldx, dx0, dv0, dmu, dk, before[0]


def test_loss_histogram_matches_oracle(oracle):
    prm, pos, vel, target = case(seed=1)
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        L, g = s.lossHistogram(target)
    Lo, go = oracle.loss(prm.to_c(), pos.astype(np.float64), target.astype(np.float64))
    assert L == pytest.approx(Lo, rel=1e-6)
    assert normwise_err(g, go) < 1e-5


def test_adjoint_matches_fp32_oracle_op_for_op(oracle):
    """Given the same final-state adjoint, the GPU adjoint performs the oracle's
    FP32 operations in the same order: identical vectors, scalars to the
    rounding of the block-ordered double reduction."""
    prm, pos, vel, target = case(seed=2)
    steps, ck = 24, 8
    L, dldx, dx0, dv0, dmu, dk, pf = gpu_grad(prm, pos, vel, target, steps, ck)
    ox, ov, om, ok, opf = oracle.adjoint(prm.to_c(), pos, vel, steps, dldx, ckpt=ck, dtype=np.float32)
    assert np.array_equal(pf.view(np.uint32), opf.view(np.uint32))
    assert np.array_equal(dv0.view(np.uint32), ov.view(np.uint32))
    assert np.array_equal(dx0.view(np.uint32), ox.view(np.uint32))
    assert dmu == pytest.approx(om, rel=1e-5, abs=1e-30)
    assert dk == pytest.approx(ok, rel=1e-5, abs=1e-30)


def test_adjoint_tracks_fp64_oracle(oracle):
    """FP32 GPU adjoint against the FP64 CPU adjoint of the same loss."""
    prm, pos, vel, target = case(seed=3)
    steps, ck = 30, 10
    L, dldx, dx0, dv0, dmu, dk, pf = gpu_grad(prm, pos, vel, target, steps, ck)
    Lo, ox, ov, om, ok, _ = oracle.grad(prm.to_c(), pos, vel, steps, target.astype(np.float64), ckpt=ck)
    assert L == pytest.approx(Lo, rel=1e-4)
    assert normwise_err(dv0, ov) < 1e-3
    assert normwise_err(dx0, ox) < 1e-3
    assert dmu == pytest.approx(om, rel=1e-3)
    assert dk == pytest.approx(ok, rel=1e-3)


def test_adjoint_independent_of_checkpoint_interval():
    prm, pos, vel, target = case(seed=4)
    a = gpu_grad(prm, pos, vel, target, 12, 1)
    b = gpu_grad(prm, pos, vel, target, 12, 5)
    c = gpu_grad(prm, pos, vel, target, 12, 12)
    for x, y in ((a, b), (a, c)):
        assert x[0] == y[0]
        for u, v in zip(x[1:4], y[1:4]):
            assert np.array_equal(u, v)
        assert x[4] == y[4] and x[5] == y[5]


def test_adjoint_rejects_missing_forward():
    prm, pos, vel, _ = case()
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        with pytest.raises(C.SFError) as e:
            s.adjoint(np.zeros_like(pos))
        assert e.value.status == C.SF_ERR_NOT_READY


# ---- torch.autograd.Function wrapper (test harness only) -------------------
torch = pytest.importorskip("torch")


class SPHRollout(torch.autograd.Function):
    """loss = histogram_loss(rollout(x0, v0; mu, k)) with the hand-written adjoint as backward."""

    @staticmethod
    def forward(ctx, v0, mu, k, pos0, target, steps, ckpt):
        prm = SPHParameters(particleRadius=0.01, kernelRadius=0.04, viscosity=float(mu), pressureStiffness=float(k))
        s = SPHSolver(prm)
        s.setParticles(pos0, v0.detach().cpu().numpy().astype(np.float32))
        s.forward(steps, ckpt)
        L, dldx = s.lossHistogram(target)
        ctx.solver, ctx.dldx = s, dldx
        return torch.tensor(L, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gL):
        dx0, dv0, dmu, dk = ctx.solver.adjoint(ctx.dldx)
        ctx.solver.close()
        g = float(gL)
        return (torch.from_numpy(dv0).double() * g, torch.tensor(dmu * g, dtype=torch.float64),
                torch.tensor(dk * g, dtype=torch.float64), None, None, None, None)


def test_autograd_wrapper_against_central_differences():
    """A viscous fluid (mu = 5) so that every parameter moves the FP32
    trajectory by many ulps within the finite-difference step."""
    prm, pos, vel, target = case(seed=5, shape=(10, 12, 10))
    steps, ck, mu0, k0 = 40, 10, 5.0, 50.0
    v0 = torch.tensor(vel, dtype=torch.float64, requires_grad=True)
    mu = torch.tensor(mu0, dtype=torch.float64, requires_grad=True)
    k = torch.tensor(k0, dtype=torch.float64, requires_grad=True)
    L = SPHRollout.apply(v0, mu, k, pos, target, steps, ck)
    L.backward()

    def loss_at(v, m, kk):
        with torch.no_grad():
            return float(SPHRollout.apply(torch.tensor(v, dtype=torch.float64), torch.tensor(m), torch.tensor(kk),
                                          pos, target, steps, ck))

    # Steps small enough that few particles cross a kink of the piecewise-
    # linear CIC weights, large enough to move the FP32 state by many ulps.
    rng = np.random.default_rng(6)
    d = rng.normal(size=vel.shape)
    eps = 2e-3
    fd = (loss_at(vel + eps * d, mu0, k0) - loss_at(vel - eps * d, mu0, k0)) / (2 * eps)
    assert fd == pytest.approx(float((v0.grad.numpy() * d).sum()), rel=1e-2)
    e = 5e-3
    fdk = (loss_at(vel, mu0, k0 * (1 + e)) - loss_at(vel, mu0, k0 * (1 - e))) / (2 * k0 * e)
    assert fdk == pytest.approx(float(k.grad), rel=2e-2)
    em = 3e-2  # the viscous signal is ~1e-7 of L: a wider step keeps it above FP32 rounding
    fdm = (loss_at(vel, mu0 * (1 + em), k0) - loss_at(vel, mu0 * (1 - em), k0)) / (2 * mu0 * em)
    assert fdm == pytest.approx(float(mu.grad), rel=2e-2)


def test_differentiable_dambreak_65k_200_steps(oracle):
    """The 65,536-particle differentiable dambreak (200 steps, checkpoints every
    20): GPU FP32 gradients track the FP64 CPU adjoint."""
    prm = SPHParameters(particleRadius=0.005, kernelRadius=0.02, scene=C.SF_SCENE_DAMBREAK_64K)
    pos = scene_positions(prm, C.SF_SCENE_DAMBREAK_64K)
    rng = np.random.default_rng(20171)
    vel = rng.normal(scale=0.05, size=pos.shape).astype(np.float32)
    res = 32
    target = rng.uniform(size=res ** 3)
    target = (target / target.sum()).astype(np.float32)
    L, dldx, dx0, dv0, dmu, dk, _ = gpu_grad(prm, pos, vel, target, 200, 20)
    Lo, ox, ov, om, ok, _ = oracle.grad(prm.to_c(), pos, vel, 200, target.astype(np.float64), ckpt=20)
    assert L == pytest.approx(Lo, rel=1e-3)
    assert normwise_err(dv0, ov) < 1e-2
    assert dmu == pytest.approx(om, rel=1e-2)
    assert dk == pytest.approx(ok, rel=1e-2)


def test_adjoint_profile_times_each_pass_and_leaves_gradients_reproducible():
    """sf_adjoint_profile needs a finished sf_adjoint, times the first
    segment's passes, and a following sf_adjoint returns the same bits."""
    import ctypes
    lib = C.load()
    prm, pos, vel, target = case(seed=4)
    npass = lib.sf_adjoint_pass_count()
    assert [lib.sf_adjoint_pass_name(p).decode() for p in range(npass)] == ["adj_integrate", "adj_forces",
                                                                             "adj_density"]
    ms = np.zeros(npass, np.float32)
    steps = ctypes.c_uint32()
    with SPHSolver(prm) as s:
        s.setParticles(pos, vel)
        assert lib.sf_adjoint_profile(s.handle, ms.ctypes.data_as(ctypes.c_void_p), npass,
                                      ctypes.byref(steps)) == C.SF_ERR_NOT_READY
        s.forward(20, 8)
        _, dldx = s.lossHistogram(target)
        first = s.adjoint(dldx)
        C.check(lib.sf_adjoint_profile(s.handle, ms.ctypes.data_as(ctypes.c_void_p), npass, ctypes.byref(steps)))
        assert steps.value == 8 and np.all(ms > 0)
        assert lib.sf_adjoint_profile(s.handle, ms.ctypes.data_as(ctypes.c_void_p), npass - 1,
                                      None) == C.SF_ERR_INVALID_ARGUMENT
        again = s.adjoint(dldx)
    for a, b in zip(first[:2], again[:2]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert first[2:] == again[2:]
