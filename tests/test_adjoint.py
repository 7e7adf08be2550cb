"""The oracle's hand-written adjoint against central finite differences (FP64,
CPU only), and its invariance to the checkpoint interval."""
import numpy as np
import pytest

from simplefluid_gb300 import SPHParameters


def small_case(seed=0, shape=(10, 12, 10)):
    prm = SPHParameters(particleRadius=0.01, kernelRadius=0.04, viscosity=0.01, pressureStiffness=50.0)
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(k) for k in shape], indexing="ij"), -1).reshape(-1, 3)
    pos = 0.1 + g * 0.02 + rng.uniform(-0.002, 0.002, size=g.shape)
    vel = rng.normal(scale=0.2, size=pos.shape)
    res = 32
    target = rng.uniform(size=res ** 3)
    target /= target.sum()
    return prm, pos, vel, target


def _params(prm, mu=None, k=None):
    p = prm.to_c()
    if mu is not None:
        p.viscosity = mu
    if k is not None:
        p.pressure_stiffness = k
    return p


def test_oracle_adjoint_matches_central_differences(oracle):
    prm, pos, vel, target = small_case()
    steps, ck = 20, 5
    L0, gx, gv, gm, gk, _ = oracle.grad(_params(prm), pos, vel, steps, target, ckpt=ck)
    assert L0 > 0
    rng = np.random.default_rng(1)
    eps = 1e-5
    dv = rng.normal(size=vel.shape)
    fd = (oracle.grad(_params(prm), pos, vel + eps * dv, steps, target, ckpt=ck)[0]
          - oracle.grad(_params(prm), pos, vel - eps * dv, steps, target, ckpt=ck)[0]) / (2 * eps)
    assert fd == pytest.approx((gv * dv).sum(), rel=1e-4)
    dx = rng.normal(size=pos.shape) * 1e-3
    fd = (oracle.grad(_params(prm), pos + eps * dx, vel, steps, target, ckpt=ck)[0]
          - oracle.grad(_params(prm), pos - eps * dx, vel, steps, target, ckpt=ck)[0]) / (2 * eps)
    assert fd == pytest.approx((gx * dx).sum(), rel=1e-4)
    e = 1e-4
    fd = (oracle.grad(_params(prm, k=50 * (1 + e)), pos, vel, steps, target, ckpt=ck)[0]
          - oracle.grad(_params(prm, k=50 * (1 - e)), pos, vel, steps, target, ckpt=ck)[0]) / (2 * 50 * e)
    assert fd == pytest.approx(gk, rel=1e-3)
    fd = (oracle.grad(_params(prm, mu=0.01 * (1 + e)), pos, vel, steps, target, ckpt=ck)[0]
          - oracle.grad(_params(prm, mu=0.01 * (1 - e)), pos, vel, steps, target, ckpt=ck)[0]) / (2 * 0.01 * e)
    assert fd == pytest.approx(gm, rel=1e-2)


def test_oracle_adjoint_independent_of_checkpoint_interval(oracle):
    prm, pos, vel, target = small_case(seed=3)
    a = oracle.grad(_params(prm), pos, vel, 12, target, ckpt=1)
    b = oracle.grad(_params(prm), pos, vel, 12, target, ckpt=5)
    c = oracle.grad(_params(prm), pos, vel, 12, target, ckpt=12)
    for x, y in ((a, b), (a, c)):
        assert x[0] == y[0] and x[3] == y[3] and x[4] == y[4]
        assert np.array_equal(x[1], y[1]) and np.array_equal(x[2], y[2])


def test_oracle_seeded_adjoint_equals_loss_adjoint(oracle):
    """Seeding the adjoint with dL/dx of the final state reproduces grad()."""
    prm, pos, vel, target = small_case(seed=4)
    L, gx, gv, gm, gk, pf = oracle.grad(_params(prm), pos, vel, 8, target, ckpt=4)
    _, seed = oracle.loss(_params(prm), pf, target)
    ax, av, am, ak, _ = oracle.adjoint(_params(prm), pos, vel, 8, seed, ckpt=4)
    # the histogram sums particles in caller order here and in sorted order
    # inside grad(): equal up to double rounding
    assert np.allclose(ax, gx, rtol=1e-9, atol=1e-18) and np.allclose(av, gv, rtol=1e-9, atol=1e-18)
    assert am == pytest.approx(gm, rel=1e-9) and ak == pytest.approx(gk, rel=1e-9)


def test_oracle_loss_gradient_matches_differences(oracle):
    prm, pos, vel, target = small_case(seed=5)
    L, g = oracle.loss(_params(prm), pos, target)
    rng = np.random.default_rng(2)
    d = rng.normal(size=pos.shape) * 1e-3
    eps = 1e-6
    fd = (oracle.loss(_params(prm), pos + eps * d, target)[0] - oracle.loss(_params(prm), pos - eps * d, target)[0]) / (2 * eps)
    assert fd == pytest.approx((g * d).sum(), rel=1e-6)
