"""Shared helpers of the test suite (parameter sets matching the workloads)."""
from __future__ import annotations

import numpy as np

from simplefluid_gb300 import SPHParameters
from simplefluid_gb300 import _capi as C


def params_16k(**kw) -> SPHParameters:
    """16,000-particle dambreak: r=0.01, h=0.04, box [0,1]^3."""
    base = dict(particleRadius=0.01, kernelRadius=0.04, pressureStiffness=50.0, viscosity=0.01,
                restDensity=1000.0, timeStep=1e-4, boundaryRestitution=0.1, scene=C.SF_SCENE_DAMBREAK_16K)
    base.update(kw)
    return SPHParameters(**base)


def params_1m(**kw) -> SPHParameters:
    """1,048,576-particle double dambreak: r=0.0025, h=4r."""
    base = dict(particleRadius=0.0025, kernelRadius=0.01, pressureStiffness=50.0, viscosity=0.01,
                restDensity=1000.0, timeStep=1e-4, boundaryRestitution=0.1, scene=C.SF_SCENE_DOUBLE_DAMBREAK_1M)
    base.update(kw)
    return SPHParameters(**base)


def params_reference_box(resolution: int = 32, **kw) -> SPHParameters:
    """The reference GUI's setting: box [-1,1]^3, kernelRadius = 2/resolution,
    particleRadius = kernelRadius / 4."""
    h = 2.0 / resolution
    base = dict(particleRadius=h / 4, kernelRadius=h, boxMin=(-1.0, -1.0, -1.0), boxMax=(1.0, 1.0, 1.0))
    base.update(kw)
    return SPHParameters(**base)


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-30)))


def normwise_err(a: np.ndarray, b: np.ndarray) -> float:
    """max |a - b| / max |b| over the whole field."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))
