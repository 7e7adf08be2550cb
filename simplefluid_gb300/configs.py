"""Workload configurations as JSON files (``simplefluid_gb300/workloads/*.json``).

The reference sets its parameters in the GUI (``Source/Controller.cpp:52-64``)
and has no file or command-line configuration; these files name the
workloads the solver is measured and tested on.  Each file holds:

* ``name`` (the file's stem), ``kind`` (``scene``, ``batch`` or ``adjoint``)
  and a ``description``;
* ``params`` (``scene`` and ``adjoint``) or ``base_params`` (``batch``): fields
  of ``SPHParameters`` by their reference names; ``scene`` is a scene name
  (the keys of ``SCENES``);
* the workload's ``seed`` and ``steps``, and per kind: ``scenes`` (batch);
  ``initial_velocity_sigma``, ``histogram_resolution`` and
  ``checkpoint_every`` (adjoint).

Unknown keys are errors, so a file cannot drift from what the loader reads.
"""
from __future__ import annotations

import dataclasses
import json
import os

from . import _capi as C
from .solver import SPHParameters

CONFIG_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "workloads")

SCENES = {
    "sphere_drop": C.SF_SCENE_SPHERE_DROP,
    "cube_drop": C.SF_SCENE_CUBE_DROP,
    "dambreak": C.SF_SCENE_DAMBREAK,
    "double_dambreak": C.SF_SCENE_DOUBLE_DAMBREAK,
    "dambreak_16k": C.SF_SCENE_DAMBREAK_16K,
    "double_dambreak_1m": C.SF_SCENE_DOUBLE_DAMBREAK_1M,
    "sphere_pool": C.SF_SCENE_SPHERE_POOL,
    "dambreak_64k": C.SF_SCENE_DAMBREAK_64K,
}

_COMMON = {"name", "kind", "description", "seed", "steps"}
_KEYS = {
    "scene": _COMMON | {"params"},
    "batch": _COMMON | {"base_params", "scenes"},
    "adjoint": _COMMON | {"params", "initial_velocity_sigma", "histogram_resolution", "checkpoint_every"},
}
_PARAM_FIELDS = {f.name for f in dataclasses.fields(SPHParameters)}


def available(kind: str | None = None) -> list[str]:
    """Names of the configuration files (optionally of one kind), sorted."""
    names = sorted(f[:-5] for f in os.listdir(CONFIG_DIR) if f.endswith(".json"))
    return [n for n in names if kind is None or load(n)["kind"] == kind]


def load(name: str) -> dict:
    """The configuration `name`, checked: known kind, known keys, known
    parameter fields and scene name; raises ValueError otherwise."""
    path = os.path.join(CONFIG_DIR, name + ".json")
    if not os.path.isfile(path):
        raise ValueError(f"no workload configuration {name!r} (have {available()})")
    with open(path) as f:
        cfg = json.load(f)
    kind = cfg.get("kind")
    if kind not in _KEYS:
        raise ValueError(f"{name}: kind must be one of {sorted(_KEYS)}, not {kind!r}")
    if cfg.get("name") != name:
        raise ValueError(f"{name}: the name field must be the file's stem")
    extra = set(cfg) - _KEYS[kind]
    if extra:
        raise ValueError(f"{name}: unknown keys {sorted(extra)}")
    pkey = "base_params" if kind == "batch" else "params"
    if pkey not in cfg:
        raise ValueError(f"{name}: missing {pkey}")
    bad = set(cfg[pkey]) - _PARAM_FIELDS
    if bad:
        raise ValueError(f"{name}: unknown SPHParameters fields {sorted(bad)}")
    scene = cfg[pkey].get("scene")
    if scene is not None and scene not in SCENES:
        raise ValueError(f"{name}: unknown scene {scene!r} (have {sorted(SCENES)})")
    return cfg


def params(name_or_cfg) -> SPHParameters:
    """SPHParameters of a configuration (its params, or a batch's base_params)."""
    cfg = load(name_or_cfg) if isinstance(name_or_cfg, str) else name_or_cfg
    fields = dict(cfg["base_params"] if cfg["kind"] == "batch" else cfg["params"])
    if "scene" in fields:
        fields["scene"] = SCENES[fields["scene"]]
    for key in ("gravity", "boxMin", "boxMax"):
        if key in fields:
            fields[key] = tuple(fields[key])
    return SPHParameters(**fields)
