"""SimpleFluid SPH step on one GB300 (sm_103a), behind the reference's solver interface.

The compute lives in the in-tree CUDA library ``_lib/libsimplefluid_gb300.so``
(C ABI: include/sf_capi.h); this package is the host-side mirror of the
reference's ``SPHParameters`` / ``SPHSolver`` / ``SceneManager`` / ``Simulator``.
"""
from ._capi import SFError, load  # noqa: F401
from .sharding import assign_scenes, shard_batch  # noqa: F401
from .solver import (  # noqa: F401
    FRAME_TIME,
    SPHBatch,
    batch_cubes,
    read_state_file,
    render_params,
    save_ppm,
    SceneManager,
    Simulator,
    SPHParameters,
    SPHSolver,
    scene_positions,
    substeps_per_frame,
)

__all__ = ["assign_scenes", "shard_batch", "render_params", "save_ppm", "read_state_file", "SPHBatch", "batch_cubes", "SFError", "SceneManager", "Simulator", "SPHParameters", "SPHSolver", "scene_positions",
           "substeps_per_frame", "FRAME_TIME", "load"]
