"""ctypes binding of the C ABI declared in include/sf_capi.h.

The shared library is built in-tree (``simplefluid_gb300/_lib``) by
``simplefluid_gb300.build``.  Loading fails loudly when it is missing: there is
no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int32, c_size_t, c_uint32, c_uint64, c_void_p

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libsimplefluid_gb300.so")
# the checked build (kernels count bad indices; build(checked=True)); the
# environment variable SIMPLEFLUID_GB300_CHECKED=1 makes it this process's library
CHECKED_LIB_PATH = os.path.join(LIB_DIR, "libsimplefluid_gb300_checked.so")
if os.environ.get("SIMPLEFLUID_GB300_CHECKED") == "1":
    LIB_PATH = CHECKED_LIB_PATH

SF_OK = 0
SF_ERR_INVALID_ARGUMENT = 1
SF_ERR_CUDA = 2
SF_ERR_OUT_OF_MEMORY = 3
SF_ERR_NOT_READY = 4
SF_ERR_GRID_TOO_LARGE = 5
SF_ERR_CAPACITY = 6
SF_ERR_NO_DEVICE = 7

SF_SCENE_SPHERE_DROP = 0
SF_SCENE_CUBE_DROP = 1
SF_SCENE_DAMBREAK = 2
SF_SCENE_DOUBLE_DAMBREAK = 3
SF_SCENE_DAMBREAK_16K = 16
SF_SCENE_DOUBLE_DAMBREAK_1M = 17
SF_SCENE_SPHERE_POOL = 18
SF_SCENE_DAMBREAK_64K = 19

SF_EOS_LINEAR = 0
SF_EOS_TAIT = 1


class sf_params(ctypes.Structure):
    """Mirror of ``struct sf_params`` (include/sf_capi.h)."""

    _fields_ = [
        ("num_threads", c_int32),
        ("kernel_radius", c_float),
        ("particle_radius", c_float),
        ("pressure_stiffness", c_float),
        ("boundary_restitution", c_float),
        ("viscosity", c_float),
        ("stop_time", c_float),
        ("use_attractive_pressure", c_int32),
        ("scene", c_int32),
        ("rest_density", c_float),
        ("gravity", c_float * 3),
        ("time_step", c_float),
        ("box_min", c_float * 3),
        ("box_max", c_float * 3),
        ("eos", c_int32),
        ("cells_per_h", c_int32),
        ("adaptive_time_step", c_int32),
        ("reserved", c_int32 * 1),
    ]


SF_LIST_NONE = 0
SF_LIST_TILE_STAGED = 1
SF_LIST_TILE = 2
SF_LIST_TILE16 = 3


class sf_tuning(ctypes.Structure):
    """Mirror of ``struct sf_tuning`` (include/sf_capi.h)."""

    _fields_ = [("list_mode", c_int32), ("density_block", c_int32), ("force_block", c_int32),
                ("prefetch", c_int32), ("l2_window", c_int32), ("batch_cluster", c_int32),
                ("batch_block", c_int32), ("reserved", c_int32 * 1)]


SF_COLOR_UNIFORM = 0
SF_COLOR_RANDOM = 1
SF_COLOR_RAMP = 2


class sf_render_params(ctypes.Structure):
    """Mirror of ``struct sf_render_params`` (include/sf_capi.h)."""

    _fields_ = [
        ("width", c_int32), ("height", c_int32),
        ("eye", c_float * 3), ("focus", c_float * 3), ("up", c_float * 3),
        ("fovy_deg", c_float), ("znear", c_float), ("zfar", c_float),
        ("point_radius", c_float),
        ("num_lights", c_int32),
        ("light_position", (c_float * 4) * 8), ("light_ambient", (c_float * 4) * 8),
        ("light_diffuse", (c_float * 4) * 8), ("light_specular", (c_float * 4) * 8),
        ("mat_ambient", c_float * 4), ("mat_diffuse", c_float * 4), ("mat_specular", c_float * 4),
        ("mat_shininess", c_float),
        ("color_mode", c_int32),
        ("color_seed", c_uint64),
        ("background", c_float * 4),
        ("reserved", c_int32 * 4),
    ]


class sf_device_view(ctypes.Structure):
    """Mirror of ``struct sf_device_view`` (include/sf_capi.h)."""

    _fields_ = [("pos4", c_void_p), ("vel4", c_void_p), ("rho", c_void_p), ("p_inv_rho", c_void_p),
                ("cell_start", c_void_p), ("n", c_uint32), ("ncells", c_uint32), ("stream", c_void_p)]


class sf_state_report(ctypes.Structure):
    """Mirror of ``struct sf_state_report`` (include/sf_capi.h)."""

    _fields_ = [("n", c_uint32), ("non_finite", c_uint32), ("outside_box", c_uint32), ("unsorted", c_uint32),
                ("cell_table_mismatch", c_uint32), ("bad_ids", c_uint32), ("list_overflow", c_uint32),
                ("max_speed", c_float)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class SFError(RuntimeError):
    """Raised when a C-ABI call returns a non-zero sf_status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"sf_status {status}: {message}")
        self.status = status


_P = POINTER
# name -> (restype, argtypes)
PROTOTYPES = {
    "sf_last_error": (c_char_p, []),
    "sf_version": (c_char_p, []),
    "sf_params_default": (c_int32, [_P(sf_params)]),
    "sf_params_update": (c_int32, [_P(sf_params)]),
    "sf_scene_count": (c_int32, [_P(sf_params), c_int32, c_uint64, _P(c_uint32)]),
    "sf_setup_scene": (c_int32, [_P(sf_params), c_int32, c_uint64, c_void_p, c_void_p, c_uint32, _P(c_uint32)]),
    "sf_select_device": (c_int32, [c_int32]),
    "sf_create": (c_int32, [_P(sf_params), _P(c_void_p)]),
    "sf_destroy": (c_int32, [c_void_p]),
    "sf_set_params": (c_int32, [c_void_p, _P(sf_params)]),
    "sf_get_params": (c_int32, [c_void_p, _P(sf_params)]),
    "sf_set_state": (c_int32, [c_void_p, c_void_p, c_void_p, c_uint32]),
    "sf_get_state": (c_int32, [c_void_p, c_void_p, c_void_p, c_uint32]),
    "sf_set_state_device": (c_int32, [c_void_p, c_void_p, c_void_p, c_uint32, c_void_p]),
    "sf_get_state_device": (c_int32, [c_void_p, c_void_p, c_void_p, c_uint32, c_void_p]),
    "sf_device_state": (c_int32, [c_void_p, _P(sf_device_view)]),
    "sf_check_state": (c_int32, [c_void_p, _P(sf_state_report)]),
    "sf_index_checks": (c_int32, [c_int32, _P(ctypes.c_uint64), _P(c_int32)]),
    "sf_test_fail_allocation": (c_int32, [ctypes.c_int64]),
    "sf_batch_check_state": (c_int32, [c_void_p, _P(sf_state_report)]),
    "sf_get_num_particles": (c_int32, [c_void_p, _P(c_uint32)]),
    "sf_make_ready": (c_int32, [c_void_p]),
    "sf_advance_frame": (c_int32, [c_void_p, _P(c_float)]),
    "sf_step": (c_int32, [c_void_p, c_uint32]),
    "sf_advance_frames": (c_int32, [c_void_p, c_uint32, c_double, c_uint32, _P(c_double), _P(c_uint32)]),
    "sf_synchronize": (c_int32, [c_void_p]),
    "sf_get_stream": (c_int32, [c_void_p, _P(c_void_p)]),
    "sf_host_alloc": (c_int32, [c_size_t, _P(c_void_p)]),
    "sf_host_free": (c_int32, [c_void_p]),
    "sf_get_grid": (c_int32, [c_void_p, c_void_p]),
    "sf_get_sorted": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_uint32]),
    "sf_get_cell_start": (c_int32, [c_void_p, c_void_p, c_uint32]),
    "sf_compute_density": (c_int32, [c_void_p, c_void_p, c_void_p, c_uint32]),
    "sf_compute_accel": (c_int32, [c_void_p, c_void_p, c_uint32]),
    "sf_neighbour_stats": (c_int32, [c_void_p, c_void_p, c_void_p, c_uint32]),
    "sf_step_timed": (c_int32, [c_void_p, c_uint32, c_uint64, _P(c_float), c_void_p]),
    "sf_stage_count": (c_uint32, []),
    "sf_stage_name": (c_char_p, [c_uint32]),
    "sf_profile_steps": (c_int32, [c_void_p, c_uint32, c_uint64, c_void_p, c_uint32]),
    "sf_adjoint_pass_count": (c_uint32, []),
    "sf_adjoint_pass_name": (c_char_p, [c_uint32]),
    "sf_adjoint_profile": (c_int32, [c_void_p, c_void_p, c_uint32, POINTER(c_uint32)]),
    "sf_get_tuning": (c_int32, [c_void_p, _P(sf_tuning)]),
    "sf_set_tuning": (c_int32, [c_void_p, _P(sf_tuning)]),
    "sf_render_params_default": (c_int32, [_P(sf_render_params)]),
    "sf_render": (c_int32, [c_void_p, _P(sf_render_params), c_void_p, c_void_p, c_void_p]),
    "sf_save_state": (c_int32, [c_void_p, c_char_p, c_double]),
    "sf_load_state": (c_int32, [c_void_p, c_char_p, _P(c_double)]),
    "sf_forward": (c_int32, [c_void_p, c_uint32, c_uint32]),
    "sf_adjoint": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, _P(c_float), _P(c_float)]),
    "sf_loss_histogram": (c_int32, [c_void_p, c_void_p, c_uint32, _P(c_double), c_void_p]),
    "sf_batch_cubes": (c_int32, [c_uint64, c_uint32, _P(sf_params), c_void_p, c_void_p, c_void_p, c_uint64,
                                 _P(c_uint64)]),
    "sf_batch_create": (c_int32, [c_void_p, c_uint32, _P(c_void_p)]),
    "sf_batch_destroy": (c_int32, [c_void_p]),
    "sf_batch_num_scenes": (c_int32, [c_void_p, _P(c_uint32)]),
    "sf_batch_get_params": (c_int32, [c_void_p, c_uint32, _P(sf_params)]),
    "sf_batch_set_state": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "sf_batch_get_state": (c_int32, [c_void_p, c_void_p, c_void_p, c_uint32]),
    "sf_batch_num_particles": (c_int32, [c_void_p, _P(c_uint32)]),
    "sf_batch_step": (c_int32, [c_void_p, c_uint32]),
    "sf_batch_synchronize": (c_int32, [c_void_p]),
    "sf_batch_step_timed": (c_int32, [c_void_p, c_uint32, c_uint64, _P(c_float), c_void_p]),
    "sf_batch_get_tuning": (c_int32, [c_void_p, _P(sf_tuning)]),
    "sf_batch_set_tuning": (c_int32, [c_void_p, _P(sf_tuning)]),
    "sf_batch_set_cells_per_h": (c_int32, [c_void_p, c_int32]),
    "sf_batch_autotune": (c_int32, [c_void_p, c_uint32, _P(sf_tuning), _P(c_int32), _P(c_float)]),
    "sf_density_noalloc": (c_int32, [_P(sf_params), c_void_p, c_uint32, c_void_p, c_void_p, c_void_p]),
}

_lib = None


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the in-tree C-ABI library; raise if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"SimpleFluid GB300 library not built: {p} is missing "
            "(run `python -c 'import __graft_entry__ as g; g.build()'`)")
    lib = ctypes.CDLL(p)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def index_checks(reset: bool = False) -> tuple:
    """(bad indices counted on the current device, whether this library is the
    checked build); `reset` clears the count (sf_index_checks)."""
    lib = load()
    failures, compiled = ctypes.c_uint64(), c_int32()
    check(lib.sf_index_checks(1 if reset else 0, ctypes.byref(failures), ctypes.byref(compiled)))
    return int(failures.value), bool(compiled.value)


def check(status: int) -> None:
    if status != SF_OK:
        msg = load().sf_last_error()
        raise SFError(status, msg.decode() if msg else "")
