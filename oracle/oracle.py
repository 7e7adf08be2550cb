"""ctypes wrapper of the CPU oracle (oracle/sph_oracle.cpp) — TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use
it, as the checker.  The product package never imports this module.

Parity with the reference's solver library (Banana SPHSolver, absent from the
reference tree) is unpinned; the scene generators, the frame loop and the
particle shaders' arithmetic are pinned against the reference's own
Source/SceneManager.cpp, Source/Simulator.cpp and Shaders/particle.*.glsl
compiled by build_ref.sh.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_int, c_uint32, c_uint64, c_void_p

import numpy as np

from simplefluid_gb300._capi import sf_params

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "libsf_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_scenes.so")
REF_SIM_LIB = os.path.join(HERE, "_ref", "libref_sim.so")
REF_SHADER_LIB = os.path.join(HERE, "_ref", "libref_shader.so")
FRAME_TIME = 0.0333333333  # Source/Simulator.cpp:47

_lib = None
_ref = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(ORACLE_LIB):
        subprocess.check_call(["sh", os.path.join(HERE, "build_oracle.sh")])
    return ORACLE_LIB


def build_ref(ref_root: str | None = None) -> str | None:
    """Compile the reference's scene generator from the reference tree at
    `ref_root` (else $SF_REFERENCE_ROOT) into oracle/_ref.  Without a tree,
    an earlier build is used when present.  Returns the library path, or
    None when there is neither."""
    root = ref_root or os.environ.get("SF_REFERENCE_ROOT")
    if not root:
        return REF_LIB if os.path.exists(REF_LIB) else None
    try:
        subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), root],
                              stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    except (subprocess.CalledProcessError, OSError):
        return None
    return REF_LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_LIB):
            build()
        l = ctypes.CDLL(ORACLE_LIB)
        P = POINTER(sf_params)
        l.sfo_derive.argtypes = [P, c_void_p]
        l.sfo_scene.argtypes = [P, c_int, c_uint64, c_void_p, c_uint32, POINTER(c_uint32)]
        for sfx in ("f32", "f64"):
            getattr(l, f"sfo_sort_{sfx}").argtypes = [P, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
            getattr(l, f"sfo_density_{sfx}").argtypes = [P, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p]
            getattr(l, f"sfo_accel_{sfx}").argtypes = [P, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
            getattr(l, f"sfo_integrate_{sfx}").argtypes = [P, c_uint32, c_void_p, c_void_p, c_void_p]
            getattr(l, f"sfo_neighbour_stats_{sfx}").argtypes = [P, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p]
            getattr(l, f"sfo_step_{sfx}").argtypes = [P, c_uint32, c_void_p, c_void_p, c_void_p, c_uint32, c_int]
        for sfx in ("f32", "f64"):
            getattr(l, f"sfo_grad_{sfx}").argtypes = [P, c_uint32, c_void_p, c_void_p, c_uint32, c_uint32, c_void_p,
                                                      c_uint32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                                      c_void_p, c_int]
            getattr(l, f"sfo_adjoint_{sfx}").argtypes = [P, c_uint32, c_void_p, c_void_p, c_uint32, c_uint32,
                                                         c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                                         c_void_p, c_int]
            getattr(l, f"sfo_loss_{sfx}").argtypes = [P, c_uint32, c_void_p, c_void_p, c_uint32, c_void_p, c_void_p,
                                                      c_void_p]
        l.sfo_render.argtypes = [P, c_void_p, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p]
        l.sfo_render_camera.argtypes = [P, c_void_p, c_void_p, c_void_p, POINTER(ctypes.c_float),
                                        POINTER(ctypes.c_float)]
        l.sfo_particle_vertex.argtypes = [P, c_void_p, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p]
        l.sfo_particle_fragment.argtypes = [P, c_void_p, c_uint32, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]
        l.sfo_frames_f32.argtypes = [P, c_uint32, c_void_p, c_void_p, c_void_p, c_uint32, ctypes.c_double, c_uint32,
                                     c_int, POINTER(ctypes.c_double), POINTER(c_uint32), c_void_p, c_uint32]
        l.sfo_max_threads.argtypes = []
        l.sfo_frame_accounting.argtypes = [c_void_p, c_uint32, ctypes.c_double, ctypes.c_float, c_uint32, c_void_p,
                                           c_void_p, POINTER(c_uint32)]
        _lib = l
    return _lib


def ref_lib() -> ctypes.CDLL | None:
    global _ref
    if _ref is None and os.path.exists(REF_LIB):
        r = ctypes.CDLL(REF_LIB)
        r.ref_setup_scene.argtypes = [c_int, ctypes.c_float, c_void_p, c_uint32, POINTER(c_uint32)]
        _ref = r
    return _ref


def _ptr(a):
    return None if a is None else a.ctypes.data_as(c_void_p)


def _chk(st: int, what: str) -> None:
    if st != 0:
        raise RuntimeError(f"oracle {what} failed with status {st}")


def derive(p: sf_params) -> dict:
    out = np.zeros(16, np.float64)
    _chk(lib().sfo_derive(ctypes.byref(p), _ptr(out)), "derive")
    keys = ["h", "h2", "mass", "cd", "cp", "cv", "lo0", "lo1", "lo2", "hi0", "hi1", "hi2", "nx", "ny", "nz", "ncells"]
    return dict(zip(keys, out.tolist()))


def scene(p: sf_params, scene_id: int, seed: int = 20171) -> np.ndarray:
    n = c_uint32(0)
    _chk(lib().sfo_scene(ctypes.byref(p), scene_id, seed, None, 0, ctypes.byref(n)), "scene count")
    out = np.zeros((n.value, 3), np.float32)
    _chk(lib().sfo_scene(ctypes.byref(p), scene_id, seed, _ptr(out), n.value, ctypes.byref(n)), "scene")
    return out


def ref_scene(scene_id: int, particle_radius: float) -> np.ndarray | None:
    """Positions from the reference's own SceneManager (None if not built)."""
    r = ref_lib()
    if r is None:
        return None
    n = c_uint32(0)
    _chk(r.ref_setup_scene(scene_id, particle_radius, None, 0, ctypes.byref(n)), "ref scene count")
    out = np.zeros((n.value, 3), np.float32)
    _chk(r.ref_setup_scene(scene_id, particle_radius, _ptr(out), n.value, ctypes.byref(n)), "ref scene")
    return out


class State:
    """Particle state in the oracle's current (sorted-after-step) order."""

    def __init__(self, pos, vel=None, dtype=np.float32):
        self.dtype = np.dtype(dtype)
        self.pos = np.ascontiguousarray(pos, dtype=self.dtype).reshape(-1, 3).copy()
        n = self.pos.shape[0]
        self.vel = (np.zeros((n, 3), self.dtype) if vel is None
                    else np.ascontiguousarray(vel, dtype=self.dtype).reshape(-1, 3).copy())
        self.ids = np.arange(n, dtype=np.uint32)

    @property
    def n(self) -> int:
        return self.pos.shape[0]

    @property
    def sfx(self) -> str:
        return "f32" if self.dtype == np.float32 else "f64"

    def sort(self, p: sf_params, want_cells: bool = False):
        d = derive(p)
        keys = np.zeros(self.n, np.uint32)
        cs = np.zeros(int(d["ncells"]) + 1, np.uint32) if want_cells else None
        _chk(getattr(lib(), f"sfo_sort_{self.sfx}")(ctypes.byref(p), self.n, _ptr(self.pos), _ptr(self.vel),
                                                    _ptr(self.ids), _ptr(keys), _ptr(cs)), "sort")
        return keys, cs

    def density(self, p: sf_params):
        rho = np.zeros(self.n, self.dtype)
        prs = np.zeros(self.n, self.dtype)
        inv = np.zeros(self.n, self.dtype)
        _chk(getattr(lib(), f"sfo_density_{self.sfx}")(ctypes.byref(p), self.n, _ptr(self.pos), _ptr(rho),
                                                       _ptr(prs), _ptr(inv)), "density")
        return rho, prs, inv

    def accel(self, p: sf_params, prs=None, inv=None):
        if prs is None:
            _, prs, inv = self.density(p)
        acc = np.zeros((self.n, 3), self.dtype)
        _chk(getattr(lib(), f"sfo_accel_{self.sfx}")(ctypes.byref(p), self.n, _ptr(self.pos), _ptr(self.vel),
                                                     _ptr(prs), _ptr(inv), _ptr(acc)), "accel")
        return acc

    def integrate(self, p: sf_params, acc):
        acc = np.ascontiguousarray(acc, self.dtype)
        _chk(getattr(lib(), f"sfo_integrate_{self.sfx}")(ctypes.byref(p), self.n, _ptr(self.pos), _ptr(self.vel),
                                                         _ptr(acc)), "integrate")

    def neighbour_stats(self, p: sf_params):
        cnt = np.zeros(self.n, np.uint32)
        hsh = np.zeros(self.n, np.uint32)
        _chk(getattr(lib(), f"sfo_neighbour_stats_{self.sfx}")(ctypes.byref(p), self.n, _ptr(self.pos),
                                                               _ptr(self.ids), _ptr(cnt), _ptr(hsh)), "nbr")
        return cnt, hsh

    def step(self, p: sf_params, nsteps: int = 1, threads: int = 0):
        _chk(getattr(lib(), f"sfo_step_{self.sfx}")(ctypes.byref(p), self.n, _ptr(self.pos), _ptr(self.vel),
                                                    _ptr(self.ids), nsteps, threads), "step")

    def frames(self, p: sf_params, frames: int, frame_time: float = 0.0333333333, max_substeps: int = 100000,
               threads: int = 0, record_dts: int = 0):
        """The frame loop (FP32); returns (sim_time, substeps, dts of the first `record_dts` sub-steps)."""
        t = ctypes.c_double()
        k = c_uint32()
        dts = np.zeros(record_dts, np.float32) if record_dts else None
        _chk(lib().sfo_frames_f32(ctypes.byref(p), self.n, _ptr(self.pos), _ptr(self.vel), _ptr(self.ids), frames,
                                  frame_time, max_substeps, threads, ctypes.byref(t), ctypes.byref(k), _ptr(dts),
                                  record_dts), "frames")
        return t.value, k.value, dts

    def original_order(self):
        """Positions and velocities in the caller's original particle order."""
        inv = np.empty_like(self.ids)
        inv[self.ids] = np.arange(self.n, dtype=np.uint32)
        return self.pos[inv], self.vel[inv]


def grad(p: sf_params, pos0, vel0, nsteps: int, target, ckpt: int = 20, dtype=np.float64, threads: int = 0):
    """Forward + CIC loss + adjoint: (loss, dL/dx0, dL/dv0, dL/dmu, dL/dk, final positions)."""
    dt = np.dtype(dtype)
    sfx = "f32" if dt == np.float32 else "f64"
    pos0 = np.ascontiguousarray(pos0, dt).reshape(-1, 3)
    vel0 = np.ascontiguousarray(vel0, dt).reshape(-1, 3)
    tgt = np.ascontiguousarray(target, dt).ravel()
    res = int(round(tgt.size ** (1 / 3)))
    n = pos0.shape[0]
    loss = np.zeros(1, dt)
    gx, gv, pf = np.zeros_like(pos0), np.zeros_like(vel0), np.zeros_like(pos0)
    gm, gk = np.zeros(1, dt), np.zeros(1, dt)
    _chk(getattr(lib(), f"sfo_grad_{sfx}")(ctypes.byref(p), n, _ptr(pos0), _ptr(vel0), nsteps, ckpt, _ptr(tgt), res,
                                           _ptr(loss), _ptr(gx), _ptr(gv), _ptr(gm), _ptr(gk), _ptr(pf), threads),
         "grad")
    return float(loss[0]), gx, gv, float(gm[0]), float(gk[0]), pf


def adjoint(p: sf_params, pos0, vel0, nsteps: int, seed_x, seed_v=None, ckpt: int = 20, dtype=np.float64,
            threads: int = 0):
    """Adjoint of `nsteps` from the given final-state adjoint: (dx0, dv0, dmu, dk, final positions)."""
    dt = np.dtype(dtype)
    sfx = "f32" if dt == np.float32 else "f64"
    pos0 = np.ascontiguousarray(pos0, dt).reshape(-1, 3)
    vel0 = np.ascontiguousarray(vel0, dt).reshape(-1, 3)
    sx = np.ascontiguousarray(seed_x, dt).reshape(-1, 3)
    sv = None if seed_v is None else np.ascontiguousarray(seed_v, dt).reshape(-1, 3)
    n = pos0.shape[0]
    gx, gv, pf = np.zeros_like(pos0), np.zeros_like(vel0), np.zeros_like(pos0)
    gm, gk = np.zeros(1, dt), np.zeros(1, dt)
    _chk(getattr(lib(), f"sfo_adjoint_{sfx}")(ctypes.byref(p), n, _ptr(pos0), _ptr(vel0), nsteps, ckpt, _ptr(sx),
                                              _ptr(sv), _ptr(gx), _ptr(gv), _ptr(gm), _ptr(gk), _ptr(pf), threads),
         "adjoint")
    return gx, gv, float(gm[0]), float(gk[0]), pf


def loss(p: sf_params, pos, target, dtype=np.float64):
    """CIC histogram loss and dL/dx of positions (n x 3)."""
    dt = np.dtype(dtype)
    sfx = "f32" if dt == np.float32 else "f64"
    pos = np.ascontiguousarray(pos, dt).reshape(-1, 3)
    tgt = np.ascontiguousarray(target, dt).ravel()
    res = int(round(tgt.size ** (1 / 3)))
    out = np.zeros(1, dt)
    g = np.zeros_like(pos)
    _chk(getattr(lib(), f"sfo_loss_{sfx}")(ctypes.byref(p), pos.shape[0], _ptr(pos), _ptr(tgt), res, _ptr(out),
                                           _ptr(g), None), "loss")
    return float(out[0]), g


def render(p: sf_params, rp, pos):
    """CPU restatement of the particle renderer: (rgba HxWx4, depth HxW, owner HxW)."""
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    h, w = rp.height, rp.width
    rgba = np.zeros((h, w, 4), np.float32)
    depth = np.zeros((h, w), np.float32)
    owner = np.zeros((h, w), np.uint32)
    _chk(lib().sfo_render(ctypes.byref(p), ctypes.byref(rp), pos.shape[0], _ptr(pos), _ptr(rgba), _ptr(depth),
                          _ptr(owner)), "render")
    return rgba, depth, owner


def render_camera(p: sf_params, rp):
    """The renderer's camera: (view matrix (16,), projection matrix (16,),
    column-major, point scale, point radius)."""
    V = np.zeros(16, np.float32)
    Pm = np.zeros(16, np.float32)
    scale, radius = ctypes.c_float(), ctypes.c_float()
    _chk(lib().sfo_render_camera(ctypes.byref(p), ctypes.byref(rp), _ptr(V), _ptr(Pm), ctypes.byref(scale),
                                 ctypes.byref(radius)), "render camera")
    return V, Pm, scale.value, radius.value


def particle_vertex(p: sf_params, rp, pos):
    """The renderer's vertex stage: (eye-space centres (n,3), point sizes (n,),
    clip positions (n,4))."""
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    n = pos.shape[0]
    eye = np.zeros((n, 3), np.float32)
    size = np.zeros(n, np.float32)
    clip = np.zeros((n, 4), np.float32)
    _chk(lib().sfo_particle_vertex(ctypes.byref(p), ctypes.byref(rp), n, _ptr(pos), _ptr(eye), _ptr(size),
                                   _ptr(clip)), "particle vertex")
    return eye, size, clip


def particle_fragment(p: sf_params, rp, eye, uv, color=None):
    """The renderer's fragment stage: (rgba (n,4), discarded (n,) bool); rgba
    is NaN where the fragment was discarded.  color None = the material's
    diffuse colour."""
    eye = np.ascontiguousarray(eye, np.float32).reshape(-1, 3)
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    n = eye.shape[0]
    col = None if color is None else np.ascontiguousarray(color, np.float32).reshape(n, 3)
    rgba = np.full((n, 4), np.nan, np.float32)
    disc = np.zeros(n, np.uint8)
    _chk(lib().sfo_particle_fragment(ctypes.byref(p), ctypes.byref(rp), n, _ptr(eye), _ptr(uv), _ptr(col),
                                     _ptr(rgba), _ptr(disc)), "particle fragment")
    return rgba, disc.astype(bool)


def _ref_shader():
    if not os.path.exists(REF_SHADER_LIB):
        return None
    r = ctypes.CDLL(REF_SHADER_LIB)
    F = ctypes.c_float
    r.ref_particle_vs.argtypes = [c_void_p, c_void_p, F, F, c_void_p, c_void_p, c_void_p, c_void_p]
    r.ref_particle_fs.argtypes = [c_void_p, c_int, c_void_p, F, c_int, c_void_p, c_void_p, c_void_p, c_void_p]
    r.ref_particle_fs.restype = c_int
    return r


def ref_particle_vertex(V, Pm, radius: float, scale: float, pos):
    """The reference's own vertex shader (Shaders/particle.vs.glsl, built by
    build_ref.sh) per particle: same outputs as particle_vertex, or None if
    it is not built."""
    r = _ref_shader()
    if r is None:
        return None
    V = np.ascontiguousarray(V, np.float32)
    Pm = np.ascontiguousarray(Pm, np.float32)
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
    n = pos.shape[0]
    eye = np.zeros((n, 3), np.float32)
    size = np.zeros(n, np.float32)
    clip = np.zeros((n, 4), np.float32)
    for i in range(n):
        r.ref_particle_vs(_ptr(V), _ptr(Pm), radius, scale, _ptr(pos[i]), _ptr(eye[i]), _ptr(size[i:i + 1]),
                          _ptr(clip[i]))
    return eye, size, clip


def ref_particle_fragment(rp, radius: float, eye, uv, color=None):
    """The reference's own fragment shader (Shaders/particle.fs.glsl, built by
    build_ref.sh) per fragment, with rp's lights and material: same outputs as
    particle_fragment, or None if it is not built."""
    r = _ref_shader()
    if r is None:
        return None
    lights = np.zeros((8, 16), np.float32)
    for l in range(8):
        lights[l, 0:4] = rp.light_ambient[l][:]
        lights[l, 4:8] = rp.light_diffuse[l][:]
        lights[l, 8:12] = rp.light_specular[l][:]
        lights[l, 12:16] = rp.light_position[l][:]
    mat = np.zeros(13, np.float32)
    mat[0:4] = rp.mat_ambient[:]
    mat[4:8] = rp.mat_diffuse[:]
    mat[8:12] = rp.mat_specular[:]
    mat[12] = rp.mat_shininess
    eye = np.ascontiguousarray(eye, np.float32).reshape(-1, 3)
    uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
    n = eye.shape[0]
    col = np.zeros((n, 3), np.float32) if color is None else np.ascontiguousarray(color, np.float32).reshape(n, 3)
    rgba = np.full((n, 4), np.nan, np.float32)
    disc = np.zeros(n, bool)
    for k in range(n):
        disc[k] = bool(r.ref_particle_fs(_ptr(lights), rp.num_lights, _ptr(mat), radius, 0 if color is None else 1,
                                         _ptr(col[k]), _ptr(eye[k]), _ptr(uv[k]), _ptr(rgba[k])))
    return rgba, disc


def frame_accounting(dts, stop_time: float, frame_time: float = FRAME_TIME, cap: int = 100000):
    """The oracle's frame accounting on given sub-step sizes: (sub-steps per
    frame, float simulated time after each frame)."""
    dts = np.ascontiguousarray(dts, np.float32)
    sub = np.zeros(cap, np.uint32)
    t = np.zeros(cap, np.float32)
    nf = c_uint32()
    _chk(lib().sfo_frame_accounting(_ptr(dts), dts.size, frame_time, stop_time, cap, _ptr(sub), _ptr(t),
                                    ctypes.byref(nf)), "frame accounting")
    return sub[:nf.value].copy(), t[:nf.value].copy()


def ref_frames(dts, stop_time: float, cap: int = 100000):
    """The reference's own frame loop (Source/Simulator.cpp, built by
    build_ref.sh) on given sub-step sizes: (sub-steps per frame, float
    simulated time after each frame), or None if it is not built."""
    if not os.path.exists(REF_SIM_LIB):
        return None
    r = ctypes.CDLL(REF_SIM_LIB)
    r.ref_frames.argtypes = [c_void_p, c_uint32, ctypes.c_float, c_uint32, c_void_p, c_void_p, POINTER(c_uint32)]
    dts = np.ascontiguousarray(dts, np.float32)
    sub = np.zeros(cap, np.uint32)
    t = np.zeros(cap, np.float32)
    nf = c_uint32()
    _chk(r.ref_frames(_ptr(dts), dts.size, stop_time, cap, _ptr(sub), _ptr(t), ctypes.byref(nf)), "reference frames")
    return sub[:nf.value].copy(), t[:nf.value].copy()


def max_threads() -> int:
    return int(lib().sfo_max_threads())
