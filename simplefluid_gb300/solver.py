"""Python mirror of the reference's solver-facing interface, over the C ABI.

Names, argument meanings and call order follow the reference:

* ``SPHParameters``  — the fields of ``SPHParameters<float>`` that
  Source/Controller.cpp:54-61 writes, plus ``particleRadius`` and ``scene``
  (Source/SceneManager.cpp:23,45) and the constants the workloads fix.
* ``SPHSolver``      — ``SPHSolver<float>`` as used through ``QtSPHSolver``
  (Include/QtSPHSolver.h:27-35): ``makeReady``, ``advanceFrame``,
  ``getNumParticles``, ``getParticles``, ``getVelocity``.
* ``SceneManager``   — Source/SceneManager.cpp:21-173.
* ``Simulator``      — the headless frame loop of Source/Simulator.cpp:22-103.

All compute runs in the CUDA library; there is no CPU fallback.  Constructing
an ``SPHSolver`` without a GPU raises ``SFError`` (SF_ERR_NO_DEVICE).
"""
from __future__ import annotations

import ctypes
import threading
from ctypes import byref, c_float, c_uint32, c_void_p
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np

from . import _capi as C


def _vp(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(c_void_p)


def _cuda_array(arr, what: str):
    """(device pointer, n) of an (n, 3) float32 C-contiguous CUDA array."""
    try:
        cai = arr.__cuda_array_interface__
    except AttributeError:
        raise TypeError(f"{what} must expose __cuda_array_interface__ (a CUDA array)") from None
    shape = tuple(cai["shape"])
    if cai["typestr"] != "<f4" or len(shape) != 2 or shape[1] != 3:
        raise ValueError(f"{what} must be an (n, 3) float32 array")
    strides = cai.get("strides")
    if strides is not None and tuple(strides) != (12, 4):
        raise ValueError(f"{what} must be C-contiguous")
    ptr = int(cai["data"][0])
    return (c_void_p(ptr) if ptr else None), int(shape[0])


def _stream_handle(stream, arr=None):
    """cudaStream_t of `stream` (an int, or an object with .cuda_stream), else
    the stream named by a version-3 __cuda_array_interface__, else None.  The
    default stream (handle 0) is passed as cudaStreamLegacy (1)."""
    if stream is None and arr is not None:
        stream = getattr(arr, "__cuda_array_interface__", {}).get("stream")
    if stream is None:
        return None
    handle = int(getattr(stream, "cuda_stream", stream))
    return c_void_p(handle if handle else 1)


@dataclass
class SPHParameters:
    """Mirror of ``SPHParameters<float>``; defaults are the 16k dambreak workload."""

    numThreads: int = 0
    kernelRadius: float = 0.04
    particleRadius: float = 0.01
    pressureStiffness: float = 50.0
    boundaryRestitution: float = 0.1
    viscosity: float = 0.01
    stopTime: float = 5.0
    bUseAttractivePressure: bool = False
    scene: int = C.SF_SCENE_DAMBREAK_16K
    restDensity: float = 1000.0
    gravity: tuple = (0.0, -9.8, 0.0)
    timeStep: float = 1e-4
    boxMin: tuple = (0.0, 0.0, 0.0)
    boxMax: tuple = (1.0, 1.0, 1.0)
    eos: int = C.SF_EOS_LINEAR
    cellsPerH: int = 2
    adaptiveTimeStep: bool = False

    def to_c(self) -> C.sf_params:
        p = C.sf_params()
        p.num_threads = int(self.numThreads)
        p.kernel_radius = self.kernelRadius
        p.particle_radius = self.particleRadius
        p.pressure_stiffness = self.pressureStiffness
        p.boundary_restitution = self.boundaryRestitution
        p.viscosity = self.viscosity
        p.stop_time = self.stopTime
        p.use_attractive_pressure = 1 if self.bUseAttractivePressure else 0
        p.scene = int(self.scene)
        p.rest_density = self.restDensity
        for a in range(3):
            p.gravity[a] = self.gravity[a]
            p.box_min[a] = self.boxMin[a]
            p.box_max[a] = self.boxMax[a]
        p.time_step = self.timeStep
        p.eos = int(self.eos)
        p.cells_per_h = int(self.cellsPerH)
        p.adaptive_time_step = 1 if self.adaptiveTimeStep else 0
        return p

    @classmethod
    def from_c(cls, p: C.sf_params) -> "SPHParameters":
        return cls(numThreads=p.num_threads, kernelRadius=p.kernel_radius, particleRadius=p.particle_radius,
                   pressureStiffness=p.pressure_stiffness, boundaryRestitution=p.boundary_restitution,
                   viscosity=p.viscosity, stopTime=p.stop_time, bUseAttractivePressure=bool(p.use_attractive_pressure),
                   scene=p.scene, restDensity=p.rest_density, gravity=tuple(p.gravity), timeStep=p.time_step,
                   boxMin=tuple(p.box_min), boxMax=tuple(p.box_max), eos=p.eos, cellsPerH=p.cells_per_h,
                   adaptiveTimeStep=bool(p.adaptive_time_step))

    def updateParams(self) -> None:
        """SPHParameters::updateParams() (Source/Controller.cpp:63): validate."""
        p = self.to_c()
        C.check(C.load().sf_params_update(byref(p)))

    @classmethod
    def for_resolution(cls, resolution: int, **kw) -> "SPHParameters":
        """The GUI's resolution control: kernelRadius = 2 / resolution (Source/Controller.cpp:55)."""
        return cls(kernelRadius=2.0 / float(resolution), **kw)


class SPHSolver:
    """``SPHSolver<float>`` on one GB300, driven through the C ABI."""

    def __init__(self, params: SPHParameters):
        self._lib = C.load()
        self.params = params
        self._ctx = c_void_p()
        cp = params.to_c()
        C.check(self._lib.sf_create(byref(cp), byref(self._ctx)))
        self._n = 0

    # -- lifetime ----------------------------------------------------------
    def close(self) -> None:
        if self._ctx:
            self._lib.sf_destroy(self._ctx)
            self._ctx = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> c_void_p:
        return self._ctx

    def setParams(self, params: SPHParameters) -> None:
        cp = params.to_c()
        C.check(self._lib.sf_set_params(self._ctx, byref(cp)))
        self.params = params

    # -- state: getParticles()/getVelocity() ------------------------------
    def setParticles(self, particles: np.ndarray, velocity: Optional[np.ndarray] = None) -> None:
        pos = np.ascontiguousarray(particles, dtype=np.float32).reshape(-1, 3)
        vel = None if velocity is None else np.ascontiguousarray(velocity, dtype=np.float32).reshape(-1, 3)
        if vel is not None and vel.shape != pos.shape:
            raise ValueError("velocity must have the same shape as particles")
        C.check(self._lib.sf_set_state(self._ctx, _vp(pos), _vp(vel), pos.shape[0]))
        self._n = pos.shape[0]

    def getNumParticles(self) -> int:
        n = c_uint32()
        C.check(self._lib.sf_get_num_particles(self._ctx, byref(n)))
        return n.value

    def getParticles(self) -> np.ndarray:
        n = self.getNumParticles()
        out = np.empty((n, 3), np.float32)
        C.check(self._lib.sf_get_state(self._ctx, _vp(out), None, n))
        return out

    def getVelocity(self) -> np.ndarray:
        n = self.getNumParticles()
        out = np.empty((n, 3), np.float32)
        C.check(self._lib.sf_get_state(self._ctx, None, _vp(out), n))
        return out

    def getState(self):
        n = self.getNumParticles()
        pos = np.empty((n, 3), np.float32)
        vel = np.empty((n, 3), np.float32)
        C.check(self._lib.sf_get_state(self._ctx, _vp(pos), _vp(vel), n))
        return pos, vel

    # -- state in device memory --------------------------------------------------
    # Arrays are (n, 3) float32, C-contiguous, in device memory of the solver's
    # GPU, given as any object exposing __cuda_array_interface__ (a torch CUDA
    # tensor, for one).  `stream` is the caller's stream (a cudaStream_t as int,
    # or an object with a ``cuda_stream`` attribute such as torch.cuda.Stream):
    # the solver reads after the work queued on it, and work queued on it after
    # getStateDevice sees the written arrays.
    def setParticlesDevice(self, particles, velocity=None, stream=None) -> None:
        pptr, n = _cuda_array(particles, "particles")
        vptr = None
        if velocity is not None:
            vptr, nv = _cuda_array(velocity, "velocity")
            if nv != n:
                raise ValueError("velocity must have the same shape as particles")
        C.check(self._lib.sf_set_state_device(self._ctx, pptr, vptr, n, _stream_handle(stream, particles)))
        self._n = n

    def getStateDevice(self, particles=None, velocity=None, stream=None) -> None:
        """Write the state, in the caller's particle order, into device arrays."""
        n = self.getNumParticles()
        ptrs = []
        for arr, what in ((particles, "particles"), (velocity, "velocity")):
            if arr is None:
                ptrs.append(None)
                continue
            ptr, na = _cuda_array(arr, what)
            if na != n:
                raise ValueError(f"{what} must hold {n} particles")
            ptrs.append(ptr)
        C.check(self._lib.sf_get_state_device(self._ctx, ptrs[0], ptrs[1], n, _stream_handle(stream, particles)))

    def checkState(self) -> dict:
        """Invariants of the current state counted on the GPU (sf_check_state):
        non-finite values, particles outside the box, sort and cell-table
        consistency, caller-index permutation, list overflows, max speed."""
        r = C.sf_state_report()
        C.check(self._lib.sf_check_state(self._ctx, byref(r)))
        return r.as_dict()

    def setTuning(self, t: C.sf_tuning) -> None:
        """Kernel choices of this solver's step (sf_set_tuning); every choice
        computes the same bits."""
        C.check(self._lib.sf_set_tuning(self._ctx, byref(t)))

    def getTuning(self) -> C.sf_tuning:
        t = C.sf_tuning()
        C.check(self._lib.sf_get_tuning(self._ctx, byref(t)))
        return t

    def deviceState(self) -> "C.sf_device_view":
        """Device pointers to the cell-sorted working arrays (sf_device_view)."""
        v = C.sf_device_view()
        C.check(self._lib.sf_device_state(self._ctx, byref(v)))
        return v

    # -- stepping ------------------------------------------------------------
    def makeReady(self) -> None:
        C.check(self._lib.sf_make_ready(self._ctx))

    def advanceFrame(self) -> float:
        dt = c_float()
        C.check(self._lib.sf_advance_frame(self._ctx, byref(dt)))
        return dt.value

    def step(self, nsteps: int) -> None:
        C.check(self._lib.sf_step(self._ctx, int(nsteps)))

    def advanceFrames(self, frames: int, frame_time: float = 0.0333333333, max_substeps: int = 100000):
        """Whole frames on the device; returns (simulated time, sub-steps taken)."""
        t = ctypes.c_double()
        k = c_uint32()
        C.check(self._lib.sf_advance_frames(self._ctx, int(frames), float(frame_time), int(max_substeps), byref(t),
                                            byref(k)))
        return t.value, k.value

    def synchronize(self) -> None:
        C.check(self._lib.sf_synchronize(self._ctx))

    # -- inspection of the cell-sorted internal order ------------------------
    def gridDims(self) -> tuple:
        d = (c_uint32 * 3)()
        C.check(self._lib.sf_get_grid(self._ctx, d))
        return tuple(d)

    def sortedState(self):
        n = self.getNumParticles()
        pos = np.empty((n, 4), np.float32)
        vel = np.empty((n, 4), np.float32)
        ids = np.empty(n, np.uint32)
        keys = np.empty(n, np.uint32)
        C.check(self._lib.sf_get_sorted(self._ctx, _vp(pos), _vp(vel), _vp(ids), _vp(keys), n))
        return pos[:, :3].copy(), vel[:, :3].copy(), ids, keys

    def cellStart(self) -> np.ndarray:
        nx, ny, nz = self.gridDims()
        out = np.empty(nx * ny * nz + 1, np.uint32)
        C.check(self._lib.sf_get_cell_start(self._ctx, _vp(out), out.size))
        return out

    def computeDensity(self):
        n = self.getNumParticles()
        rho = np.empty(n, np.float32)
        prs = np.empty(n, np.float32)
        C.check(self._lib.sf_compute_density(self._ctx, _vp(rho), _vp(prs), n))
        return rho, prs

    def computeAccel(self) -> np.ndarray:
        n = self.getNumParticles()
        acc = np.empty((n, 3), np.float32)
        C.check(self._lib.sf_compute_accel(self._ctx, _vp(acc), n))
        return acc

    # -- headless rendering ------------------------------------------------
    def render(self, rp: Optional[C.sf_render_params] = None):
        """Sphere-impostor image of the particles: (rgba HxWx4, depth HxW, owner HxW)."""
        rp = rp or render_params()
        h, w = rp.height, rp.width
        rgba = np.empty((h, w, 4), np.float32)
        depth = np.empty((h, w), np.float32)
        owner = np.empty((h, w), np.uint32)
        C.check(self._lib.sf_render(self._ctx, byref(rp), _vp(rgba), _vp(depth), _vp(owner)))
        return rgba, depth, owner

    # -- state files -----------------------------------------------------
    def saveState(self, path: str, sim_time: float = 0.0) -> None:
        C.check(self._lib.sf_save_state(self._ctx, str(path).encode(), float(sim_time)))

    def loadState(self, path: str) -> float:
        """Load parameters and state (solver order kept); returns the saved sim time."""
        t = ctypes.c_double()
        C.check(self._lib.sf_load_state(self._ctx, str(path).encode(), byref(t)))
        pr = C.sf_params()
        C.check(self._lib.sf_get_params(self._ctx, byref(pr)))
        self.params = SPHParameters.from_c(pr)
        return t.value

    # -- differentiation ---------------------------------------------------
    def forward(self, nsteps: int, ckpt_every: int = 20) -> None:
        """Advance `nsteps` recording checkpoints for :meth:`adjoint`."""
        C.check(self._lib.sf_forward(self._ctx, int(nsteps), int(ckpt_every)))

    def lossHistogram(self, target: np.ndarray, with_grad: bool = True):
        """CIC-histogram loss of the current positions against `target` (res^3)."""
        t = np.ascontiguousarray(target, np.float32)
        res = int(round(t.size ** (1.0 / 3.0)))
        if res ** 3 != t.size:
            raise ValueError("target must have res^3 entries")
        loss = ctypes.c_double()
        g = np.empty((self.getNumParticles(), 3), np.float32) if with_grad else None
        C.check(self._lib.sf_loss_histogram(self._ctx, _vp(t), res, byref(loss), _vp(g)))
        return (loss.value, g) if with_grad else loss.value

    def adjoint(self, dloss_dx: np.ndarray, dloss_dv: Optional[np.ndarray] = None):
        """Gradients of the loss w.r.t. the state at the last :meth:`forward` call
        and w.r.t. viscosity and stiffness: (dx0, dv0, dmu, dk)."""
        n = self.getNumParticles()
        gx = np.ascontiguousarray(dloss_dx, np.float32).reshape(n, 3)
        gv = None if dloss_dv is None else np.ascontiguousarray(dloss_dv, np.float32).reshape(n, 3)
        dx0 = np.empty((n, 3), np.float32)
        dv0 = np.empty((n, 3), np.float32)
        dmu = c_float()
        dk = c_float()
        C.check(self._lib.sf_adjoint(self._ctx, _vp(gx), _vp(gv), _vp(dx0), _vp(dv0), byref(dmu), byref(dk)))
        return dx0, dv0, dmu.value, dk.value

    def neighbourStats(self):
        n = self.getNumParticles()
        cnt = np.empty(n, np.uint32)
        hsh = np.empty(n, np.uint32)
        C.check(self._lib.sf_neighbour_stats(self._ctx, _vp(cnt), _vp(hsh), n))
        return cnt, hsh


def scene_positions(params: SPHParameters, scene: int, seed: int = 20171) -> np.ndarray:
    """Positions of a scene from the library's generator (host code, no GPU needed)."""
    lib = C.load()
    cp = params.to_c()
    n = c_uint32()
    C.check(lib.sf_scene_count(byref(cp), int(scene), seed, byref(n)))
    out = np.empty((n.value, 3), np.float32)
    C.check(lib.sf_setup_scene(byref(cp), int(scene), seed, _vp(out), None, n.value, byref(n)))
    return out


class SceneManager:
    """Source/SceneManager.cpp:21-173 — fills particle and velocity arrays."""

    def __init__(self, params: SPHParameters, seed: int = 20171):
        self.params = params
        self.seed = seed

    def setupScene(self):
        return self._make(self.params.scene)

    def setupSceneCubeDrop(self):
        return self._make(C.SF_SCENE_CUBE_DROP)

    def setupSceneSphereDrop(self):
        return self._make(C.SF_SCENE_SPHERE_DROP)

    def setupSceneDambreak(self):
        return self._make(C.SF_SCENE_DAMBREAK)

    def setupSceneDoubleDambreak(self):
        return self._make(C.SF_SCENE_DOUBLE_DAMBREAK)

    def _make(self, scene: int):
        pos = scene_positions(self.params, scene, self.seed)
        return pos, np.zeros_like(pos)


FRAME_TIME = 0.0333333333  # Source/Simulator.cpp:47


def substeps_per_frame(dt: float) -> int:
    """Sub-steps the frame loop of Source/Simulator.cpp:46-51 takes with a fixed
    dt: frameTime (float32) accumulates dt until it reaches 1/30 s."""
    ft = np.float32(0.0)
    k = 0
    d = np.float32(dt)
    while float(ft) < FRAME_TIME:
        ft = np.float32(ft + d)
        k += 1
    return k


class Simulator:
    """Headless restatement of Source/Simulator.cpp:22-103.

    Qt signals become optional callbacks: ``particleChanged`` (per sub-step,
    Source/Simulator.cpp:50), ``systemTimeChanged`` / ``frameFinished`` (per
    frame, :54-55), ``simulationFinished`` (:60), ``numParticleChanged`` (:102).
    With no ``particleChanged`` callback a frame runs on the device as one
    graph launch (``sf_advance_frames``: same arithmetic, no per-sub-step host
    round trip).
    """

    def __init__(self, params: Optional[SPHParameters] = None, seed: int = 20171):
        self.m_SimParams = params or SPHParameters()
        self.m_SPHSolver = SPHSolver(self.m_SimParams)
        self.m_SceneManager = SceneManager(self.m_SimParams, seed)
        self.m_SimTime = np.float32(0.0)
        self.m_bStop = True
        self._worker: Optional[threading.Thread] = None
        self._error: Optional[BaseException] = None
        self.particleChanged: Optional[Callable[[], None]] = None
        self.systemTimeChanged: Optional[Callable[[float], None]] = None
        self.frameFinished: Optional[Callable[[], None]] = None
        self.simulationFinished: Optional[Callable[[], None]] = None
        self.numParticleChanged: Optional[Callable[[int], None]] = None

    def getSimParams(self) -> SPHParameters:
        return self.m_SimParams

    def isRunning(self) -> bool:
        return not self.m_bStop

    def startSimulation(self) -> None:
        self.m_bStop = False
        self.wait()
        self._worker = threading.Thread(target=self._run, daemon=True)
        self._worker.start()

    def _run(self):
        try:
            self.doSimulation()
        except BaseException as e:  # surfaced by wait()
            self._error = e
            self.m_bStop = True

    def wait(self) -> None:
        if self._worker is not None:
            self._worker.join()
            self._worker = None
        if self._error is not None:
            e, self._error = self._error, None
            raise e

    def doSimulation(self) -> None:
        solver = self.m_SPHSolver
        solver.makeReady()
        while float(self.m_SimTime) < self.m_SimParams.stopTime and not self.m_bStop:
            frame_time = np.float32(0.0)
            if self.particleChanged is None:
                # the whole frame on the device: one graph launch
                t, _ = solver.advanceFrames(1, FRAME_TIME)
                frame_time = np.float32(t)
            else:
                while float(frame_time) < FRAME_TIME:
                    frame_time = np.float32(frame_time + np.float32(solver.advanceFrame()))
                    self.particleChanged()
            self.m_SimTime = np.float32(self.m_SimTime + frame_time)
            if self.systemTimeChanged:
                self.systemTimeChanged(float(self.m_SimTime))
            if self.frameFinished:
                self.frameFinished()
        solver.synchronize()
        if not self.m_bStop:
            self.m_bStop = True
            if self.simulationFinished:
                self.simulationFinished()

    def stop(self) -> None:
        self.m_bStop = True

    def reset(self) -> None:
        self.m_bStop = True
        self.setupScene()

    def changeScene(self, scene: int) -> None:
        self.m_SimParams.scene = scene
        self.setupScene()

    def setupScene(self) -> None:
        self.m_SimTime = np.float32(0.0)
        if self.systemTimeChanged:
            self.systemTimeChanged(0.0)
        self.wait()
        pos, vel = self.m_SceneManager.setupScene()
        self.m_SPHSolver.setParams(self.m_SimParams)
        self.m_SPHSolver.setParticles(pos, vel)
        if self.particleChanged:
            self.particleChanged()
        if self.numParticleChanged:
            self.numParticleChanged(self.m_SPHSolver.getNumParticles())


def render_params(**kw) -> C.sf_render_params:
    """The reference viewer's render settings, with keyword overrides."""
    rp = C.sf_render_params()
    C.check(C.load().sf_render_params_default(byref(rp)))
    for k, v in kw.items():
        if k in ("eye", "focus", "up", "background"):
            for a, x in enumerate(v):
                getattr(rp, k)[a] = x
        else:
            setattr(rp, k, v)
    return rp


def save_ppm(path: str, rgba: np.ndarray) -> None:
    """Write an RGBA float image (rows top to bottom) as an 8-bit binary PPM."""
    img = (np.clip(rgba[..., :3], 0.0, 1.0) * 255.0 + 0.5).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (img.shape[1], img.shape[0]))
        f.write(img.tobytes())


STATE_MAGIC = b"SFSTATE1"


def read_state_file(path: str):
    """Read a state file (no GPU needed): dict with sim_time, params, and
    positions/velocities in the caller's particle order."""
    with open(path, "rb") as f:
        raw = f.read()
    if raw[:8] != STATE_MAGIC:
        raise ValueError("not a SimpleFluid state file")
    version, n = np.frombuffer(raw, np.uint32, 2, 8)
    if version != 1:
        raise ValueError(f"unsupported state file version {version}")
    t = float(np.frombuffer(raw, np.float64, 1, 16)[0])
    psize = ctypes.sizeof(C.sf_params)
    params = C.sf_params.from_buffer_copy(raw[24:24 + psize])
    off = 24 + psize
    pv = np.frombuffer(raw, np.float32, 6 * int(n), off)
    ids = np.frombuffer(raw, np.uint32, int(n), off + 24 * int(n))
    pos = np.empty((int(n), 3), np.float32)
    vel = np.empty((int(n), 3), np.float32)
    pos[ids] = pv[:3 * int(n)].reshape(-1, 3)
    vel[ids] = pv[3 * int(n):].reshape(-1, 3)
    return {"sim_time": t, "params": params, "positions": pos, "velocities": vel, "solver_order": ids.copy()}


def batch_cubes(seed: int, nscenes: int, base: SPHParameters):
    """The batched-cube workload: (per-scene sf_params list, counts, concatenated positions)."""
    lib = C.load()
    bp = base.to_c()
    total = ctypes.c_uint64()
    C.check(lib.sf_batch_cubes(seed, nscenes, byref(bp), None, None, None, 0, byref(total)))
    params = (C.sf_params * nscenes)()
    counts = np.empty(nscenes, np.uint32)
    pos = np.empty((total.value, 3), np.float32)
    C.check(lib.sf_batch_cubes(seed, nscenes, byref(bp), params, _vp(counts), _vp(pos), total.value, byref(total)))
    return list(params), counts, pos


class SPHBatch:
    """Many independent scenes advanced together (one graph launch per step)."""

    def __init__(self, scene_params):
        self._lib = C.load()
        n = len(scene_params)
        arr = (C.sf_params * n)()
        for s, p in enumerate(scene_params):
            arr[s] = p.to_c() if isinstance(p, SPHParameters) else p
        self._b = c_void_p()
        C.check(self._lib.sf_batch_create(arr, n, byref(self._b)))
        self.nscenes = n

    def close(self):
        if self._b:
            self._lib.sf_batch_destroy(self._b)
            self._b = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._b

    def setState(self, counts, pos, vel=None):
        counts = np.ascontiguousarray(counts, np.uint32)
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        if counts.size != self.nscenes or int(counts.sum()) != pos.shape[0]:
            raise ValueError("counts must have one entry per scene and sum to the number of particles")
        C.check(self._lib.sf_batch_set_state(self._b, _vp(counts), _vp(pos), _vp(vel)))

    def numParticles(self) -> int:
        n = c_uint32()
        C.check(self._lib.sf_batch_num_particles(self._b, byref(n)))
        return n.value

    def getState(self):
        n = self.numParticles()
        pos = np.empty((n, 3), np.float32)
        vel = np.empty((n, 3), np.float32)
        C.check(self._lib.sf_batch_get_state(self._b, _vp(pos), _vp(vel), n))
        return pos, vel

    def checkState(self) -> dict:
        """sf_check_state over all scenes (see SPHSolver.checkState)."""
        r = C.sf_state_report()
        C.check(self._lib.sf_batch_check_state(self._b, byref(r)))
        return r.as_dict()

    def getParams(self, scene: int) -> C.sf_params:
        p = C.sf_params()
        C.check(self._lib.sf_batch_get_params(self._b, scene, byref(p)))
        return p

    def step(self, nsteps: int):
        C.check(self._lib.sf_batch_step(self._b, int(nsteps)))

    def synchronize(self):
        C.check(self._lib.sf_batch_synchronize(self._b))

    def setCellsPerH(self, k: int):
        C.check(self._lib.sf_batch_set_cells_per_h(self._b, int(k)))

    def setTuning(self, t: C.sf_tuning):
        C.check(self._lib.sf_batch_set_tuning(self._b, byref(t)))

    def getTuning(self) -> C.sf_tuning:
        t = C.sf_tuning()
        C.check(self._lib.sf_batch_get_tuning(self._b, byref(t)))
        return t

    def autotune(self, trial_steps: int = 10):
        t = C.sf_tuning()
        k = ctypes.c_int32()
        ms = c_float()
        C.check(self._lib.sf_batch_autotune(self._b, int(trial_steps), byref(t), byref(k), byref(ms)))
        return t, k.value, ms.value

    def timedSteps(self, nsteps: int, flush_bytes: int = 0) -> float:
        ms = c_float()
        C.check(self._lib.sf_batch_step_timed(self._b, int(nsteps), int(flush_bytes), byref(ms), None))
        return ms.value
