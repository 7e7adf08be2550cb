"""Generate the golden fixtures in tests/golden/.

1. ``ref_scenes.npz`` — positions written by the reference's OWN scene
   generator (Source/SceneManager.cpp, compiled in place by oracle/build_ref.sh
   into oracle/_ref/libref_scenes.so) for the four SimulationScenes at several
   particle radii.  Small cases are stored whole; all cases carry a SHA-256 of
   the float32 bytes and the particle count.  These pin the scene generators of
   the oracle and of the product.
2. ``ref_frames.npz`` — the frame accounting of the reference's OWN frame loop
   (Source/Simulator.cpp's doSimulation, compiled in place by
   oracle/build_ref.sh into oracle/_ref/libref_sim.so with a solver that
   returns given sub-step sizes): sub-steps per 1/30 s frame and the float
   simulated time after each frame, for a fixed step, a seeded varied one, and
   the adaptive sub-steps the oracle takes on the 16,000-particle dambreak.
   These pin the frame loops of the oracle and of the product.
3. ``ref_shader.npz`` — outputs of the reference's OWN particle shaders
   (Shaders/particle.vs.glsl and particle.fs.glsl, compiled as C++ by
   oracle/build_ref.sh into oracle/_ref/libref_shader.so) for two render
   settings (the viewer's defaults, and eight seeded lights with another
   camera and material): per seeded particle the eye-space centre, point size
   and clip position; per seeded fragment (point coordinate, sprite centre,
   colour) the discard decision and the colour, for uniform and per-particle
   colours.  The render settings are stored as the bytes of sf_render_params.
   These pin the oracle's restatement of the shader arithmetic.
4. ``oracle_regression.npz`` — outputs of the CPU oracle (built on x86-64) for a
   small SPH case: one sort, density, acceleration and 5 full steps.  They are a
   regression record of the oracle itself (not a pin to the reference's solver,
   which is absent) and let a run on another host architecture check that its
   oracle build computes the same bits.

Run from the repository root with the reference tree's location:
    python tests/golden/make_golden.py <reference root>
(or with SF_REFERENCE_ROOT set).
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O
from simplefluid_gb300 import SPHParameters, render_params  # noqa: E402
from simplefluid_gb300._capi import sf_params  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

# (scene id, particle radius); radii chosen so counts stay small for whole storage
REF_CASES = [(s, r) for s in range(4) for r in (0.05, 0.04, 1 / 32, 0.025, 0.02, 1 / 64, 0.01)]
WHOLE_LIMIT = 20000


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def small_params() -> sf_params:
    p = sf_params()
    p.num_threads = 0
    p.particle_radius = 0.02
    p.kernel_radius = 0.08
    p.pressure_stiffness = 50.0
    p.boundary_restitution = 0.1
    p.viscosity = 0.01
    p.stop_time = 5.0
    p.rest_density = 1000.0
    p.gravity[1] = -9.8
    p.time_step = 1e-4
    for a in range(3):
        p.box_min[a] = 0.0
        p.box_max[a] = 1.0
    return p


def _same(a, b) -> bool:
    """Equal arrays, floats compared by their bits."""
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype != b.dtype or a.shape != b.shape:
        return False
    return a.tobytes() == b.tobytes()


def save_if_changed(path: str, arrays: dict) -> None:
    """Write the fixture unless the file already holds exactly these arrays."""
    if os.path.exists(path):
        old = np.load(path)
        if set(old.files) == set(arrays) and all(_same(old[k], v) for k, v in arrays.items()):
            return
    np.savez_compressed(path, **arrays)


# point coordinates at the disc's centre, on its rim (kept: the shader
# discards only where the squared length exceeds 1) and at the corners
EDGE_UV = np.array([[0.5, 0.5], [0.5, 0.0], [0.0, 0.5], [1.0, 0.5], [0.5, 1.0], [0.0, 0.0], [1.0, 1.0],
                    [0.25, 0.25]], np.float32)


def shader_cases() -> dict:
    """The reference's particle shaders on seeded particles and fragments."""
    rng = np.random.default_rng(4101)
    viewer = render_params()
    lights8 = render_params(width=640, height=480, eye=(2.5, 1.5, -2.0), focus=(0.1, 0.0, 0.2), fovy_deg=40.0,
                            point_radius=0.03, num_lights=8, mat_shininess=64.0)
    for l in range(8):
        lights8.light_position[l][:] = [*rng.uniform(-20, 20, 3), 1.0]
        lights8.light_ambient[l][:] = [*rng.uniform(0, 0.2, 3), 1.0]
        lights8.light_diffuse[l][:] = [*rng.uniform(0, 1, 3), 1.0]
        lights8.light_specular[l][:] = [*rng.uniform(0, 1, 3), 1.0]
    lights8.mat_ambient[:] = [*rng.uniform(0, 1, 3), 1.0]
    lights8.mat_diffuse[:] = [*rng.uniform(0, 1, 3), 1.0]
    lights8.mat_specular[:] = [*rng.uniform(0, 1, 3), 1.0]
    out = {}
    for name, rp, radius in (("viewer", viewer, 0.01), ("lights8", lights8, 0.02)):
        p = SPHParameters(particleRadius=radius).to_c()
        V, Pm, scale, rad = O.render_camera(p, rp)
        pos = rng.uniform(-1.0, 1.0, size=(1024, 3)).astype(np.float32)
        eye, size, clip = O.ref_particle_vertex(V, Pm, rad, scale, pos)
        m = 2048
        idx = rng.integers(0, pos.shape[0], m + EDGE_UV.shape[0])
        uv = np.concatenate([rng.uniform(0.0, 1.0, size=(m, 2)).astype(np.float32), EDGE_UV])
        color = rng.uniform(0.0, 1.0, size=(idx.size, 3)).astype(np.float32)
        rgba_u, disc = O.ref_particle_fragment(rp, rad, eye[idx], uv)
        rgba_c, disc_c = O.ref_particle_fragment(rp, rad, eye[idx], uv, color)
        assert np.array_equal(disc, disc_c)
        out.update({f"{name}_rp": np.frombuffer(bytes(rp), np.uint8).copy(),
                    f"{name}_radius": np.array(radius, np.float32), f"{name}_pos": pos, f"{name}_eye": eye,
                    f"{name}_size": size, f"{name}_clip": clip, f"{name}_frag_idx": idx.astype(np.int32),
                    f"{name}_uv": uv, f"{name}_color": color, f"{name}_discarded": disc,
                    f"{name}_rgba_uniform": rgba_u, f"{name}_rgba_color": rgba_c})
    return out


def main() -> None:
    O.build(force=True)
    if O.build_ref(sys.argv[1] if len(sys.argv) > 1 else None) is None:
        raise SystemExit("reference tree not available: cannot build oracle/_ref")
    out = {}
    for s, r in REF_CASES:
        pos = O.ref_scene(s, r)
        key = f"s{s}_r{r:.6f}"
        out[f"{key}_n"] = np.array(pos.shape[0], np.int64)
        out[f"{key}_sha"] = np.array(sha(pos))
        out[f"{key}_r"] = np.array(r, np.float32)
        out[f"{key}_scene"] = np.array(s, np.int32)
        if pos.shape[0] <= WHOLE_LIMIT:
            out[f"{key}_pos"] = pos
    save_if_changed(os.path.join(HERE, "ref_scenes.npz"), out)

    # the reference's frame loop on given sub-step sizes
    frames = {}
    rng = np.random.default_rng(20171)
    adaptive = SPHParameters(particleRadius=0.01, kernelRadius=0.04, adaptiveTimeStep=True, timeStep=5e-3,
                             stopTime=0.1, scene=16)
    st = O.State(O.scene(adaptive.to_c(), 16))
    _, k, adts = st.frames(adaptive.to_c(), 4, record_dts=20000)
    cases = {"fixed": (np.full(3000, 1e-4, np.float32), 0.2),
             "varied": (rng.uniform(2e-5, 2e-3, size=4000).astype(np.float32), 0.25),
             "adaptive16k": (adts[:k].copy(), 0.1)}
    for name, (dts, stop) in cases.items():
        sub, times = O.ref_frames(dts, stop)
        frames[f"{name}_dts"] = dts
        frames[f"{name}_stop"] = np.array(stop, np.float32)
        frames[f"{name}_substeps"] = sub
        frames[f"{name}_sim_times"] = times
    save_if_changed(os.path.join(HERE, "ref_frames.npz"), frames)

    save_if_changed(os.path.join(HERE, "ref_shader.npz"), shader_cases())

    # oracle regression: 10x20x10 block, jitter-free, small box
    p = small_params()
    pos = O.scene(p, 16)[:2000]  # first 2000 of the 20x40x20 block (r=0.02 spacing 0.04)
    st = O.State(pos)
    keys, cs = st.sort(p, want_cells=True)
    rho, prs, inv = st.density(p)
    acc = st.accel(p, prs, inv)
    cnt, hsh = st.neighbour_stats(p)
    st2 = O.State(pos)
    st2.step(p, 5)
    p5, v5 = st2.original_order()
    save_if_changed(os.path.join(HERE, "oracle_regression.npz"),
                    dict(pos0=pos, keys=keys, ids=st.ids, cell_start=cs, rho=rho, prs=prs, acc=acc, nbr_count=cnt,
                         nbr_hash=hsh, pos5=p5, vel5=v5))
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
