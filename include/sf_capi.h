/*
 * sf_capi.h — C ABI of the GB300 SPH step (SimpleFluid drop-in).
 *
 * The reference drives its fluid through a C++ template class from an external
 * solver library:
 *
 *   SPHSolver<float>(std::shared_ptr<SPHParameters<float>>)   Include/QtSPHSolver.h:30-31
 *   void  SPHSolver::makeReady()                              Source/Simulator.cpp:42
 *   float SPHSolver::advanceFrame()                           Source/Simulator.cpp:49
 *   QtSPHSolver::getNumParticles/getParticles/getVelocity     Include/QtSPHSolver.h:33-35
 *   SPHParameters<float> fields + updateParams()              Source/Controller.cpp:54-63
 *   SceneManager::setupScene*(particles, velocity)            Source/SceneManager.cpp:21-173
 *
 * Every entry point below replaces one of those calls with a plain C function:
 * plain pointers and sizes, no C++ or torch types.  All functions return an
 * sf_status; on failure sf_last_error() returns a message for the calling
 * thread.  Host arrays are owned by the caller and copied in or out; the context
 * owns all device memory.  One context is driven by one host thread at a time;
 * different contexts are independent.  All device work of a context runs on its
 * own CUDA stream.
 *
 * Particle arrays at this boundary are host AoS float3 (x0 y0 z0 x1 y1 z1 ...),
 * the layout of the reference's Vec_Vec3<float> (std::vector<glm::vec3>), in the
 * caller's particle order.
 */
#ifndef SF_CAPI_H
#define SF_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define SF_API __declspec(dllexport)
#else
#define SF_API __attribute__((visibility("default")))
#endif

/* ---- status codes ------------------------------------------------------- */
typedef int sf_status;
#define SF_OK 0
#define SF_ERR_INVALID_ARGUMENT 1 /* bad pointer, size or parameter value        */
#define SF_ERR_CUDA 2             /* a CUDA runtime call failed                  */
#define SF_ERR_OUT_OF_MEMORY 3    /* device or pinned host allocation failed     */
#define SF_ERR_NOT_READY 4        /* advance before makeReady / no particles set */
#define SF_ERR_GRID_TOO_LARGE 5   /* box / kernel radius give too many cells     */
#define SF_ERR_CAPACITY 6         /* a fixed-size buffer is too small            */
#define SF_ERR_NO_DEVICE 7        /* no usable CUDA device                       */

/* ---- scenes: SimulationScenes::Scene (Include/Common.h:49-60) ------------ */
#define SF_SCENE_SPHERE_DROP 0
#define SF_SCENE_CUBE_DROP 1
#define SF_SCENE_DAMBREAK 2
#define SF_SCENE_DOUBLE_DAMBREAK 3
/* benchmark workloads (box [0,1]^3, sizes fixed by the workload definitions) */
#define SF_SCENE_DAMBREAK_16K 16        /* 20x40x20 lattice, spacing 0.02          */
#define SF_SCENE_DOUBLE_DAMBREAK_1M 17  /* two 64x128x64 jittered blocks, r=0.0025 */
#define SF_SCENE_SPHERE_POOL 18         /* pool of depth 0.3 + sphere R=0.15       */
#define SF_SCENE_DAMBREAK_64K 19        /* 32x64x32 lattice, r=0.005               */

/* ---- equation of state -------------------------------------------------- */
#define SF_EOS_LINEAR 0 /* p = k (rho - rho0)            */
#define SF_EOS_TAIT 1   /* p = k ((rho/rho0)^7 - 1)      */

/*
 * Parameter block.  The first group is SPHParameters<float> as the reference
 * GUI writes it (Source/Controller.cpp:54-61) plus particleRadius and scene
 * (Source/SceneManager.cpp:23,45); the second group holds the constants the
 * reference leaves inside its solver library, which the benchmark workloads fix.
 */
typedef struct sf_params {
    int32_t num_threads;             /* numThreads; 0 = automatic. Host-side only. */
    float kernel_radius;             /* kernelRadius h                              */
    float particle_radius;           /* particleRadius r (lattice spacing 2r)       */
    float pressure_stiffness;        /* pressureStiffness k                         */
    float boundary_restitution;      /* boundaryRestitution e in [0,1]              */
    float viscosity;                 /* viscosity mu                                */
    float stop_time;                 /* stopTime, seconds of simulated time         */
    int32_t use_attractive_pressure; /* bUseAttractivePressure: keep p < 0 if set   */
    int32_t scene;                   /* SF_SCENE_*                                  */
    float rest_density;              /* rho0                                        */
    float gravity[3];                /* body acceleration                           */
    float time_step;                 /* fixed sub-step; advanceFrame returns it     */
    float box_min[3];                /* simulation box                              */
    float box_max[3];
    int32_t eos;                     /* SF_EOS_*                                    */
    int32_t cells_per_h;             /* uniform-grid cells per kernel radius: 1, 2
                                        or 3 (0 = 2).  The neighbour search visits
                                        the (2K+1)^3 cells around a particle's cell
                                        and the summation order follows the grid,
                                        so K is part of the arithmetic.            */
    int32_t adaptive_time_step;      /* 0: every sub-step is time_step.  1: CFL
                                        sub-step dt = min(time_step,
                                        0.4 h / max|v|, 0.25 sqrt(h / max|a|)),
                                        maxima over the previous sub-step (the
                                        initial state's |v| for the first)      */
    int32_t reserved[1];             /* must be zero                                */
} sf_params;

typedef struct sf_ctx sf_ctx;

/* ---- errors / version --------------------------------------------------- */
SF_API const char* sf_last_error(void);
SF_API const char* sf_version(void);

/* ---- parameters --------------------------------------------------------- */
/* Fill with the defaults of the 16,000-particle dambreak workload. */
SF_API sf_status sf_params_default(sf_params* p);
/* SPHParameters::updateParams() (Source/Controller.cpp:63): validate. */
SF_API sf_status sf_params_update(sf_params* p);

/* ---- scenes: SceneManager::setupScene (Source/SceneManager.cpp:21-38) --- */
/* Number of particles the scene generator makes for these parameters. */
SF_API sf_status sf_scene_count(const sf_params* p, int32_t scene, uint64_t seed, uint32_t* n_out);
/* Write the scene's positions (and zero velocities) into caller arrays of
 * capacity `capacity` particles.  vel_xyz may be NULL. */
SF_API sf_status sf_setup_scene(const sf_params* p, int32_t scene, uint64_t seed, float* pos_xyz,
                                float* vel_xyz, uint32_t capacity, uint32_t* n_out);

/* ---- device selection ----------------------------------------------------
 * Make `device` current for the calling thread; contexts created afterwards on
 * this thread live on it (default: the thread's current device, normally 0). */
SF_API sf_status sf_select_device(int32_t device);

/* ---- solver lifetime: SPHSolver<float>(params) -------------------------- */
SF_API sf_status sf_create(const sf_params* p, sf_ctx** out);
SF_API sf_status sf_destroy(sf_ctx* ctx);
SF_API sf_status sf_set_params(sf_ctx* ctx, const sf_params* p);
SF_API sf_status sf_get_params(const sf_ctx* ctx, sf_params* p);

/* ---- particle state: getParticles() / getVelocity() --------------------- */
/* Copy a host AoS float3 state in (n * 3 floats each).  vel_xyz may be NULL
 * (zero velocity).  Page-locked arrays (sf_host_alloc) are copied by DMA, the
 * velocities while the positions are sorted; the call returns once both
 * copies are done, with the sort still running on the context's stream
 * (later calls queue behind it).  Pageable arrays are read by the GPU in place
 * where it accesses pageable memory through the host's page tables (Grace:
 * NVLink-C2C), else staged through a page-locked buffer.  Either way the
 * caller may reuse its arrays once the call returns. */
SF_API sf_status sf_set_state(sf_ctx* ctx, const float* pos_xyz, const float* vel_xyz, uint32_t n);
/* Copy the state out in the caller's original particle order.  Either output
 * may be NULL.  Page-locked arrays are filled by DMA; pageable ones are
 * written by the GPU in place where it can, else through staging.  Waits for
 * the context's stream. */
SF_API sf_status sf_get_state(sf_ctx* ctx, float* pos_xyz, float* vel_xyz, uint32_t n);
/* getNumParticles() */
SF_API sf_status sf_get_num_particles(const sf_ctx* ctx, uint32_t* n_out);

/* ---- particle state in device memory (no host round trip) ----------------
 * The same state transfers with AoS float3 arrays that live in device memory
 * of the context's GPU (cudaMalloc'd, or a framework tensor's storage).  Both
 * are ordered on the context's stream and do not wait on the host.  `other`
 * is the caller's cudaStream_t (as void*, NULL for none; the default stream
 * is cudaStreamLegacy or cudaStreamPerThread, not NULL): set_state waits for
 * the work already queued on it before reading, and get_state makes work
 * queued on it afterwards wait for the written arrays.  A pointer that is not
 * device memory of this GPU is rejected with SF_ERR_INVALID_ARGUMENT. */
SF_API sf_status sf_set_state_device(sf_ctx* ctx, const float* d_pos_xyz, const float* d_vel_xyz, uint32_t n,
                                     void* other);
SF_API sf_status sf_get_state_device(sf_ctx* ctx, float* d_pos_xyz, float* d_vel_xyz, uint32_t n, void* other);

/* Device views of the solver's working arrays, in its cell-sorted order:
 *   pos4      float4 per particle: x, y, z, and in w the bit pattern of the
 *             particle's caller index (uint32);
 *   vel4      float4 per particle: vx, vy, vz, 0;
 *   rho       density of the last density pass;
 *   p_inv_rho float2 per particle: pressure and 1/rho of that pass;
 *   cell_start ncells + 1 entries: the particles of cell c are
 *             [cell_start[c], cell_start[c+1]).
 * The pointers stay valid until the particle count changes or the context is
 * destroyed; their contents change with every step.  Reads must be ordered
 * after the context's stream (`stream`). */
typedef struct sf_device_view {
    const float* pos4;
    const float* vel4;
    const float* rho;
    const float* p_inv_rho;
    const uint32_t* cell_start;
    uint32_t n;
    uint32_t ncells;
    void* stream;
} sf_device_view;
SF_API sf_status sf_device_state(sf_ctx* ctx, sf_device_view* view);

/* ---- stepping: makeReady() / advanceFrame() ----------------------------- */
/* Build the uniform grid, sort the particles and capture the step graph. */
SF_API sf_status sf_make_ready(sf_ctx* ctx);
/* One sub-step; *dt_out receives the simulated time advanced.  With a fixed
 * time step the work is queued and the call does not wait; with the adaptive
 * step it waits to read the sub-step's dt (pass NULL to skip the wait). */
SF_API sf_status sf_advance_frame(sf_ctx* ctx, float* dt_out);
/* Whole frames on the device: per frame, sub-steps are taken until their dt,
 * summed in float, reach frame_time (the loop of Source/Simulator.cpp:46-51,
 * frame_time 0.0333333333) or max_substeps were taken.  Each frame is one CUDA
 * graph launch whose sub-step loop is a device-side conditional while node.
 * Waits; reports the simulated time and the sub-steps taken in total. */
SF_API sf_status sf_advance_frames(sf_ctx* ctx, uint32_t frames, double frame_time, uint32_t max_substeps,
                                   double* sim_time_out, uint32_t* substeps_out);
/* `nsteps` sub-steps, queued as replays of one captured step graph. */
SF_API sf_status sf_step(sf_ctx* ctx, uint32_t nsteps);
/* Wait for all queued work of the context. */
SF_API sf_status sf_synchronize(sf_ctx* ctx);
/* The context's cudaStream_t, as void*. */
SF_API sf_status sf_get_stream(sf_ctx* ctx, void** stream_out);

/* ---- pinned host buffers (optional; makes sf_set_state/sf_get_state DMA) - */
SF_API sf_status sf_host_alloc(size_t bytes, void** ptr_out);
SF_API sf_status sf_host_free(void* ptr);

/* ---- inspection of the solver's internal (cell-sorted) order ------------
 * These expose the neighbour-search structures so that callers and tests
 * can check them; they wait for the stream. */
/* Grid dimensions (cells per axis) of the context's uniform grid. */
SF_API sf_status sf_get_grid(const sf_ctx* ctx, uint32_t dims_out[3]);
/* Sorted state: pos4/vel4 are n*4 floats (w of pos4 is 0), ids are the
 * caller's original indices, keys the linear cell keys.  Any may be NULL. */
SF_API sf_status sf_get_sorted(sf_ctx* ctx, float* pos4, float* vel4, uint32_t* ids, uint32_t* keys,
                               uint32_t n);
/* cell_start has ncells+1 entries: particles of cell c are [cs[c], cs[c+1]). */
SF_API sf_status sf_get_cell_start(sf_ctx* ctx, uint32_t* cell_start, uint32_t count);
/* Run the density pass on the current sorted state and return rho and p in
 * sorted order.  Either output may be NULL. */
SF_API sf_status sf_compute_density(sf_ctx* ctx, float* rho, float* pressure, uint32_t n);
/* Run density + forces on the current sorted state without integrating and
 * return the acceleration (n*3 floats, sorted order). */
SF_API sf_status sf_compute_accel(sf_ctx* ctx, float* accel_xyz, uint32_t n);
/* Per sorted particle: number of neighbours j != i with |xi-xj|^2 < h^2 and a
 * order-independent hash of their original indices. */
SF_API sf_status sf_neighbour_stats(sf_ctx* ctx, uint32_t* count, uint32_t* hash, uint32_t n);

/* ---- failure detection: invariants of the current state -------------------
 * Counted on the GPU over the cell-sorted state; a healthy state has every
 * count zero except possibly list_overflow.  Waits for the stream. */
typedef struct sf_state_report {
    uint32_t n;                   /* particles                                       */
    uint32_t non_finite;          /* NaN or Inf in a position or velocity            */
    uint32_t outside_box;         /* outside [box_min + r, box_max - r] (only before
                                     the first step after an upload)                 */
    uint32_t unsorted;            /* sorted neighbours whose cell keys decrease      */
    uint32_t cell_table_mismatch; /* particles outside their cell's table range      */
    uint32_t bad_ids;             /* caller indices out of range, repeated or absent */
    uint32_t list_overflow;       /* neighbour lists of the last density pass that
                                     exceeded their capacity (rescanned, correct)    */
    float max_speed;              /* max |v| over finite particles                   */
} sf_state_report;
SF_API sf_status sf_check_state(sf_ctx* ctx, sf_state_report* report);

/* ---- index checks (checked build) -----------------------------------------
 * The checked build of this library (compiled with SF_DEVICE_CHECKS=1; see
 * simplefluid_gb300/build.py) checks every cell-table range end and every
 * neighbour-list entry on the device before it is used; a bad value is
 * counted and replaced by an in-range one (nothing traps).  *failures
 * receives the count on the current device since the last reset, and
 * *compiled_in whether this build has the checks (0: the release build,
 * *failures = 0).  A non-zero `reset` clears the count.  Either output may be
 * null. */
SF_API sf_status sf_index_checks(int32_t reset, uint64_t* failures, int32_t* compiled_in);

/* ---- fault injection (tests) ---------------------------------------------
 * The device allocation `after` allocations from now (0: the next one) fails
 * as out of memory, once; a negative value disarms it.  The call that hits it
 * returns SF_ERR_OUT_OF_MEMORY and releases what it had allocated: the
 * context stays usable and may need a new sf_set_state. */
SF_API sf_status sf_test_fail_allocation(int64_t after);

/* ---- kernel tuning -----------------------------------------------------------
 * Implementation choices of a context's step.  Every choice computes the same
 * bits; they differ only in speed.  Not part of the reference interface. */
#define SF_LIST_NONE 0        /* force pass rescans the candidate cells       */
#define SF_LIST_TILE_STAGED 1 /* density pass stages neighbour lists in shared
                                 memory, writes 128-particle tiles             */
#define SF_LIST_TILE 2        /* direct stores, 128-particle tiles             */
#define SF_LIST_TILE16 3      /* direct stores of 16-bit entries (the low half
                                 of the neighbour's index, exact within
                                 +-32767 sorted places) in 32-particle tiles; a
                                 tile whose candidate span is wider stores
                                 32-bit entries instead                        */
typedef struct sf_tuning {
    int32_t list_mode;     /* SF_LIST_*                                       */
    int32_t density_block; /* threads per block of the density pass: 128, 256 */
    int32_t force_block;   /* threads per block of the force pass: 128, 256   */
    int32_t prefetch;      /* neighbours gathered per batch: 2 or 4           */
    int32_t l2_window;     /* 1: the force pass's gather records are kept in
                              L2 with a persisting access-policy window on the
                              density and force launches; 0: no window       */
    int32_t batch_cluster; /* batches only.  0: each step is five launches
                              over all scenes' particles.  2, 4 or 8: each step
                              is one persistent launch of thread-block
                              clusters of that many blocks; a cluster takes
                              whole scenes, largest first, and runs their five
                              stages between cluster barriers (needs
                              SF_LIST_TILE; the other fields then do not
                              apply).  Both compute the same bits.           */
    int32_t batch_block;   /* threads per block of the persistent step: 256,
                              512 or 1024 (0 is taken as 256)                */
    int32_t reserved[1];   /* must be zero                                    */
} sf_tuning;
SF_API sf_status sf_get_tuning(const sf_ctx* ctx, sf_tuning* t);
SF_API sf_status sf_set_tuning(sf_ctx* ctx, const sf_tuning* t);

/* ---- measurement ----------------------------------------------------------
 * Device-side timing with CUDA events on the context's stream.  Not part of
 * the reference interface (which has none); used by benchmarks. */
/* Run `nsteps` sub-steps (graph replays).  With flush_bytes > 0 a scratch
 * buffer of that size is overwritten before every step, outside the timed
 * intervals, to evict the L2 cache.  *total_ms receives the summed device time
 * of the steps; step_ms (may be NULL) receives each step's time. */
SF_API sf_status sf_step_timed(sf_ctx* ctx, uint32_t nsteps, uint64_t flush_bytes, float* total_ms,
                               float* step_ms);
/* Number of kernel stages in one sub-step and their names. */
SF_API uint32_t sf_stage_count(void);
SF_API const char* sf_stage_name(uint32_t stage);
/* Run `nsteps` sub-steps stage by stage (no graph) with an event between
 * stages; stage_ms[s] receives the summed device time of stage s over all
 * steps (nstages must equal sf_stage_count()). */
SF_API sf_status sf_profile_steps(sf_ctx* ctx, uint32_t nsteps, uint64_t flush_bytes, float* stage_ms,
                                  uint32_t nstages);

/* ---- headless particle rendering ------------------------------------------------
 * The arithmetic of the reference's point-sprite sphere impostors
 * (Shaders/particle.vs.glsl: eye-space position, gl_PointSize = radius *
 * scale / distance; Shaders/particle.fs.glsl: disc test on gl_PointCoord,
 * impostor normal, fragment position, Blinn-Phong over up to 8 point lights)
 * evaluated by CUDA kernels into a device image, without a graphics API.
 * Visibility: per pixel the fragment with the smallest window depth of its
 * particle's centre wins (ties: lower particle index), as a depth test on
 * point sprites without depth correction does.  Image rows run top to bottom. */
#define SF_COLOR_UNIFORM 0 /* material diffuse                                 */
#define SF_COLOR_RANDOM 1  /* per-particle colour, uniform in [0,1]^3 from seed */
#define SF_COLOR_RAMP 2    /* by particle index along PARTICLE_COLOR_RAMP        */
typedef struct sf_render_params {
    int32_t width, height;
    float eye[3], focus[3], up[3]; /* camera: DEFAULT_CAMERA_POSITION/FOCUS, +y up */
    float fovy_deg, znear, zfar;   /* perspective projection (fovy 55 deg)          */
    float point_radius;            /* u_PointRadius; 0 = the particle radius         */
    int32_t num_lights;            /* 1..8                                           */
    float light_position[8][4];    /* used as given, like the shader does            */
    float light_ambient[8][4], light_diffuse[8][4], light_specular[8][4];
    float mat_ambient[4], mat_diffuse[4], mat_specular[4];
    float mat_shininess;
    int32_t color_mode;            /* SF_COLOR_*                                     */
    uint64_t color_seed;
    float background[4];
    int32_t reserved[4];
} sf_render_params;
/* The reference viewer's settings: 1200 x 1000, camera (-3, 0.8, 0) looking at
 * (0, -0.2, 0), fovy 55, one light at (-10, 10, 10), CUSTOM_PARTICLE_MATERIAL. */
SF_API sf_status sf_render_params_default(sf_render_params* rp);
/* Render the current particles.  rgba_out: width*height*4 floats, depth_out:
 * width*height floats (1 where empty), owner_out: width*height u32 particle
 * indices in the caller's order (0xffffffff where empty); any may be NULL. */
SF_API sf_status sf_render(sf_ctx* ctx, const sf_render_params* rp, float* rgba_out, float* depth_out,
                           uint32_t* owner_out);

/* ---- state files -------------------------------------------------------------
 * Not in the reference (it only exports screenshots, Source/MainWindow.cpp:108-113).
 * A state file holds the parameters, the caller's simulated time and the
 * particles in the solver's cell-sorted order with their indices; loading it
 * (parameters included) and stepping reproduces the saved run bit for bit.
 * Layout: "SFSTATE1", u32 version (1), u32 n, f64 sim_time, sf_params,
 * n x 3 f32 positions, n x 3 f32 velocities, n u32 caller indices. */
SF_API sf_status sf_save_state(sf_ctx* ctx, const char* path, double sim_time);
SF_API sf_status sf_load_state(sf_ctx* ctx, const char* path, double* sim_time_out);

/* ---- differentiation -------------------------------------------------------
 * Not in the reference.  A hand-written adjoint of the sub-step (density, EOS,
 * forces, integration and box), with each step's neighbour structure held
 * fixed.  sf_forward advances like sf_step and records checkpoints of the
 * state every `ckpt_every` steps; sf_adjoint re-runs each segment forward from
 * its checkpoint (recomputing neighbour lists and states) and propagates the
 * given adjoint of the final state back to the state at the sf_forward call,
 * plus the gradients with respect to viscosity and stiffness.  Memory is the
 * checkpoints (32 B per particle each) plus one segment of step records.
 * All arrays are host AoS float3 in the caller's particle order; inputs may be
 * NULL (zero), outputs may be NULL (not returned).  The particle state after
 * sf_adjoint is the state sf_forward ended with. */
SF_API sf_status sf_forward(sf_ctx* ctx, uint32_t nsteps, uint32_t ckpt_every);
SF_API sf_status sf_adjoint(sf_ctx* ctx, const float* dloss_dx, const float* dloss_dv, float* dloss_dx0,
                            float* dloss_dv0, float* dloss_dviscosity, float* dloss_dstiffness);
/* Measurement of the adjoint (not in the reference; for benchmarks): after
 * sf_adjoint, re-runs the reverse sweep of the trajectory's first segment pass
 * by pass with an event between passes; pass_ms[p] receives pass p's device
 * time summed over the segment's steps (npasses must equal
 * sf_adjoint_pass_count()), *steps_out (may be NULL) the number of steps.
 * It overwrites the adjoint's working buffers: the gradients sf_adjoint
 * returned are unaffected, and the next sf_adjoint starts afresh. */
SF_API uint32_t sf_adjoint_pass_count(void);
SF_API const char* sf_adjoint_pass_name(uint32_t pass);
SF_API sf_status sf_adjoint_profile(sf_ctx* ctx, float* pass_ms, uint32_t npasses, uint32_t* steps_out);
/* Loss = sum over res^3 cells of (H_c - target_c)^2, H the cloud-in-cell
 * histogram of the current positions on cell-centred bins over the box,
 * normalised by the particle count (accumulated in 2^-32 fixed point, so it
 * does not depend on summation order; the loss is returned in double);
 * dloss_dx (may be NULL) receives dL/dx. */
SF_API sf_status sf_loss_histogram(sf_ctx* ctx, const float* target, uint32_t res, double* loss_out, float* dloss_dx);

/* ---- batches of independent scenes -------------------------------------
 * Not in the reference (which runs one scene): many independent scenes of
 * uneven size, each with its own parameters and box, advanced together — one
 * CUDA-graph launch per step covers every scene.  Scenes must share
 * cells_per_h (1 or 2).  Particle arrays are the scenes' particles
 * concatenated in scene order, host AoS float3. */
typedef struct sf_batch sf_batch;
/* The batched-cube workload: nscenes scenes drawn from `seed` (counts
 * log-uniform in [2000, 65536], viscosity U[0.005, 0.05], stiffness
 * U[20, 100]); a falling lattice block centred in a box of twice its size.
 * Call with pos_xyz = NULL to learn *total_out first. */
SF_API sf_status sf_batch_cubes(uint64_t seed, uint32_t nscenes, const sf_params* base, sf_params* params_out,
                                uint32_t* counts_out, float* pos_xyz, uint64_t capacity, uint64_t* total_out);
SF_API sf_status sf_batch_create(const sf_params* per_scene, uint32_t nscenes, sf_batch** out);
SF_API sf_status sf_batch_destroy(sf_batch* b);
SF_API sf_status sf_batch_num_scenes(const sf_batch* b, uint32_t* n_out);
SF_API sf_status sf_batch_get_params(const sf_batch* b, uint32_t scene, sf_params* p);
SF_API sf_status sf_batch_set_state(sf_batch* b, const uint32_t* counts, const float* pos_xyz, const float* vel_xyz);
SF_API sf_status sf_batch_get_state(sf_batch* b, float* pos_xyz, float* vel_xyz, uint32_t n);
SF_API sf_status sf_batch_num_particles(const sf_batch* b, uint32_t* n_out);
/* `nsteps` sub-steps of every scene: one graph launch per step. */
SF_API sf_status sf_batch_step(sf_batch* b, uint32_t nsteps);
/* sf_check_state over all scenes of the batch. */
SF_API sf_status sf_batch_check_state(sf_batch* b, sf_state_report* report);
SF_API sf_status sf_batch_synchronize(sf_batch* b);
SF_API sf_status sf_batch_step_timed(sf_batch* b, uint32_t nsteps, uint64_t flush_bytes, float* total_ms,
                                     float* step_ms);
SF_API sf_status sf_batch_get_tuning(const sf_batch* b, sf_tuning* t);
SF_API sf_status sf_batch_set_tuning(sf_batch* b, const sf_tuning* t);
/* Re-grid every scene with K cells per kernel radius (1 or 2). */
SF_API sf_status sf_batch_set_cells_per_h(sf_batch* b, int32_t cells_per_h);
/* Autotuner: try every grid granularity and kernel variant for `trial_steps`
 * steps from the current state, keep the fastest, restore the state. */
SF_API sf_status sf_batch_autotune(sf_batch* b, uint32_t trial_steps, sf_tuning* chosen, int32_t* chosen_cells_per_h,
                                   float* chosen_ms_per_step);

/* ---- allocation-free density ----------------------------------------------
 * No counterpart in the reference: an addition of this library for callers
 * that cannot allocate device memory (an application or plugin that owns a
 * fixed device-memory budget, a real-time loop where an allocation may block
 * or fail).  Computes rho and p (equation of state of `p`) of n particles whose
 * AoS float3 positions are in device memory, writing device outputs in the
 * caller's particle order; either output may be NULL, not both.  Work is
 * queued on `stream` (a cudaStream_t; NULL = default stream) and not waited
 * for.  Calls no allocator: the grid sort runs in one fixed static device
 * array (about 7.6 MB, held by every GPU that loads the library until exit),
 * which limits a call to 65,536 particles and 262,144 grid cells; larger
 * requests fail with SF_ERR_CAPACITY before any GPU work.  All calls share that
 * array: calls whose GPU work overlaps race, so serialise them on one stream.
 * The first call on a device looks up the array's address; make it before any
 * stream capture. */
SF_API sf_status sf_density_noalloc(const sf_params* p, const float* d_pos_xyz, uint32_t n, float* d_rho,
                                    float* d_pressure, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SF_CAPI_H */
