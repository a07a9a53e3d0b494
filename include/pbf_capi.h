/*
 * pbf_capi.h — C-ABI of the GB300 PBF substep pipeline.
 *
 * The reference drives this path through the C++ class `Simulation`
 * (src/Simulation.hpp:28-151) and the global `Parameters Params` with its
 * loader `LoadParameters` (src/ParamUtils.hpp, src/ParamUtils.cpp:19-100).
 * Every entry point below replaces one of those members; the citation on each
 * names the member it stands in for.
 *
 * Conventions
 *   - Every function returns an int status: PBF_OK (0) or a negative PBF_ERR_*.
 *     `pbf_last_error(ctx)` returns the message of the last failure on that
 *     context (ctx == NULL: the last failure of a call that had no context).
 *     No C++ exception crosses this boundary.
 *   - Particle arrays are float4 records (x, y, z, w) stored as 4 consecutive
 *     floats, `particleCount` records long, in host memory unless a name says
 *     `device`.
 *   - The handle is opaque; the library owns all device memory of a context.
 *   - One CUDA stream per context; calls on one context are not re-entrant,
 *     contexts on different host threads are independent.
 */
#ifndef PBF_CAPI_H
#define PBF_CAPI_H

#include <stddef.h>
#include <stdint.h>
#include "pbf_params.h"

#ifdef __cplusplus
extern "C" {
#endif

#define PBF_OK                 0
#define PBF_ERR_INVALID       -1   /* bad argument or parameter value        */
#define PBF_ERR_CUDA          -2   /* a CUDA runtime call failed             */
#define PBF_ERR_STATE         -3   /* call out of order (e.g. step before init) */
#define PBF_ERR_UNSUPPORTED   -4   /* feature of the reference not built here */
#define PBF_ERR_DEVICE_FLAG   -5   /* a kernel raised its error word          */
#define PBF_ERR_NO_DEVICE     -6   /* no usable CUDA device                   */

typedef struct pbf_ctx pbf_ctx;

/* ---------------------------------------------------------------- params -- */

/* Zero-filled parameters with the loader's computed fields applied
   (h_2 = h*h, friendsCircles = 5, particlesPerCircle = 50).
   Replaces the zero-initialised global `Parameters Params`
   (src/ParamUtils.cpp:19). */
int pbf_default_parameters(PbfParameters* out);

/* Parse `.par` text into *inout, updating only the keys present, then apply
   the computed fields.  Same grammar and error behaviour as
   `LoadParameters(string)` (src/ParamUtils.cpp:24-100): one `key value` per
   line, `#` starts a comment, keys case-insensitive, unknown keys reported on
   stderr and ignored, and a final line with no trailing newline is dropped
   with "Error parsing parameters file".  Extra keys accepted here:
   gravityx / gravityy / gravityz (any of them enables the gravity vector),
   boxclamp, zerodistanceguard and relaxedmath.  Returns the number of unknown keys through *unknown (may be NULL). */
int pbf_load_parameters(const char* text, PbfParameters* inout, int* unknown);

/* The scene keys of `.par` text (BlockDims, BlockOrigin, Jitter, Seed) into
   *scene; PBF_ERR_INVALID without a BlockDims line.  pbf_load_parameters
   accepts these keys silently. */
int pbf_load_scene(const char* text, PbfScene* scene);

/* The scene's nx*ny*nz particles (4 floats each, x fastest): lattice spacing
   p->h * p->setupSpacing from blockOrigin, each coordinate jittered by
   U(-jitter, jitter) from a 64-bit Mersenne Twister seeded with seed. */
int pbf_scene_positions(const PbfParameters* p, const PbfScene* scene, float* pos);

/* -------------------------------------------------------------- lifetime -- */

/* Create a context on CUDA device `device`.
   Replaces Simulation::Simulation(const cl::Context&, const cl::Device&)
   (src/Simulation.cpp:56-63): the in-order profiling queue becomes one CUDA
   stream. */
int pbf_create(const PbfParameters* params, int device, pbf_ctx** out);

/* Release every device allocation of the context.
   Replaces Simulation::~Simulation (src/Simulation.cpp:65-69). */
int pbf_destroy(pbf_ctx* ctx);

/* Message of the last failure (never NULL). */
const char* pbf_last_error(const pbf_ctx* ctx);

/* ------------------------------------------------------ init (reference) -- */

/* Allocate the particle buffers for params.particleCount particles and load
   the initial state.  init_pos == NULL: the reference's CreateParticles
   lattice (src/Simulation.cpp:71-101); init_vel == NULL: zero velocities.
   Replaces Simulation::InitBuffers (src/Simulation.cpp:206-244). */
int pbf_init_buffers(pbf_ctx* ctx, const float* init_pos, const float* init_vel);

/* Allocate the cell table (gridBufSize entries, every entry 0xFFFFFFFF) and
   the neighbour ("friends") list storage.
   Replaces Simulation::InitCells (src/Simulation.cpp:246-255). */
int pbf_init_cells(pbf_ctx* ctx);

/* Load the force-plane mask image: width x height texels, row-major, one
   uint32 per texel (the R channel the reference keeps, CL_R /
   CL_UNSIGNED_INT32, with nearest sampling clamped to the edge).  mask ==
   NULL loads the empty mask, for which every force plane is the identity
   (compute_delta.cl:33-38).
   Replaces Simulation::LoadForceMasks (src/Simulation.cpp:257-281), which
   reads the mask from Scene_fp_mask.png. */
int pbf_load_force_masks(pbf_ctx* ctx, const uint32_t* mask, int width, int height);

/* Set the force planes of the delta-p stage (at most PBF_MAX_FORCE_QUADS;
   count 0 removes them).  They are applied in order to the updated position
   of every particle of every solver iteration, after the position update
   and before the box clamp, with the reference's noise edge offset
   1 + (3 + sin(5x/h) + sin(5y/h) + sin(5z/h)) h 0.03 (compute_delta.cl:157-161).
   The sine is the library's own FP32 definition (the oracle holds the same
   one), so results are reproducible across host and device.
   The reference hard-codes its 14 planes (compute_delta.cl:169-182); here
   they are data.  Rollouts reject contexts with force planes. */
int pbf_set_force_quads(pbf_ctx* ctx, const PbfForceQuad* quads, int count);

/* The wave generator as a moving wall: with boxClamp, the clamp's low x bound
   becomes xMin + wavePos for the steps enqueued after this call.  The
   reference computes wavePos every frame (src/Runner.cpp:100-116) and passes
   it to computeDelta (src/Simulation.cpp:421, fWavePos), whose kernel does
   not read it (compute_delta.cl:50).  wavePos must be >= 0. */
int pbf_set_wave_position(pbf_ctx* ctx, float wavePos);

/* The reference's wave position at `waveTime` seconds of generation
   (src/Runner.cpp:103-107): (1 - cos(2 pi fmod(waveGenFreq t, 1)^waveGenDuty))
   * waveGenAmp (xMax - xMin) / 2, evaluated in double.  The caller advances
   waveTime by timeStep per frame while waves are generated (:110-111). */
float pbf_wave_position(const PbfParameters* p, float waveTime);

/* Validate the parameters against the allocated buffers and prepare the
   launch plan (sort passes, grid shapes).  Returns PBF_ERR_INVALID where the
   reference's InitKernels would have failed to build.
   Replaces bool Simulation::InitKernels (src/Simulation.cpp:129-204). */
int pbf_init_kernels(pbf_ctx* ctx);

/* Replace the parameters of an initialised context (same particleCount and
   gridBufSize).  Stands in for the reference's reload of `Params` followed by
   the re-upload at src/Simulation.cpp:243. */
int pbf_set_params(pbf_ctx* ctx, const PbfParameters* params);

/* Simulation::bPauseSim (src/Simulation.hpp:146): when set, a step adds no
   gravity and skips the sort (src/Simulation.cpp:563-567). */
int pbf_set_pause(pbf_ctx* ctx, int paused);

/* ------------------------------------------------------------------ step -- */

/* Run Simulation::Step() (src/Simulation.cpp:554-621) `substeps` times and
   wait for the device.  Each substep uses the full params.timeStep, as the
   reference's frame loop does (src/Runner.cpp:124-130). */
int pbf_step(pbf_ctx* ctx, int substeps);

/* As pbf_step, but only enqueues the work on the context's stream. */
int pbf_step_async(pbf_ctx* ctx, int substeps);

/* Wait for all work enqueued on the context's stream; reports a kernel error
   word raised since the last check as PBF_ERR_DEVICE_FLAG. */
int pbf_synchronize(pbf_ctx* ctx);

/* ----------------------------------------------------------------- state -- */

/* Copy the current state to host memory (any pointer may be NULL):
   positions (w = |v|, update_velocities.cl:14), velocities, and predicted
   positions (w = density after a step, pack_data.cl with the density source).
   Replaces reading the GL-shared position buffers the renderer draws. */
int pbf_read_state(pbf_ctx* ctx, float* pos, float* vel, float* pred);

/* Save the particle state (positions, velocities, particle ids, and the
   parameters it ran with) to a binary file: "PBFSTATE", uint32 version 1,
   uint32 N, uint32 sizeof(PbfParameters), PbfParameters, N float4
   positions, N float4 velocities, N uint32 ids, host byte order.  Stepping a
   context after pbf_load_state of a saved file gives the same results, bit
   for bit, as stepping the context that saved it.  Replaces the reference's
   buffer dumps (SaveFile, src/Simulation.cpp:287-313) and its unfinished
   particle dump (bDumpParticlesData, :605-611). */
int pbf_save_state(pbf_ctx* ctx, const char* path);

/* Restore a state saved by pbf_save_state into a context with the same N;
   the context keeps its own parameters. */
int pbf_load_state(pbf_ctx* ctx, const char* path);

/* Overwrite positions and velocities from host memory (either may be NULL).
   Writing positions renumbers the particles: record k becomes particle k
   (pbf_read_ids). */
int pbf_write_state(pbf_ctx* ctx, const float* pos, const float* vel);

/* pbf_write_state / pbf_read_state enqueued on the context's stream without
   waiting: with page-locked host memory the copies run in stream order with
   the steps around them, and pbf_synchronize waits for all of it (a frame
   loop: write_async, step_async, read_async, synchronize).  The host memory
   must stay valid until then. */
int pbf_write_state_async(pbf_ctx* ctx, const float* pos, const float* vel);
int pbf_read_state_async(pbf_ctx* ctx, float* pos, float* vel, float* pred);

/* pbf_step_async(substeps) followed by pbf_read_state_async(pos, vel, NULL),
   with the same results, but the position copy overlaps the last substep:
   positions are final after updateVelocities (update_velocities.cl), so they
   are copied on a second stream while applyViscosity and applyVorticity run.
   With both pointers given, applyVorticity runs in two launches over the two
   halves of the particles, and the first half's velocities are copied while
   the second half runs; the rest follows it.  The reference's frame loop
   (src/Runner.cpp:118-130) steps and then hands positions to the renderer;
   this call is that frame for a host-memory consumer.  Either pointer may be
   NULL; page-locked memory is needed for the overlap.  With stage timing on,
   the copies follow the step. */
int pbf_step_read_async(pbf_ctx* ctx, int substeps, float* pos, float* vel);

/* Device address of the current positions (float4 x particleCount), valid
   until the next step.  Headless replacement of the GL buffer IDs
   mSharedPingBufferID / mSharedPongBufferID (src/Simulation.hpp:130-135). */
int pbf_device_positions(pbf_ctx* ctx, void** dptr);

/* The context's CUDA stream (a cudaStream_t), for callers that time or order
   work against it. */
int pbf_get_stream(pbf_ctx* ctx, void** stream);

/* ----------------------------------------------------------- parity hooks -- */

/* From the predicted positions `pred` (host), run the key / sort / cell-table
   stages alone and copy out
     keys  : IntCeil(N, 2048) sorted keys, padding entries 2147483646
             (radixsort.cl:1-20, Simulation.cpp:223),
     perm  : the same length, the sort permutation,
     cells : 2 * gridBufSize words, start / inclusive end per hash,
             0xFFFFFFFF for empty hashes (update_cells.cl:1-26).
   Any output may be NULL.  The context's particle state is not changed. */
int pbf_sort_state(pbf_ctx* ctx, const float* pred,
                   uint32_t* keys, uint32_t* perm, uint32_t* cells);

/* Sort state of the last substep, as the pipeline left it (the reference
   keeps it in its sort and cell buffers after Step, src/Simulation.cpp:
   466-536): the sorted keys and permutation (IntCeil(N, 2048) entries each,
   the tail padded with 2147483646 and the identity as radixsort.cl:17 pads
   it) and the cell table updateCells builds from those keys (2 *
   gridBufSize words, x the scenes of a batch).  A parity hook: the keys and
   permutation are copied from the sort's own buffers; the cell table, which
   the substep resets after the friends build, is rebuilt from them by the
   same kernel and reset again.  Any output may be NULL; the particle state
   is not changed. */
int pbf_read_sort(pbf_ctx* ctx, uint32_t* keys, uint32_t* perm, uint32_t* cells);

/* Neighbour ("friends") list of the last substep, as used by the solver:
   counts[2*i+0] = entries used by computeScaling (circles kept while
   processed/total <= 0.6, compute_scaling.cl:47-54), counts[2*i+1] = entries
   used by computeDelta / applyViscosity / applyVorticity (<= 0.5,
   compute_delta.cl:97-104); list[s * N + i] = s-th neighbour of particle i in
   circle-major order (build_friends_list.cl:74-94).  `list_slots` is the
   number of slots the caller's list buffer holds per particle; entries beyond
   it are not copied.  Either pointer may be NULL. */
int pbf_read_friends(pbf_ctx* ctx, uint32_t* counts, uint32_t* list, int list_slots);

/* ------------------------------------------------------------ diagnostics -- */

/* Per-stage device times of the last pbf_step with stage timing enabled, in
   milliseconds, under the reference tracker names (OCLPerfMon usage in
   src/Simulation.cpp:315-535).  names receives a '\n'-separated list. */
int pbf_enable_stage_timing(pbf_ctx* ctx, int enable);
int pbf_stage_timings(pbf_ctx* ctx, float* ms, int capacity, int* count,
                      char* names, size_t names_len);

/* NVTX ranges (named as the trackers) around the stages of every substep
   enqueued eagerly (stage timing on, or graphs off), for nsys / ncu
   --nvtx-include.  Header-only NVTX: a no-op without a profiler attached. */
int pbf_enable_nvtx(pbf_ctx* ctx, int enable);

/* One performance tracker, the fields of the reference's
   PM_PERFORMANCE_TRACKER (src/OCLPerfMon.h) without the OpenCL event.
   Trackers are named as OCLPerfMon::GetTrackerEvent names them: the stage,
   with "_<iteration>" for the per-iteration stages (computeScaling_0, ...).
   A stage here may cover several reference kernels: predictPositions also
   computes the keys, radixsort is the whole sort, computeScaling_i includes
   packData_i and computeDelta_i includes updatePredicted_i. */
typedef struct PbfPerfTracker {
    char     eventName[48];
    uint64_t time_start;  /* ns since pbf_enable_stage_timing turned timing on */
    uint64_t time_end;
    double   total_time;  /* ms: current * 0.5 + last_time * 0.5 (OCLPerfMon::UpdateTimings) */
    double   last_time;   /* ms */
} PbfPerfTracker;

/* The trackers in order of first use (the order the reference's UI draws
   them, src/UIManager.cpp:185-215), updated after every timed step.
   Replaces PerfData.Trackers (src/Simulation.hpp, OCLPerfMon). */
int pbf_perf_trackers(pbf_ctx* ctx, PbfPerfTracker* out, int capacity, int* count);

/* The trackers as one JSON object for dashboards: {"trackers": [{"eventName",
   "time_start", "time_end", "total_time", "last_time"}, ...], "total_time",
   "unit": "ms"}.  *length receives the size needed including the NUL; buf
   (capacity bytes) receives as much as fits. */
int pbf_perf_export_json(pbf_ctx* ctx, char* buf, size_t capacity, size_t* length);

/* Number of kernels this context has launched so far (graph nodes counted
   one by one). */
int pbf_launch_count(pbf_ctx* ctx, uint64_t* count);

/* Use (1) or stop using (0) a captured CUDA graph for each substep. */
int pbf_use_graph(pbf_ctx* ctx, int enable);

/* ------------------------------------------------ allocation-free variant -- */

/* Largest particle count pbf_sort_state_noalloc accepts, and the size of the
   fixed working array it keeps on every GPU that loads this library (held
   until the process exits). */
#define PBF_NOALLOC_MAX_KEYS       (1u << 20)
#define PBF_NOALLOC_SCRATCH_BYTES  8913920u   /* 8.5 MiB + 1 KiB */

/* The key / sort / cell-table stage of pbf_sort_state for callers that may
   not allocate device memory: hosts that reserve all device memory at start-up
   and forbid allocations afterwards (real-time frame loops, engines that own
   the GPU's memory budget).  It has no counterpart in the reference.

   Every pointer is a device address on the calling thread's current device:
     d_pred  : float4 x params->particleCount predicted positions (input,
               16-byte aligned),
     d_keys  : params->particleCount sorted keys (output, no padding entries),
     d_perm  : params->particleCount sort permutation (output),
     d_cells : 2 * params->gridBufSize words of cell table (output; may be NULL);
   the last three 4-byte aligned.  A misaligned pointer, a host pointer, a
   buffer or a stream of another device returns PBF_ERR_INVALID, and a CUDA
   error left pending by earlier work returns PBF_ERR_CUDA (and stays
   pending), all before any work is enqueued.
   The outputs equal the first particleCount keys / permutation entries and
   the cell table of pbf_sort_state.  Work is enqueued on `stream` (a
   cudaStream_t; NULL is the legacy default stream) and is complete when the
   stream reaches it.

   The call allocates nothing: its working memory is one fixed array of
   PBF_NOALLOC_SCRATCH_BYTES per device, shared by every call on that device.
   The first call on a device looks up that array's address (a runtime call,
   no allocation); make that first call before any stream capture.  Calls
   whose work overlaps on the GPU (e.g. on two streams at once) race on the
   shared array and must be ordered by the caller.  particleCount above
   PBF_NOALLOC_MAX_KEYS returns PBF_ERR_INVALID without enqueuing work. */
int pbf_sort_state_noalloc(const PbfParameters* params, const float* d_pred,
                           uint32_t* d_keys, uint32_t* d_perm, uint32_t* d_cells, void* stream);

/* ------------------------------------------------------------- batches -- */

/* A context that advances `nscenes` independent scenes together, every stage
   one launch over all of them (no counterpart in the reference, which runs one
   scene).  scenes[s] describes scene s; the scenes must agree on every field
   except particleCount, the box (xMin..zMax), the gravity (garvity or the
   gravity vector) and viscosityFactor.  The particle arrays of the other calls
   are the scenes' arrays concatenated in order (pbf_scene_offsets gives the
   boundaries); each scene's particles stay inside its range across steps and
   its results are bit-identical to running it alone with the same
   gridBufSize.  InitBuffers with init_pos == NULL places each scene's
   reference lattice. */
int pbf_create_batch(const PbfParameters* scenes, int nscenes, int device, pbf_ctx** out);

/* offsets[s] .. offsets[s+1] is scene s's index range (nscenes + 1 words; a
   single-scene context reports 0 and particleCount). */
int pbf_scene_offsets(pbf_ctx* ctx, uint32_t* offsets);

/* ------------------------------------------------------------ rollouts -- */

/* Original index (0 .. N-1 at InitBuffers) of each particle record in the
   current order; the sort permutes the records every substep. */
int pbf_read_ids(pbf_ctx* ctx, uint32_t* ids);

/* Differentiable rollout (no counterpart in the reference).  Run `substeps`
   substeps from the current state, keeping the state every
   `checkpoint_every` substeps (and at the end) so that the reverse pass can
   recompute each segment instead of storing every substep. */
int pbf_rollout_forward(pbf_ctx* ctx, int substeps, int checkpoint_every);

/* Reverse pass of the last pbf_rollout_forward, over a fixed neighbour
   structure (each substep's sort permutation, friend lists and box-clamp
   decisions are constants of the derivative; recomputing a segment from its
   checkpoint reproduces them exactly).  dL_dx: adjoint of the final positions
   (4 floats per particle, indexed by original particle index, w ignored).
   Outputs (any may be NULL): dL_dv0 (4 per particle, by original index) for
   the initial velocities, dL_dvisc for viscosityFactor, dL_dg (3) for the
   gravity vector.  Memory: one segment of intermediate values.  The context's
   state is left at the end of the rollout.  Returns PBF_ERR_STATE when the
   buffers, cells, kernels, parameters, pause flag, force planes, force mask or
   wave wall were set after the forward pass (its substeps could no longer be
   recomputed); run pbf_rollout_forward again. */
int pbf_rollout_backward(pbf_ctx* ctx, const float* dL_dx, float* dL_dv0, float* dL_dvisc, float* dL_dg);

/* ------------------------------------------------------ headless render -- */

/* PbfCamera (include/pbf_params.h) is the renderer's camera. */

/* Fill *cam like the reference: lookAt(eye, at, up), perspective(fovyDeg,
   width/height, 0.1, 1000), widthOfNearPlane = width / (2 tan(fovy/2)),
   invFocalLen = (tan(fovy/2) aspect, tan(fovy/2)). */
int pbf_render_camera(const float eye[3], const float at[3], const float up[3], float fovyDeg, int width, int height,
                      float pointSize, PbfCamera* cam);

/* Render the current particle positions into width x height RGBA float
   images on the device (no graphics API; the shaders' arithmetic as CUDA
   kernels, pixel (0,0) at the bottom left as in OpenGL windows):
     mode 0 (smooth, UICmd_RenderMode 0): particles.vs + particles_color.fs
       splat the particles as sphere impostors with a LEQUAL depth test
       (colour = fragment depth, particle index), then vis_scan.cms marks the
       visible particles, grid_build.cms hashes them into a 2048 x 2048 grid,
       fluid_depth_smoothing.fs moves every pixel onto the density shell
       (colour = depth, gradient direction) and fluid_final_render.fs shades
       it;
     mode 1 / 2: the splat coloured by speed / by particle index
       (particles_color.fs renderMethod 1 / 2), copied to the output.
   Orders the shaders leave to the hardware are fixed: among fragments of
   equal depth the last drawn (highest index) wins, and a grid cell's chain
   lists its visible particles in decreasing index order.  Reproducible bit
   for bit against the oracle's restatement. */
int pbf_render_frame(pbf_ctx* ctx, const PbfCamera* cam, int mode);

/* Copy an image of the last pbf_render_frame to host memory (width x height
   float4, row 0 at the bottom): which 0 = output, 1 = splat colour,
   2 = smoothed depth (mode 0 only). */
int pbf_render_read(pbf_ctx* ctx, int which, float* rgba);

/* ------------------------------------------------------------ autotuner -- */

/* The launch shape, PBF_LAUNCH_SHAPE_FIELDS ints: threads per block of the
   five neighbour kernels in the order friends, density (scaling), delta,
   viscosity, vorticity (multiples of 32 in [32, 512]), then the friends
   algorithm (0: one thread scans the 27 cells per particle; 1: a warp scans
   the cells of each run of same-cell particles together; 2: a block stages
   the 6x6x6-cell halo of a 4x4x4-cell brick in shared memory and its threads
   scan from there, for power-of-two GridBufferSize >= 64, else 0), then the balance
   flag (1: the four solver passes hand each block's particles to its threads
   in decreasing order of friend count, so warps walk lists of similar
   length), then the persistent flag (1: the four solver passes launch at
   most as many blocks as the device keeps resident,
   and each block walks the tiles of particles grid-stride; blocks never wait
   on one another).  Results do not depend on any of them. */
#define PBF_LAUNCH_SHAPE_FIELDS 8
int pbf_get_launch_shape(pbf_ctx* ctx, int* blocks);
int pbf_set_launch_shape(pbf_ctx* ctx, const int* blocks);

/* Time `trial_substeps` substeps from the current state for each candidate
   block size (64, 128, 256, 512), the three friends algorithms and both balance
   settings, keep the fastest per kernel (the balance setting by the sum of
   the solver passes), then time that shape with and without persistent
   grids and keep the faster, restore the state (positions, velocities, particle ids
   and the per-stage trackers as they were), and report the choice through
   blocks_out (PBF_LAUNCH_SHAPE_FIELDS ints, may be NULL). */
int pbf_autotune(pbf_ctx* ctx, int trial_substeps, int* blocks_out);

/* ------------------------------------------------------------- scenarios -- */

/* The reference's initial lattice (Simulation::CreateParticles,
   src/Simulation.cpp:71-101) for params->particleCount particles. */
int pbf_reference_lattice(const PbfParameters* params, float* pos);

/* A jittered block lattice: particle i = ix + nx*(iy + ny*iz) sits at
   origin + (ix, iy, iz) * spacing + u, u uniform in [-jitter, jitter) per
   component from std::mt19937_64(seed); w = 0.  Computed in double, rounded
   once to float. */
int pbf_scene_block(int nx, int ny, int nz, float spacing,
                    float ox, float oy, float oz,
                    float jitter, uint64_t seed, float* pos);

/* Double dam break for the particle-count sweep: n particles in two 1:2:1
   blocks on the floor of opposite corners of a 2:1:1 box whose volume is
   n * spacing^3 / fill.  pos receives n float4 records; box receives xMin,
   xMax, yMin, yMax, zMin, zMax. */
int pbf_scene_double_dam_break(int n, float spacing, float fill, float jitter, uint64_t seed,
                               float* pos, float* box);

#ifdef __cplusplus
}
#endif

#endif /* PBF_CAPI_H */
