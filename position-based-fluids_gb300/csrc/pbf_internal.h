// pbf_internal.h — declarations shared by the library's translation units.
#pragma once

#include <cstdint>
#include <string>

#include "pbf_capi.h"

#include <cuda_runtime.h>

namespace pbf {

// Constants every solver kernel reads, formed once on the host from the
// parameters (src/Simulation.cpp:169-183 bakes the same values into the
// OpenCL build as -D literals).
// One force plane with its per-plane constants formed on the host
// (compute_delta.cl:3-9): a, b, c, invdet = 1.0 / (a c - b b) taken in
// double and rounded once (the literal 1.0 is a double), and
// planeNorm = normalize(cross(E0, E1)) as cross / sqrt(dot).
struct QuadDev {
    float B[3], E0[3], E1[3], n[3];
    float a, b, c, invdet;
    int maskYOffset, maskHeight;
};

// Bits of the device error word (pbf_synchronize reports it).
constexpr int kErrCellTable = 1;    // a cell range that runs backwards
constexpr int kErrFriendIndex = 2;  // a friend-list entry >= N (bounds-checked builds)
constexpr int kErrSortIndex = 4;    // a permutation entry >= N (bounds-checked builds)
constexpr int kErrCellKey = 8;      // a key beyond the cell table (bounds-checked builds)

struct DevConsts {
    float dt, h, h2, minR, hMinusMinR;
    float poly6, gradSpiky, negGradSpiky, poly6q;
    float rho0, rho0sq, eps, K, visc, vort;
    float gx, gy, gz;
    float lo[3], hi[3];
    int clamp, guard;
    int relaxed;                 // relaxedMath: the neighbour passes' relaxed variants
    int complete;                // completeNeighbours: all circles in every pass, self in the density
    int nquads, maskW, maskH;    // force planes (pbf_set_force_quads) and their mask
    const QuadDev* quads;
    const uint32_t* mask;        // NULL: the empty mask
    const float* wave;           // device scalar: the moving wall's offset from xMin (NULL: none)
    int* err;                    // the context's error word (bounds-checked builds record bad indices there)
    float dpScale, invPoly6q;    // -gradSpiky / rho0 and 1 / poly6q (relaxed variants only)
    // Exact passes: quotients by |r| and by poly6q through a reciprocal and
    // one remainder correction (quotient_rn, sqrt_recip_rn), where the
    // parameters keep every numerator and quotient in the range that makes it
    // equal to IEEE division (make_consts decides), for the particles whose
    // friends all sit at regular positions (quotients_tainted).
    int quotients;               // divisions by |r| in the four neighbour passes
    int quotientPoly6q;          // the s_corr division by poly6q in the position pass
    float recipPoly6q;           // RN(1 / poly6q)
    uint32_t* epoch;             // device word: the substep's number, counted by the predict kernel
    uint32_t* taint;             // per particle: the last substep that tainted it (quotients_tainted)
    int4* cellXYZ;               // per particle: the cell its friends were taken around, and the scene's first key
                                 // (NULL in relaxed mode: nothing is tainted)
    const uint32_t* cellStart;   // per cell key: its first particle, when the substep's keys confirm it
    const uint32_t* keys;        // the substep's sorted cell keys (set per substep)
    int circles, perCircle;
    uint32_t grid;
    int n;
    // circT[k-1]: the smallest r^2 whose friend circle is >= k (k = 1..C-1),
    // +inf where no r^2 < h^2 reaches circle k.  The circle of r^2 is the
    // number of thresholds it reaches.
    float circT[PBF_MAX_CIRCLES];
};

// Records `msg` as the last error of `ctx` (or of the calling thread when ctx
// is NULL) and returns `code`.
int fail(pbf_ctx* ctx, int code, const std::string& msg);

DevConsts make_consts(const PbfParameters& p, int n);

// The values that may differ between the scenes of a batch.  A batch keeps
// all scenes in one particle array; scene s owns a fixed index range (its
// keys are offset by s * gridBufSize, so the stable sort never moves a
// particle out of it) and sceneOf[i] names the scene of particle i.
struct SceneParams {
    float gx, gy, gz;
    float lo[3], hi[3];
    float visc;
    uint32_t keyBase;  // s * gridBufSize
    uint32_t pad;
};
// scenes == nullptr: a single scene whose values are those of DevConsts.
struct Batch {
    const SceneParams* scenes;
    const uint16_t* sceneOf;
    int nscenes = 0;
};
SceneParams make_scene_params(const PbfParameters& p, uint32_t keyBase);

// Threads per block of the kernels whose block size the autotuner chooses.
struct LaunchShape {
    int friends = 256, scaling = 256, delta = 256, viscosity = 256, vorticity = 256;
    int friendsAlgorithm = 0;  // 0: one thread scans per particle; 1: warp-cooperative runs;
                               // 2: 4x4x4-cell bricks streamed through shared memory
    int balance = 0;           // solver passes: threads take the block's particles by friend count
    int persistent = 0;        // the four solver passes: a grid of the resident blocks takes
                               // the particle tiles from a counter (no waits between blocks)
};
constexpr int kMaxBlock = 512;

// ---- kernels (pbf_kernels.cu) ----
void launch_predict_keys(const DevConsts& c, Batch b, const float4* pos, float4* vel, float4* pred,
                         uint32_t* keys, uint32_t* perm, int paused, cudaStream_t s);
void launch_compute_keys(const DevConsts& c, Batch b, const float4* pred, uint32_t* keys, uint32_t* perm,
                         cudaStream_t s);
// err (may be NULL): the error word that bounds-checked builds report bad
// permutation entries or keys to; keyLimit: the number of cell-table entries.
void launch_gather_sorted(int n, const uint32_t* perm, const float4* pos, const float4* pred, const uint32_t* ids,
                          float4* posOut, float4* predOut, uint32_t* idsOut, int* err, cudaStream_t s);
// cellStart (may be NULL): also each occupied cell's first particle.
void launch_update_cells(int n, const uint32_t* keys, uint32_t* cells, uint32_t keyLimit, int* err, cudaStream_t s,
                         uint32_t* cellStart = nullptr);
void launch_reset_cells(int n, const uint32_t* keys, uint32_t* cells, uint32_t keyLimit, int* err, cudaStream_t s);
// tileCounter (two device words, zero between launches; NULL for one block
// per tile of particles): the solver passes' persistent grid, whose
// blocks take the tiles from it (LaunchShape::persistent).
// algorithm: LaunchShape::friendsAlgorithm.  Every build writes the circle
// rows into `list`; none writes the flat rows (the first density pass
// records them), so the return value, whether `flat` was written, is false.
bool launch_build_friends(const DevConsts& c, Batch b, const float4* pred, const uint32_t* cells, uint32_t* list,
                          uint32_t* flat, uint2* meta, int* errorWord, int block, int algorithm, cudaStream_t s);
// The flat rows from the circle rows, when no density pass records them.
void launch_flatten_friends(const DevConsts& c, const uint32_t* list, const uint2* meta, uint32_t* flat, cudaStream_t s);
// flatIn / flatOut (may be NULL): the friends recorded in order as flat rows
// flat[t * N + i] by the first density pass of a substep (flatOut) and read
// from there by the passes after it (flatIn) instead of the circle rows.
void launch_compute_scaling(const DevConsts& c, const float4* pred, float4* predPacked, float* density,
                            const uint32_t* list, const uint2* meta, const uint32_t* flatIn, uint32_t* flatOut,
                            int block, int balance, int* tileCounter, cudaStream_t s);
// posPrev: the sorted positions, read only by the force planes.
void launch_compute_delta(const DevConsts& c, Batch b, const float4* predPacked, const float4* posPrev,
                          float4* predOut, const float* density, const uint32_t* list, const uint2* meta,
                          int lastIteration, uint8_t* clampMask, const uint32_t* flatIn, int block, int balance,
                          int* tileCounter, cudaStream_t s);
void launch_update_velocities(const DevConsts& c, const float4* pred, const float4* posIn, float4* posOut,
                              float4* vel, const uint32_t* idsIn, uint32_t* idsOut, cudaStream_t s);
void launch_apply_viscosity(const DevConsts& c, Batch b, const float4* pred, const float4* velIn, float4* velOut,
                            float4* omega, const uint32_t* list, const uint2* meta, const uint32_t* flatIn, int block,
                            int balance, int* tileCounter, cudaStream_t s);
// tileCount > 0: only the particle tiles [firstTile, firstTile + tileCount)
// of `block` particles, one block per tile (a frame's read-back splits the
// last vorticity pass so that the first part's velocities copy out while the
// rest runs).
void launch_apply_vorticity(const DevConsts& c, const float4* pred, const float4* omega, const float4* velIn,
                            float4* velOut, const uint32_t* list, const uint2* meta, const uint32_t* flatIn, int block,
                            int balance, int* tileCounter, cudaStream_t s, int firstTile = 0, int tileCount = 0);

// ---- radix sort (pbf_sort.cu) ----
struct SortPlan {
    int n = 0;
    int passes = 0;       // 8-bit digits needed for keys < gridBufSize
    int rounds = 16;      // keys per thread and tile: 256 x rounds per tile (4 at <= 2^18 keys)
    int tiles = 0;        // ceil(n / (256 * rounds))
    size_t histWords = 0; // 256 * tiles
};
SortPlan make_sort_plan(int n, uint32_t gridBufSize);
// Sorts (keys[0], perm[0]) by key, stably, ping-ponging through keys[1] /
// perm[1]; returns the index (0 or 1) of the buffers holding the result.
// When posIn/predIn are given, the last pass also writes posOut/predOut
// gathered through the permutation (the reference's sortParticles).
int launch_radix_sort(const SortPlan& plan, uint32_t* keys[2], uint32_t* perm[2], uint32_t* hist,
                      const float4* posIn, const float4* predIn, float4* posOut, float4* predOut,
                      cudaStream_t s);
// Kernels launched by one launch_radix_sort call.
int radix_sort_launches(const SortPlan& plan);

// ---- adjoint (pbf_adjoint.cu) ----
// What one substep of a rollout leaves for its reverse pass.
struct AdjointTape {
    int iterations = 0;
    uint32_t* perm = nullptr;      // sorted index k came from perm[k]
    uint32_t* list = nullptr;      // the substep's kept friends as flat rows (friend t of i at t * N + i)
    uint2* meta = nullptr;
    float4* q[64] = {};            // (p^t, lambda^t), t < iterations
    uint8_t* mask = nullptr;       // iterations x N box-clamp decisions (NULL: no clamp)
    float4* pI = nullptr;          // final predictions, w = density
    float4* v2 = nullptr;          // velocities before XSPH
    float4* omega = nullptr;
};
// Adjoint state; xb / vb hold the adjoints of the substep's output on entry
// and of its input on return (the pointers are swapped with xo / vo).
struct AdjointBuffers {
    float4 *xb, *vb, *xo, *vo, *pb, *pbt, *omb, *v2b, *xsb;
    float* lb;
    float* scalars;  // [0] dL/d viscosityFactor, [1..3] dL/d gravity
};
void adjoint_substep(const DevConsts& c, const AdjointTape& tp, AdjointBuffers& ab, cudaStream_t s);
int adjoint_launches(int iterations);
void scatter_by_id(int n, const uint32_t* ids, const float4* byId, float4* out, cudaStream_t s);
void gather_to_id(int n, const uint32_t* ids, const float4* in, float4* byId, cudaStream_t s);

// ---- headless render (pbf_render.cu) ----
struct RenderBuffers {
    int width = 0, height = 0, n = 0;
    unsigned long long* dkey = nullptr;  // per pixel: (depth bits, ~particle index) of the nearest fragment
    float4* splat = nullptr;             // particles_color.fs output
    float4* smooth = nullptr;            // fluid_depth_smoothing.fs output
    float4* out = nullptr;               // the frame
    uint8_t* vis = nullptr;              // per particle: seen in the splat
    uint32_t* keys[2] = {nullptr, nullptr};
    uint32_t* perm[2] = {nullptr, nullptr};
    uint32_t* hist = nullptr;
    uint32_t* cells = nullptr;           // 2 x 2048^2: first / last sorted index per bucket
    SortPlan plan{};
};
void render_frame(const PbfCamera& cam, int mode, int n, float h, const float4* pos, RenderBuffers& rb, cudaStream_t s);
int render_launches(int mode, const SortPlan& plan);
size_t render_grid_words();

}  // namespace pbf
