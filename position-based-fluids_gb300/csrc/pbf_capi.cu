// pbf_capi.cu — the C-ABI (include/pbf_capi.h): context lifetime, device
// buffers, the substep orchestration of Simulation::Step
// (src/Simulation.cpp:554-621) and the parity hooks.
//
// Buffer roles within one substep (N particles; index in brackets):
//   predict      pos[P] vel[V]            -> pred[0], keys[0], perm[0]
//   sort         keys/perm ping-pong      -> keys[k], perm[k]
//   gather       pos[P] pred[0]           -> pos[P^1], pred[1]   (sortParticles)
//   cells        keys[k]                  -> cells
//   friends      pred[1] cells            -> list, counts; cells reset
//   iterations   pred[1] -> pred[0] (lambda packed in w) -> pred[1]
//   velocities   pred[1] pos[P^1]         -> pos[P], vel[V]
//   viscosity    pred[1] vel[V]           -> vel[V^1], omega
//   vorticity    vel[V^1] omega           -> vel[V]
// so an unpaused substep starts and ends with the same roles and one
// captured CUDA graph replays every substep.

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "pbf_capi.h"
#include "pbf_internal.h"

struct pbf_ctx {
    PbfParameters params{};
    int device = 0;
    int n = 0;
    cudaStream_t stream = nullptr;
    bool buffersReady = false, cellsReady = false, kernelsReady = false;
    int paused = 0;
    std::string lastError;

    float4* pos[2] = {nullptr, nullptr};
    float4* pred[2] = {nullptr, nullptr};
    float4* vel[2] = {nullptr, nullptr};
    float4* omega = nullptr;
    float* density = nullptr;
    uint32_t* keys[2] = {nullptr, nullptr};
    uint32_t* perm[2] = {nullptr, nullptr};
    uint32_t* hist = nullptr;
    uint32_t* cells = nullptr;
    uint32_t* list = nullptr;
    uint32_t* flat = nullptr;    // the friends of the substep in order, one flat row per position (see enqueue_substep)
    uint2* meta = nullptr;       // per-particle friend counts per circle + kept circles
    uint32_t* taint = nullptr;          // per particle: the substep that tainted it (pbf::DevConsts::taint)
    int4* cellXYZ = nullptr;            // per particle: its cell at the friends build and the scene's first key
    uint32_t* cellStart = nullptr;      // per cell key: its first particle (pbf::DevConsts::cellStart)
    int* errWord = nullptr;
    int* tileCounters = nullptr;  // 2 words per neighbour kernel: its persistent grid's tile counter
    size_t histWords = 0;
    uint32_t cellsWords = 0;  // gridBufSize the cell table was allocated for
    int listSlots = 0;
    int cellsN = 0;           // particle count the friend rows were allocated for
    // bumped by every call that changes what a substep computes (buffers,
    // cells, parameters, pause, force planes, wave wall)
    uint64_t epoch = 0;

    // batch: scene s owns particles [sceneOffsets[s], sceneOffsets[s+1])
    std::vector<PbfParameters> sceneParams;  // empty for a single scene
    std::vector<uint32_t> sceneOffsets;
    pbf::SceneParams* scenes = nullptr;      // device table, batches only
    float* waveDev = nullptr;                // moving wall offset (pbf_set_wave_position)
    pbf::RenderBuffers render;               // pbf_render_frame
    int renderMode = -1;
    pbf::QuadDev* quadsDev = nullptr;        // force planes (pbf_set_force_quads)
    int nquads = 0;
    uint32_t* maskDev = nullptr;             // force mask (pbf_load_force_masks)
    int maskW = 0, maskH = 0;
    uint32_t* ids = nullptr;                 // original index of each particle record
    uint32_t* idsTmp = nullptr;
    uint16_t* sceneOf = nullptr;             // device, batches only
    pbf::LaunchShape shape;

    pbf::SortPlan plan;
    pbf::DevConsts consts{};
    int curPos = 0, curVel = 0, curPred = 1, keysIdx = 0;
    bool stepped = false;

    // pbf_step_read_async: the last substep copies its final positions out on
    // copyStream while XSPH and vorticity run, and its velocities in two
    // parts: the first half's on copyStream while the vorticity pass runs
    // over the second half, the rest after it
    cudaStream_t copyStream = nullptr;
    cudaEvent_t evPosReady = nullptr, evCopyDone = nullptr, evVelHead = nullptr;
    float* readPos = nullptr;
    float* readVel = nullptr;

    // A captured substep: the plain one, and the one with pbf_step_read_async's
    // copies (for one pair of page-locked destinations)
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        int pos = -1;          // the position buffer it starts from
        size_t kernels = 0;    // its kernel nodes, counted as launches
        float* host[2] = {nullptr, nullptr};
    };
    bool useGraph = true;
    StepGraph graph, readGraph;
    uint64_t launches = 0;

    bool stageTiming = false;
    bool nvtx = false;                       // NVTX ranges around the stages of eager substeps
    std::vector<std::string> stageNames;
    std::vector<float> stageMs;
    // per-launch trackers in the reference's naming (OCLPerfMon), EMA 0.5
    std::vector<PbfPerfTracker> trackers;
    cudaEvent_t timingAnchor = nullptr;  // time zero of the trackers' timestamps

    // rollout: state at the start of every segment of `rollEvery` substeps,
    // and at the end (pbf_rollout_forward / pbf_rollout_backward)
    struct Checkpoint {
        float4* pos = nullptr;
        float4* vel = nullptr;
        uint32_t* ids = nullptr;
        int curPos = 0, curVel = 0, curPred = 1, keysIdx = 0;
    };
    std::vector<Checkpoint> ckpt;
    Checkpoint ckptEnd;
    int rollSubsteps = 0, rollEvery = 0;
    uint64_t rollEpoch = 0;                  // epoch the forward pass ran under
    // reverse pass: one segment of tape plus the adjoint buffers, kept
    // between calls while (rollEvery, simIterations, boxClamp) stay the same
    std::vector<void*> tapeMem;
    std::vector<pbf::AdjointTape> tapes;
    pbf::AdjointBuffers adj{};
    float4* adjById = nullptr;
    int tapeEvery = 0, tapeIters = 0, tapeClamp = -1, tapeN = 0, tapeSlots = 0;
    // one CUDA graph per segment shape of the reverse pass: the segment's
    // recompute and its adjoint substeps, for a segment length and the adjoint
    // buffers' roles at its start (and their roles at its end)
    struct SegmentGraph {
        int len = 0;
        int pos = 0, vel = 0;  // the position / velocity buffer roles it was captured with
        pbf::AdjointBuffers pre{}, post{};
        cudaGraphExec_t exec = nullptr;
        size_t nodes = 0;
    };
    std::vector<SegmentGraph> segGraphs;
};

namespace pbf {

thread_local std::string tls_error = "no error";

int fail(pbf_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->lastError = msg;
    tls_error = msg;
    return code;
}

// The -D constants of src/Simulation.cpp:169-183 and the two powers of
// compute_delta.cl:81-82, formed on the host.  POLY6_FACTOR and
// GRAD_SPIKY_FACTOR go through the reference's text round trip: the double
// value printed with 6 significant digits and read back as a float literal.
static float six_digit_literal(double v) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.6g", v);
    return std::strtof(buf, nullptr);
}

// Friend circle of a neighbour at squared distance r2 (< h^2), evaluated as
// build_friends_list.cl:75-76 does, one IEEE operation at a time.
static int circle_of(float r2, float minR, float hMinusMinR, int C) {
    const float adj = std::fmax(0.0f, (std::sqrt(r2) - minR) / hMinusMinR);
    const int circ = (int)(adj * adj * adj * (float)C);
    return circ < C - 1 ? circ : C - 1;
}

// Every operation in circle_of rounds monotonically, so the circle is a
// non-decreasing step function of r2 (r2 >= 0).  For each k, bisect over the
// bit patterns of the non-negative floats below h^2 for the first r2 whose
// circle reaches k.
static void circle_thresholds(DevConsts& c) {
    for (int k = 0; k < PBF_MAX_CIRCLES; ++k) c.circT[k] = INFINITY;
    uint32_t h2bits;
    std::memcpy(&h2bits, &c.h2, 4);
    for (int k = 1; k < c.circles; ++k) {
        auto circ = [&](uint32_t bits) {
            float r2;
            std::memcpy(&r2, &bits, 4);
            return circle_of(r2, c.minR, c.hMinusMinR, c.circles);
        };
        if (h2bits == 0 || circ(h2bits - 1) < k) continue;  // no r2 < h^2 reaches k
        if (circ(0) >= k) { c.circT[k - 1] = 0.0f; continue; }
        uint32_t lo = 0, hi = h2bits - 1;  // circ(lo) < k <= circ(hi)
        while (hi - lo > 1) {
            const uint32_t mid = lo + (hi - lo) / 2;
            if (circ(mid) >= k) hi = mid; else lo = mid;
        }
        float t;
        std::memcpy(&t, &hi, 4);
        c.circT[k - 1] = t;
    }
}

DevConsts make_consts(const PbfParameters& p, int n) {
    DevConsts c{};
    const double kPi = 3.14159265358979323846;
    c.dt = p.timeStep;
    c.h = p.h;
    c.h2 = p.h_2;
    c.minR = 0.3f * p.h;
    c.hMinusMinR = p.h - c.minR;
    c.poly6 = six_digit_literal(315.0f / (64.0f * kPi * std::pow((double)p.h, 9.0)));
    c.gradSpiky = six_digit_literal(45.0f / (kPi * std::pow((double)p.h, 6.0)));
    c.negGradSpiky = -c.gradSpiky;
    const float qh = p.surfaceTenstionDist * p.h;
    const float q2 = (float)((double)qh * (double)qh);
    const float d = p.h_2 - q2;
    c.poly6q = (float)((double)d * (double)d * (double)d);
    c.rho0 = p.restDensity;
    c.rho0sq = p.restDensity * p.restDensity;
    c.eps = p.epsilon;
    c.K = p.surfaceTenstionK;
    c.visc = p.viscosityFactor;
    c.vort = p.vorticityFactor;
    if (p.gravityVectorEnable) { c.gx = p.gravityX; c.gy = p.gravityY; c.gz = p.gravityZ; }
    else { c.gx = 0.0f; c.gy = -p.garvity; c.gz = 0.0f; }
    c.lo[0] = p.xMin; c.lo[1] = p.yMin; c.lo[2] = p.zMin;
    c.hi[0] = p.xMax; c.hi[1] = p.yMax; c.hi[2] = p.zMax;
    c.clamp = p.boxClamp ? 1 : 0;
    c.guard = p.zeroDistanceGuard ? 1 : 0;
    c.relaxed = p.relaxedMath ? 1 : 0;
    c.complete = p.completeNeighbours ? 1 : 0;
    c.dpScale = c.negGradSpiky / c.rho0;
    c.invPoly6q = 1.0f / c.poly6q;
    // Exact-mode quotients by reciprocal (quotient_rn in pbf_device.cuh).  For
    // particles whose friends all sit at coordinates that are 0 or at least
    // 2^-27 in magnitude (the others divide the IEEE way), a coordinate
    // difference is 0 or at least 2^-50, so r^2 is 0 or at least 2^-100 and
    // |r| (when r != 0) is normal.  A nonzero remaining distance h - |r| is at
    // least h 2^-25 (one half ulp of h), so the density pass's numerator
    // gradSpiky (h - |r|)^2 r_x is 0 or at least gradSpiky (h 2^-25)^2 2^-50,
    // which must not fall below 2^-100; the quotients themselves are at most
    // gradSpiky h^2 (|r_x| <= |r|).
    const double hrMin = (double)p.h * std::ldexp(1.0, -25);
    c.quotients = (p.h >= std::ldexp(1.0f, -10) && p.h <= 1024.0f &&
                   (double)c.gradSpiky * hrMin * hrMin >= std::ldexp(1.0, -50) &&
                   (double)c.gradSpiky * (double)p.h * (double)p.h < 1e30) ? 1 : 0;
    // s_corr: for r^2 < h^2 the numerator (h^2 - r^2)^3 is at least
    // (h^2 2^-25)^3 >= 2^-99 when h^2 >= 2^-8, and with poly6q <= h^6 <= 1 the
    // quotient is at least as large; at most h^6 / poly6q.
    c.recipPoly6q = 1.0f / c.poly6q;
    c.quotientPoly6q = (std::isnormal(c.poly6q) && std::isnormal(c.recipPoly6q) && c.h2 >= std::ldexp(1.0f, -8) &&
                        c.h2 <= 1.0f && (double)c.h2 * c.h2 * c.h2 / c.poly6q < 1e30) ? 1 : 0;
    c.circles = (int)p.friendsCircles;
    c.perCircle = (int)p.particlesPerCircle;
    c.grid = p.gridBufSize;
    c.n = n;
    if (c.circles >= 1 && c.circles <= PBF_MAX_CIRCLES && c.h2 > 0.0f) circle_thresholds(c);
    return c;
}

SceneParams make_scene_params(const PbfParameters& p, uint32_t keyBase) {
    const DevConsts c = make_consts(p, 0);
    SceneParams s{};
    s.gx = c.gx; s.gy = c.gy; s.gz = c.gz;
    for (int k = 0; k < 3; ++k) { s.lo[k] = c.lo[k]; s.hi[k] = c.hi[k]; }
    s.visc = c.visc;
    s.keyBase = keyBase;
    return s;
}

}  // namespace pbf

namespace {

using pbf::fail;

#define PBF_CUDA(ctx, call)                                                                      \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return fail((ctx), PBF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T> int dev_alloc(pbf_ctx* ctx, T** p, size_t count) {
    if (*p) { cudaFree(*p); *p = nullptr; }
    if (count == 0) count = 1;
    PBF_CUDA(ctx, cudaMalloc((void**)p, sizeof(T) * count));
    return PBF_OK;
}

template <typename T> void dev_free(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// Per-plane constants of BouncePointQuad (compute_delta.cl:3-9), in the
// reference's operation order.
pbf::QuadDev quad_constants(const PbfForceQuad& in) {
    pbf::QuadDev q{};
    for (int k = 0; k < 3; ++k) { q.B[k] = in.B[k]; q.E0[k] = in.E0[k]; q.E1[k] = in.E1[k]; }
    auto dot = [](const float* u, const float* v) { return (u[0] * v[0] + u[1] * v[1]) + u[2] * v[2]; };
    q.a = dot(q.E0, q.E0);
    q.b = dot(q.E0, q.E1);
    q.c = dot(q.E1, q.E1);
    q.invdet = (float)(1.0 / (double)(q.a * q.c - q.b * q.b));
    const float cr[3] = {q.E0[1] * q.E1[2] - q.E0[2] * q.E1[1], q.E0[2] * q.E1[0] - q.E0[0] * q.E1[2],
                         q.E0[0] * q.E1[1] - q.E0[1] * q.E1[0]};
    const float len = std::sqrt(dot(cr, cr));
    for (int k = 0; k < 3; ++k) q.n[k] = cr[k] / len;
    q.maskYOffset = in.maskYOffset;
    q.maskHeight = in.maskHeight;
    return q;
}

void drop_graph(pbf_ctx* ctx);

void free_render(pbf_ctx* ctx) {
    pbf::RenderBuffers& r = ctx->render;
    dev_free(r.dkey); dev_free(r.splat); dev_free(r.smooth); dev_free(r.out); dev_free(r.vis);
    for (int k = 0; k < 2; ++k) { dev_free(r.keys[k]); dev_free(r.perm[k]); }
    dev_free(r.hist); dev_free(r.cells);
    r.width = r.height = r.n = 0;
}

// Copies the force planes and mask into the kernel constants.
void apply_planes(pbf_ctx* ctx) {
    ctx->consts.nquads = ctx->nquads;
    ctx->consts.quads = ctx->quadsDev;
    ctx->consts.mask = ctx->maskDev;
    ctx->consts.maskW = ctx->maskW;
    ctx->consts.maskH = ctx->maskH;
    ctx->consts.wave = ctx->waveDev;
    ctx->consts.err = ctx->errWord;
    ctx->consts.epoch = reinterpret_cast<uint32_t*>(ctx->errWord + 1);
    ctx->consts.taint = ctx->taint;
    // the cells of irregular positions: exact mode (relaxed passes divide no way but their own)
    ctx->consts.cellXYZ = ctx->consts.relaxed ? nullptr : ctx->cellXYZ;
    ctx->consts.cellStart = ctx->cellStart;
}

// The captured substep; the reverse pass's segment graphs are dropped with
// it by drop_graph (they bake in the same constants, shapes and buffers).
void drop_one_graph(pbf_ctx::StepGraph& g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = pbf_ctx::StepGraph{};
}

void drop_step_graph(pbf_ctx* ctx) {
    drop_one_graph(ctx->graph);
    drop_one_graph(ctx->readGraph);
}

void drop_segment_graphs(pbf_ctx* ctx) {
    for (auto& g : ctx->segGraphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    ctx->segGraphs.clear();
}

void drop_graph(pbf_ctx* ctx) {
    drop_step_graph(ctx);
    drop_segment_graphs(ctx);
}

int validate(pbf_ctx* ctx, const PbfParameters& p) {
    if (p.particleCount < 1 || p.particleCount > PBF_MAX_PARTICLES)
        return fail(ctx, PBF_ERR_INVALID, "particleCount must be in [1, 2^26]");
    if (p.friendsCircles < 1 || p.friendsCircles > PBF_MAX_CIRCLES)
        return fail(ctx, PBF_ERR_INVALID, "friendsCircles must be in [1, 8]");
    if (p.particlesPerCircle < 1 || p.particlesPerCircle > PBF_MAX_PER_CIRCLE)
        return fail(ctx, PBF_ERR_INVALID, "particlesPerCircle must be in [1, 64]");
    if (p.gridBufSize < 1 || p.gridBufSize > (1u << 30))
        return fail(ctx, PBF_ERR_INVALID, "gridBufSize must be in [1, 2^30]");
    if (!(p.h > 0.0f) || !(p.timeStep > 0.0f))
        return fail(ctx, PBF_ERR_INVALID, "SmoothLen and TimeStep must be positive");
    if (p.simIterations > 1000) return fail(ctx, PBF_ERR_INVALID, "simIterations must be <= 1000");
    return PBF_OK;
}

bool is_batch(const pbf_ctx* ctx) { return !ctx->sceneParams.empty(); }

pbf::Batch batch_of(const pbf_ctx* ctx) {
    return pbf::Batch{ctx->scenes, ctx->sceneOf, ctx->scenes ? (int)ctx->sceneParams.size() : 0};
}

// Scenes of a batch share every parameter but the particle count, the box,
// the gravity and the XSPH factor.
int check_batch_compatible(pbf_ctx* ctx, const std::vector<PbfParameters>& sp) {
    const PbfParameters& a = sp[0];
    for (size_t s = 1; s < sp.size(); ++s) {
        const PbfParameters& b = sp[s];
        const bool same = a.timeStep == b.timeStep && a.simIterations == b.simIterations && a.subSteps == b.subSteps &&
                          a.h == b.h && a.h_2 == b.h_2 && a.restDensity == b.restDensity && a.epsilon == b.epsilon &&
                          a.vorticityFactor == b.vorticityFactor && a.surfaceTenstionK == b.surfaceTenstionK &&
                          a.surfaceTenstionDist == b.surfaceTenstionDist && a.friendsCircles == b.friendsCircles &&
                          a.particlesPerCircle == b.particlesPerCircle && a.gridBufSize == b.gridBufSize &&
                          a.boxClamp == b.boxClamp && a.zeroDistanceGuard == b.zeroDistanceGuard &&
                          a.relaxedMath == b.relaxedMath && a.completeNeighbours == b.completeNeighbours;
        if (!same)
            return fail(ctx, PBF_ERR_INVALID,
                        "scene " + std::to_string(s) + " differs from scene 0 in a parameter scenes must share "
                        "(only particleCount, the box, gravity and viscosityFactor may differ)");
    }
    return PBF_OK;
}

// ------------------------------------------------------------- the step --
struct StageClock {
    pbf_ctx* ctx;
    struct Mark {
        int stage;      // index into stageNames (the base name)
        int tracker;    // index into trackers (the name with its iteration suffix)
        cudaEvent_t event;
    };
    std::vector<Mark> marks;
    ~StageClock() {  // events of a substep that failed before finish()
        for (auto& m : marks) cudaEventDestroy(m.event);
    }
    // `iteration` >= 0 names the tracker name_iteration, as
    // OCLPerfMon::GetTrackerEvent(name, iterationIndex) does (src/OCLPerfMon.cpp:3-31).
    int stage(const char* name, int iteration = -1) {
        if (!ctx->stageTiming) return PBF_OK;
        int idx = -1;
        for (size_t k = 0; k < ctx->stageNames.size(); ++k)
            if (ctx->stageNames[k] == name) idx = (int)k;
        if (idx < 0) { ctx->stageNames.push_back(name); ctx->stageMs.push_back(0.0f); idx = (int)ctx->stageNames.size() - 1; }
        std::string tname = name;
        if (iteration >= 0) tname += "_" + std::to_string(iteration);
        int tidx = -1;
        for (size_t k = 0; k < ctx->trackers.size(); ++k)
            if (tname == ctx->trackers[k].eventName) tidx = (int)k;
        if (tidx < 0) {
            PbfPerfTracker t{};
            std::snprintf(t.eventName, sizeof t.eventName, "%s", tname.c_str());
            ctx->trackers.push_back(t);
            tidx = (int)ctx->trackers.size() - 1;
        }
        cudaEvent_t e;
        PBF_CUDA(ctx, cudaEventCreate(&e));
        PBF_CUDA(ctx, cudaEventRecord(e, ctx->stream));
        marks.push_back({idx, tidx, e});
        return PBF_OK;
    }
    int finish() {
        if (!ctx->stageTiming || marks.empty()) return PBF_OK;
        cudaEvent_t end;
        PBF_CUDA(ctx, cudaEventCreate(&end));
        PBF_CUDA(ctx, cudaEventRecord(end, ctx->stream));
        PBF_CUDA(ctx, cudaEventSynchronize(end));
        for (size_t k = 0; k < marks.size(); ++k) {
            float ms = 0.0f, t0 = 0.0f, t1 = 0.0f;
            cudaEvent_t next = k + 1 < marks.size() ? marks[k + 1].event : end;
            cudaEventElapsedTime(&ms, marks[k].event, next);
            ctx->stageMs[marks[k].stage] += ms;
            PbfPerfTracker& t = ctx->trackers[marks[k].tracker];
            if (ctx->timingAnchor) {
                cudaEventElapsedTime(&t0, ctx->timingAnchor, marks[k].event);
                cudaEventElapsedTime(&t1, ctx->timingAnchor, next);
            }
            t.time_start = (uint64_t)((double)t0 * 1e6);
            t.time_end = (uint64_t)((double)t1 * 1e6);
            // OCLPerfMon::UpdateTimings (src/OCLPerfMon.cpp:33-49): weight 0.5
            t.total_time = (double)ms * (1.0 - 0.5) + t.last_time * 0.5;
            t.last_time = t.total_time;
        }
        for (auto& m : marks) cudaEventDestroy(m.event);
        cudaEventDestroy(end);
        marks.clear();
        return PBF_OK;
    }
};

__global__ void iota_kernel(int n, uint32_t* ids) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) ids[i] = (uint32_t)i;
}

__global__ void pack_density_kernel(int n, float4* pred, const float* density) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pred[i].w = density[i];
}


// Enqueue one Simulation::Step on the context's stream; with a tape, also
// copy out what the reverse pass needs.
int enqueue_substep(pbf_ctx* ctx, StageClock* clock, const pbf::AdjointTape* tape = nullptr) {
    const bool paused = ctx->paused != 0;
    pbf::DevConsts c = ctx->consts;
    if (paused) c.quotients = 0;  // no sort: the keys need not give the cells of the friends build
    cudaStream_t s = ctx->stream;
    const int P = ctx->curPos, V = ctx->curVel;
    uint64_t launched = 0;
    bool rangeOpen = false;
    bool velCopied = false;  // the read-back's velocities, copied in two parts around a split vorticity pass
    auto mark = [&](const char* name, int iteration = -1) {
        if (ctx->nvtx) {  // one range per stage, named as its tracker
            if (rangeOpen) nvtxRangePop();
            char label[64];
            if (iteration >= 0) std::snprintf(label, sizeof label, "%s_%d", name, iteration);
            else std::snprintf(label, sizeof label, "%s", name);
            nvtxRangePushA(label);
            rangeOpen = true;
        }
        return clock ? clock->stage(name, iteration) : PBF_OK;
    };

    mark("predictPositions");
    const pbf::Batch b = batch_of(ctx);
    const pbf::LaunchShape& ls = ctx->shape;
    // persistent grids: each neighbour kernel's pair of tile-counter words
    auto tiles = [&](int kernel) { return ls.persistent ? ctx->tileCounters + 2 * kernel : nullptr; };
    pbf::launch_predict_keys(c, b, ctx->pos[P], ctx->vel[V], ctx->pred[0], ctx->keys[0], ctx->perm[0], paused, s);
    ++launched;
    int sortedPos = P, sortedPred = 0;
    if (!paused) {
        mark("radixsort");
        ctx->keysIdx = pbf::launch_radix_sort(ctx->plan, ctx->keys, ctx->perm, ctx->hist, nullptr, nullptr, nullptr,
                                              nullptr, s);
        launched += pbf::radix_sort_launches(ctx->plan);
        mark("sortParticles");
        pbf::launch_gather_sorted(c.n, ctx->perm[ctx->keysIdx], ctx->pos[P], ctx->pred[0], ctx->ids, ctx->pos[P ^ 1],
                                  ctx->pred[1], ctx->idsTmp, ctx->errWord, s);
        ++launched;
        sortedPos = P ^ 1;
        sortedPred = 1;
    }
    const uint32_t* keys = ctx->keys[ctx->keysIdx];
    const size_t v4 = 16 * (size_t)c.n;
    // With a tape, the friends (flat rows), the packed (p, lambda) of every
    // iteration and omega are written straight into the tape's buffers.  The
    // circle rows (friends builds 1 and 2), or the staged build's scratch,
    // stay in ctx->list.
    uint32_t* list = ctx->list;
    uint32_t* flat = tape ? tape->list : ctx->flat;
    uint2* meta = tape ? tape->meta : ctx->meta;
    float4* omega = tape ? tape->omega : ctx->omega;
    if (tape) PBF_CUDA(ctx, cudaMemcpyAsync(tape->perm, ctx->perm[ctx->keysIdx], 4 * (size_t)c.n, cudaMemcpyDeviceToDevice, s));
    mark("updateCells");
    const uint32_t tableKeys = ctx->cellsWords * (uint32_t)(is_batch(ctx) ? ctx->sceneParams.size() : 1);
    c.keys = keys;  // the taint of irregular positions finds a cell's particles in them
    pbf::launch_update_cells(c.n, keys, ctx->cells, tableKeys, ctx->errWord, s, ctx->cellStart);
    mark("buildFriendsList");
    // the flat rows of the kept friends: written by the staged build, else
    // recorded by the first density pass (or flattened when there is none)
    bool haveFlat = pbf::launch_build_friends(c, b, ctx->pred[sortedPred], ctx->cells, list, flat, meta, ctx->errWord,
                                              ls.friends, ls.friendsAlgorithm, s);
    mark("resetPartList");
    pbf::launch_reset_cells(c.n, keys, ctx->cells, tableKeys, ctx->errWord, s);
    launched += 3;
    int a = sortedPred;
    const unsigned iters = ctx->params.simIterations;
    for (unsigned it = 0; it < iters; ++it) {
        float4* packed = tape ? tape->q[it] : ctx->pred[a ^ 1];
        mark("computeScaling", (int)it);
        // the first density pass records the flat rows from circle rows when the build wrote those
        pbf::launch_compute_scaling(c, ctx->pred[a], packed, ctx->density, list, meta, haveFlat ? flat : nullptr,
                                    haveFlat ? nullptr : flat, ls.scaling, ls.balance, tiles(1), s);
        haveFlat = true;
        mark("computeDelta", (int)it);
        pbf::launch_compute_delta(c, b, packed, ctx->pos[sortedPos], ctx->pred[a], ctx->density, list, meta,
                                  it + 1 == iters, tape && tape->mask ? tape->mask + (size_t)it * c.n : nullptr,
                                  flat, ls.delta, ls.balance, tiles(2), s);
        launched += 2;
    }
    if (!haveFlat) {
        pbf::launch_flatten_friends(c, list, meta, flat, s);
        ++launched;
    }
    if (iters == 0) {  // packData with the density buffer as it stands (src/Simulation.cpp:591)
        mark("packData");
        pack_density_kernel<<<(c.n + 255) / 256, 256, 0, s>>>(c.n, ctx->pred[a], ctx->density);
        ++launched;
    }
    if (tape) PBF_CUDA(ctx, cudaMemcpyAsync(tape->pI, ctx->pred[a], v4, cudaMemcpyDeviceToDevice, s));
    mark("updateVelocities");
    pbf::launch_update_velocities(c, ctx->pred[a], ctx->pos[sortedPos], ctx->pos[sortedPos ^ 1], ctx->vel[V],
                                  paused ? nullptr : ctx->idsTmp, ctx->ids, s);
    if (ctx->readPos) {  // the positions are final: copy them out while XSPH and vorticity run
        PBF_CUDA(ctx, cudaEventRecord(ctx->evPosReady, s));
        PBF_CUDA(ctx, cudaStreamWaitEvent(ctx->copyStream, ctx->evPosReady, 0));
        PBF_CUDA(ctx, cudaMemcpyAsync(ctx->readPos, ctx->pos[sortedPos ^ 1], v4, cudaMemcpyDeviceToHost, ctx->copyStream));
        PBF_CUDA(ctx, cudaEventRecord(ctx->evCopyDone, ctx->copyStream));
    }
    if (tape) PBF_CUDA(ctx, cudaMemcpyAsync(tape->v2, ctx->vel[V], v4, cudaMemcpyDeviceToDevice, s));
    mark("applyViscosity");
    pbf::launch_apply_viscosity(c, b, ctx->pred[a], ctx->vel[V], ctx->vel[V ^ 1], omega, list, meta, flat, ls.viscosity,
                                ls.balance, tiles(3), s);
    mark("applyVorticity");
    const int vortTiles = (c.n + ls.vorticity - 1) / ls.vorticity;
    if (ctx->readVel && ctx->readPos && vortTiles >= 2) {
        // the first half of the particles' velocities copy out while the second half runs
        const int half = vortTiles / 2;
        const size_t headBytes = 16 * (size_t)half * (size_t)ls.vorticity;
        pbf::launch_apply_vorticity(c, ctx->pred[a], omega, ctx->vel[V ^ 1], ctx->vel[V], list, meta, flat,
                                    ls.vorticity, ls.balance, nullptr, s, 0, half);
        PBF_CUDA(ctx, cudaEventRecord(ctx->evVelHead, s));
        PBF_CUDA(ctx, cudaStreamWaitEvent(ctx->copyStream, ctx->evVelHead, 0));
        PBF_CUDA(ctx, cudaMemcpyAsync(ctx->readVel, ctx->vel[V], headBytes, cudaMemcpyDeviceToHost, ctx->copyStream));
        PBF_CUDA(ctx, cudaEventRecord(ctx->evCopyDone, ctx->copyStream));
        pbf::launch_apply_vorticity(c, ctx->pred[a], omega, ctx->vel[V ^ 1], ctx->vel[V], list, meta, flat,
                                    ls.vorticity, ls.balance, nullptr, s, half, vortTiles - half);
        PBF_CUDA(ctx, cudaMemcpyAsync(reinterpret_cast<char*>(ctx->readVel) + headBytes,
                                      reinterpret_cast<const char*>(ctx->vel[V]) + headBytes, v4 - headBytes,
                                      cudaMemcpyDeviceToHost, s));
        velCopied = true;
        ++launched;
    } else {
        pbf::launch_apply_vorticity(c, ctx->pred[a], omega, ctx->vel[V ^ 1], ctx->vel[V], list, meta, flat,
                                    ls.vorticity, ls.balance, tiles(4), s);
    }
    launched += 3;
    if (rangeOpen) nvtxRangePop();
    if (ctx->readVel && !velCopied) PBF_CUDA(ctx, cudaMemcpyAsync(ctx->readVel, ctx->vel[V], v4, cudaMemcpyDeviceToHost, s));
    if (ctx->readPos) PBF_CUDA(ctx, cudaStreamWaitEvent(s, ctx->evCopyDone, 0));  // later work waits for the copy
    PBF_CUDA(ctx, cudaGetLastError());
    ctx->curPos = sortedPos ^ 1;
    ctx->curPred = a;
    ctx->launches += launched;
    return PBF_OK;
}

// Capture one substep into the plain slot, or with the copies to
// ctx->readPos / readVel into the read slot.
int capture_graph(pbf_ctx* ctx, bool read) {
    pbf_ctx::StepGraph& slot = read ? ctx->readGraph : ctx->graph;
    drop_one_graph(slot);
    if (!read) drop_segment_graphs(ctx);
    const int savedPos = ctx->curPos, savedPred = ctx->curPred, savedKeys = ctx->keysIdx;
    const uint64_t savedLaunches = ctx->launches;
    cudaGraph_t g = nullptr;
    PBF_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_substep(ctx, nullptr);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    ctx->curPos = savedPos;
    ctx->curPred = savedPred;
    ctx->keysIdx = savedKeys;
    ctx->launches = savedLaunches;
    if (rc != PBF_OK) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return fail(ctx, PBF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    size_t nodes = 0, kernels = 0;
    cudaGraphGetNodes(g, nullptr, &nodes);
    std::vector<cudaGraphNode_t> list(nodes);
    if (nodes) cudaGraphGetNodes(g, list.data(), &nodes);
    for (cudaGraphNode_t node : list) {
        cudaGraphNodeType type;
        if (cudaGraphNodeGetType(node, &type) == cudaSuccess && type == cudaGraphNodeTypeKernel) ++kernels;
    }
    e = cudaGraphInstantiate(&slot.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { slot.exec = nullptr; return fail(ctx, PBF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e)); }
    slot.pos = savedPos;
    slot.kernels = kernels;
    slot.host[0] = ctx->readPos;
    slot.host[1] = ctx->readVel;
    return PBF_OK;
}

int check_ready(pbf_ctx* ctx) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    if (!ctx->buffersReady || !ctx->cellsReady || !ctx->kernelsReady)
        return fail(ctx, PBF_ERR_STATE, "InitBuffers, InitCells and InitKernels must run before stepping");
    return PBF_OK;
}

int read_error_word(pbf_ctx* ctx) {
    int word = 0;
    PBF_CUDA(ctx, cudaMemcpyAsync(&word, ctx->errWord, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (word) {
        PBF_CUDA(ctx, cudaMemsetAsync(ctx->errWord, 0, sizeof(int), ctx->stream));
        std::string what;
        if (word & pbf::kErrCellTable) what += ", an inconsistent cell table";
        if (word & pbf::kErrFriendIndex) what += ", a friend-list entry out of range";
        if (word & pbf::kErrSortIndex) what += ", a permutation entry out of range";
        if (word & pbf::kErrCellKey) what += ", a key beyond the cell table";
        return fail(ctx, PBF_ERR_DEVICE_FLAG, "a kernel reported" + what.substr(1) + " (error word " + std::to_string(word) + ")");
    }
    return PBF_OK;
}

int save_checkpoint(pbf_ctx* ctx, pbf_ctx::Checkpoint& k) {
    const size_t n = (size_t)ctx->n;
    int rc;
    if (!k.pos && ((rc = dev_alloc(ctx, &k.pos, n)) || (rc = dev_alloc(ctx, &k.vel, n)) || (rc = dev_alloc(ctx, &k.ids, n))))
        return rc;
    k.curPos = ctx->curPos; k.curVel = ctx->curVel; k.curPred = ctx->curPred; k.keysIdx = ctx->keysIdx;
    PBF_CUDA(ctx, cudaMemcpyAsync(k.pos, ctx->pos[ctx->curPos], 16 * n, cudaMemcpyDeviceToDevice, ctx->stream));
    PBF_CUDA(ctx, cudaMemcpyAsync(k.vel, ctx->vel[ctx->curVel], 16 * n, cudaMemcpyDeviceToDevice, ctx->stream));
    PBF_CUDA(ctx, cudaMemcpyAsync(k.ids, ctx->ids, 4 * n, cudaMemcpyDeviceToDevice, ctx->stream));
    return PBF_OK;
}

int load_checkpoint(pbf_ctx* ctx, const pbf_ctx::Checkpoint& k) {
    const size_t n = (size_t)ctx->n;
    ctx->curPos = k.curPos; ctx->curVel = k.curVel; ctx->curPred = k.curPred; ctx->keysIdx = k.keysIdx;
    PBF_CUDA(ctx, cudaMemcpyAsync(ctx->pos[ctx->curPos], k.pos, 16 * n, cudaMemcpyDeviceToDevice, ctx->stream));
    PBF_CUDA(ctx, cudaMemcpyAsync(ctx->vel[ctx->curVel], k.vel, 16 * n, cudaMemcpyDeviceToDevice, ctx->stream));
    PBF_CUDA(ctx, cudaMemcpyAsync(ctx->ids, k.ids, 4 * n, cudaMemcpyDeviceToDevice, ctx->stream));
    return PBF_OK;
}

void free_tape(pbf_ctx* ctx) {
    drop_segment_graphs(ctx);
    for (void* p : ctx->tapeMem) cudaFree(p);
    ctx->tapeMem.clear();
    ctx->tapes.clear();
    ctx->adj = pbf::AdjointBuffers{};
    ctx->adjById = nullptr;
    ctx->tapeEvery = ctx->tapeIters = ctx->tapeN = ctx->tapeSlots = 0;
    ctx->tapeClamp = -1;
}

// Checkpoints and tape are sized for the particle count and the friend rows
// they were taken with; a new count or new friend limits drop them.
void free_rollout(pbf_ctx* ctx) {
    for (auto& k : ctx->ckpt) { dev_free(k.pos); dev_free(k.vel); dev_free(k.ids); }
    ctx->ckpt.clear();
    dev_free(ctx->ckptEnd.pos); dev_free(ctx->ckptEnd.vel); dev_free(ctx->ckptEnd.ids);
    ctx->rollSubsteps = ctx->rollEvery = 0;
    free_tape(ctx);
}

// One segment of tape (rollEvery substeps) and the adjoint buffers.
int ensure_tape(pbf_ctx* ctx) {
    const int n = ctx->n, iters = (int)ctx->params.simIterations, every = ctx->rollEvery;
    const int clamp = ctx->params.boxClamp != 0;
    if (ctx->tapeEvery == every && ctx->tapeIters == iters && ctx->tapeClamp == clamp && ctx->tapeN == n &&
        ctx->tapeSlots == ctx->listSlots)
        return PBF_OK;
    free_tape(ctx);
    const size_t v4 = 16 * (size_t)n;
    bool ok = true;
    auto take = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) { ok = false; return nullptr; }
        ctx->tapeMem.push_back(p);
        return p;
    };
    ctx->tapes.assign(every, pbf::AdjointTape{});
    for (pbf::AdjointTape& t : ctx->tapes) {
        t.iterations = iters;
        t.perm = (uint32_t*)take(4 * (size_t)n);
        t.list = (uint32_t*)take(4 * (size_t)ctx->listSlots * n);
        t.meta = (uint2*)take(8 * (size_t)n);
        for (int it = 0; it < iters; ++it) t.q[it] = (float4*)take(v4);
        t.mask = clamp ? (uint8_t*)take((size_t)iters * n) : nullptr;
        t.pI = (float4*)take(v4);
        t.v2 = (float4*)take(v4);
        t.omega = (float4*)take(v4);
    }
    pbf::AdjointBuffers& ab = ctx->adj;
    float4** vecs[] = {&ab.xb, &ab.vb, &ab.xo, &ab.vo, &ab.pb, &ab.pbt, &ab.omb, &ab.v2b, &ab.xsb, &ctx->adjById};
    for (float4** v : vecs) *v = (float4*)take(v4);
    ab.lb = (float*)take(4 * (size_t)n);
    ab.scalars = (float*)take(16);
    cudaGetLastError();
    if (!ok) {
        free_tape(ctx);
        return fail(ctx, PBF_ERR_CUDA, "pbf_rollout_backward: cannot allocate one segment of tape");
    }
    ctx->tapeEvery = every;
    ctx->tapeIters = iters;
    ctx->tapeClamp = clamp;
    ctx->tapeN = n;
    ctx->tapeSlots = ctx->listSlots;
    return PBF_OK;
}

bool same_buffers(const pbf::AdjointBuffers& a, const pbf::AdjointBuffers& b) {
    return a.xb == b.xb && a.vb == b.vb && a.xo == b.xo && a.vo == b.vo && a.pb == b.pb && a.pbt == b.pbt &&
           a.omb == b.omb && a.v2b == b.v2b && a.xsb == b.xsb && a.lb == b.lb && a.scalars == b.scalars;
}

// One segment of the reverse pass (its `len` substeps recomputed into the
// tape, then their adjoints in reverse) as a CUDA graph: captured once per
// segment length and starting role of the adjoint buffers, replayed for every
// segment of that shape.  Every checkpoint starts a segment with the same
// buffer roles (an unpaused substep keeps them), so the same recompute fits
// all of them.
int run_segment_graph(pbf_ctx* ctx, int len, pbf::AdjointBuffers& ab) {
    cudaStream_t s = ctx->stream;
    const int pos0 = ctx->curPos, pred0 = ctx->curPred, keys0 = ctx->keysIdx;
    pbf_ctx::SegmentGraph* hit = nullptr;
    for (auto& g : ctx->segGraphs)
        if (g.len == len && g.pos == pos0 && g.vel == ctx->curVel && same_buffers(g.pre, ab)) hit = &g;
    if (!hit) {
        pbf_ctx::SegmentGraph g;
        g.len = len;
        g.pos = pos0;
        g.vel = ctx->curVel;
        g.pre = ab;
        const uint64_t launches0 = ctx->launches;
        cudaGraph_t graph = nullptr;
        PBF_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int rc = PBF_OK;
        for (int k = 0; k < len && rc == PBF_OK; ++k) rc = enqueue_substep(ctx, nullptr, &ctx->tapes[k]);
        for (int k = len - 1; k >= 0 && rc == PBF_OK; --k) pbf::adjoint_substep(ctx->consts, ctx->tapes[k], ab, s);
        const cudaError_t e = cudaStreamEndCapture(s, &graph);
        g.post = ab;
        // the capture only recorded the work: roles and buffers as they were
        ab = g.pre;
        ctx->curPos = pos0; ctx->curPred = pred0; ctx->keysIdx = keys0;
        ctx->launches = launches0;
        if (rc != PBF_OK || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            if (rc != PBF_OK) return rc;
            return fail(ctx, PBF_ERR_CUDA, std::string("reverse-pass graph capture: ") + cudaGetErrorString(e));
        }
        size_t count = 0;  // its kernel launches (the memsets and tape copies are not counted)
        cudaGraphGetNodes(graph, nullptr, &count);
        std::vector<cudaGraphNode_t> nodes(count);
        if (count) cudaGraphGetNodes(graph, nodes.data(), &count);
        for (cudaGraphNode_t node : nodes) {
            cudaGraphNodeType type;
            if (cudaGraphNodeGetType(node, &type) == cudaSuccess && type == cudaGraphNodeTypeKernel) ++g.nodes;
        }
        const cudaError_t ei = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) return fail(ctx, PBF_ERR_CUDA, std::string("reverse-pass graph: ") + cudaGetErrorString(ei));
        ctx->segGraphs.push_back(g);
        hit = &ctx->segGraphs.back();
    }
    PBF_CUDA(ctx, cudaGraphLaunch(hit->exec, s));
    ab = hit->post;
    ctx->launches += hit->nodes;
    // the replayed substeps leave the roles as the eager ones do: an unpaused
    // substep keeps the position role and ends with the sorted keys and
    // predictions in their second buffers
    if (len > 0) {
        ctx->keysIdx = ctx->plan.passes & 1;
        ctx->curPred = 1;
    }
    return PBF_OK;
}

// Host memory the driver has page-locked (allocated or registered by CUDA)
bool page_locked(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeHost;
}
}  // namespace

// ================================================================ C-ABI ==
extern "C" {

const char* pbf_last_error(const pbf_ctx* ctx) {
    return ctx ? ctx->lastError.c_str() : pbf::tls_error.c_str();
}

int pbf_create_batch(const PbfParameters* scenes, int nscenes, int device, pbf_ctx** out) {
    if (!scenes || !out || nscenes < 1) return fail(nullptr, PBF_ERR_INVALID, "pbf_create_batch: bad arguments");
    if (nscenes > 65535) return fail(nullptr, PBF_ERR_INVALID, "pbf_create_batch: at most 65535 scenes");
    std::vector<PbfParameters> sp(scenes, scenes + nscenes);
    if (int rc = check_batch_compatible(nullptr, sp)) return rc;
    uint64_t total = 0;
    for (const auto& p : sp) {
        if (p.particleCount < 1) return fail(nullptr, PBF_ERR_INVALID, "pbf_create_batch: a scene has no particles");
        total += p.particleCount;
    }
    if (total > PBF_MAX_PARTICLES) return fail(nullptr, PBF_ERR_INVALID, "pbf_create_batch: more than 2^26 particles in all");
    if ((uint64_t)nscenes * sp[0].gridBufSize > (1ull << 28))
        return fail(nullptr, PBF_ERR_INVALID, "pbf_create_batch: scenes x gridBufSize must be <= 2^28");
    PbfParameters merged = sp[0];
    merged.particleCount = (unsigned)total;
    int rc = pbf_create(&merged, device, out);
    if (rc) return rc;
    if (nscenes > 1) {
        (*out)->sceneParams = sp;
        (*out)->sceneOffsets.assign(1, 0u);
        for (const auto& p : sp) (*out)->sceneOffsets.push_back((*out)->sceneOffsets.back() + p.particleCount);
    }
    return PBF_OK;
}

int pbf_scene_offsets(pbf_ctx* ctx, uint32_t* offsets) {
    if (!ctx || !offsets) return fail(ctx, PBF_ERR_INVALID, "pbf_scene_offsets: NULL argument");
    if (!is_batch(ctx)) { offsets[0] = 0; offsets[1] = ctx->params.particleCount; return PBF_OK; }
    std::copy(ctx->sceneOffsets.begin(), ctx->sceneOffsets.end(), offsets);
    return PBF_OK;
}

int pbf_create(const PbfParameters* params, int device, pbf_ctx** out) {
    if (!params || !out) return fail(nullptr, PBF_ERR_INVALID, "pbf_create: NULL argument");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0)
        return fail(nullptr, PBF_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (device < 0 || device >= count) return fail(nullptr, PBF_ERR_INVALID, "pbf_create: device ordinal out of range");
    std::unique_ptr<pbf_ctx> ctx(new pbf_ctx());
    ctx->params = *params;
    ctx->device = device;
    PBF_CUDA(nullptr, cudaSetDevice(device));
    PBF_CUDA(nullptr, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    // [0]: the error word; [1]: the substep counter of the taint marks (pbf::DevConsts::epoch)
    PBF_CUDA(nullptr, cudaMalloc((void**)&ctx->errWord, 2 * sizeof(int)));
    PBF_CUDA(nullptr, cudaMemset(ctx->errWord, 0, 2 * sizeof(int)));
    PBF_CUDA(nullptr, cudaMalloc((void**)&ctx->tileCounters, 10 * sizeof(int)));
    PBF_CUDA(nullptr, cudaMemset(ctx->tileCounters, 0, 10 * sizeof(int)));
    *out = ctx.release();
    return PBF_OK;
}

int pbf_destroy(pbf_ctx* ctx) {
    if (!ctx) return PBF_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    drop_graph(ctx);
    for (int k = 0; k < 2; ++k) {
        dev_free(ctx->pos[k]); dev_free(ctx->pred[k]); dev_free(ctx->vel[k]);
        dev_free(ctx->keys[k]); dev_free(ctx->perm[k]);
    }
    dev_free(ctx->omega); dev_free(ctx->density); dev_free(ctx->hist); dev_free(ctx->cells);
    dev_free(ctx->list); dev_free(ctx->flat); dev_free(ctx->meta); dev_free(ctx->errWord); dev_free(ctx->tileCounters);
    dev_free(ctx->taint); dev_free(ctx->cellXYZ); dev_free(ctx->cellStart);
    dev_free(ctx->scenes); dev_free(ctx->sceneOf); dev_free(ctx->ids); dev_free(ctx->idsTmp);
    dev_free(ctx->quadsDev); dev_free(ctx->maskDev); dev_free(ctx->waveDev);
    if (ctx->timingAnchor) cudaEventDestroy(ctx->timingAnchor);
    if (ctx->evPosReady) cudaEventDestroy(ctx->evPosReady);
    if (ctx->evCopyDone) cudaEventDestroy(ctx->evCopyDone);
    if (ctx->evVelHead) cudaEventDestroy(ctx->evVelHead);
    if (ctx->copyStream) cudaStreamDestroy(ctx->copyStream);
    free_render(ctx);
    free_rollout(ctx);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return PBF_OK;
}

int pbf_init_buffers(pbf_ctx* ctx, const float* init_pos, const float* init_vel) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    const PbfParameters& p = ctx->params;
    if (p.particleCount < 1 || p.particleCount > PBF_MAX_PARTICLES)
        return fail(ctx, PBF_ERR_INVALID, "particleCount must be in [1, 2^26]");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    drop_graph(ctx);
    const int n = (int)p.particleCount;
    if (n != ctx->n) free_rollout(ctx);
    ctx->n = n;
    ++ctx->epoch;
    int rc;
    for (int k = 0; k < 2; ++k) {
        if ((rc = dev_alloc(ctx, &ctx->pos[k], n)) || (rc = dev_alloc(ctx, &ctx->pred[k], n)) ||
            (rc = dev_alloc(ctx, &ctx->vel[k], n)) || (rc = dev_alloc(ctx, &ctx->keys[k], n)) ||
            (rc = dev_alloc(ctx, &ctx->perm[k], n)))
            return rc;
        PBF_CUDA(ctx, cudaMemset(ctx->keys[k], 0, 4 * (size_t)n));
        PBF_CUDA(ctx, cudaMemset(ctx->pred[k], 0, 16 * (size_t)n));
    }
    if ((rc = dev_alloc(ctx, &ctx->omega, n)) || (rc = dev_alloc(ctx, &ctx->density, n)) ||
        (rc = dev_alloc(ctx, &ctx->ids, n)) || (rc = dev_alloc(ctx, &ctx->idsTmp, n)))
        return rc;
    {
        iota_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, ctx->ids);
        PBF_CUDA(ctx, cudaGetLastError());
    }
    PBF_CUDA(ctx, cudaMemset(ctx->omega, 0, 16 * (size_t)n));
    PBF_CUDA(ctx, cudaMemset(ctx->density, 0, 4 * (size_t)n));
    ctx->curPos = 0; ctx->curVel = 0; ctx->curPred = 1; ctx->keysIdx = 0; ctx->stepped = false;
    std::vector<float> host;
    const float* src = init_pos;
    if (!src) {
        host.assign(4 * (size_t)n, 0.0f);
        if (is_batch(ctx)) {
            for (size_t s = 0; s < ctx->sceneParams.size(); ++s)
                if ((rc = pbf_reference_lattice(&ctx->sceneParams[s], host.data() + 4 * (size_t)ctx->sceneOffsets[s])))
                    return fail(ctx, rc, pbf_last_error(nullptr));
        } else if ((rc = pbf_reference_lattice(&p, host.data())) != PBF_OK) {
            return fail(ctx, rc, pbf_last_error(nullptr));
        }
        src = host.data();
    }
    if (is_batch(ctx)) {
        std::vector<uint16_t> ids(n);
        for (size_t s = 0; s + 1 < ctx->sceneOffsets.size(); ++s)
            std::fill(ids.begin() + ctx->sceneOffsets[s], ids.begin() + ctx->sceneOffsets[s + 1], (uint16_t)s);
        if ((rc = dev_alloc(ctx, &ctx->sceneOf, n))) return rc;
        PBF_CUDA(ctx, cudaMemcpy(ctx->sceneOf, ids.data(), 2 * (size_t)n, cudaMemcpyHostToDevice));
    }
    PBF_CUDA(ctx, cudaMemcpy(ctx->pos[0], src, 16 * (size_t)n, cudaMemcpyHostToDevice));
    if (init_vel) PBF_CUDA(ctx, cudaMemcpy(ctx->vel[0], init_vel, 16 * (size_t)n, cudaMemcpyHostToDevice));
    else PBF_CUDA(ctx, cudaMemset(ctx->vel[0], 0, 16 * (size_t)n));
    PBF_CUDA(ctx, cudaMemset(ctx->vel[1], 0, 16 * (size_t)n));
    ctx->buffersReady = true;
    ctx->cellsReady = ctx->cellsReady && ctx->cellsN == n;  // friend rows are sized per particle
    ctx->kernelsReady = false;
    return PBF_OK;
}

int pbf_init_cells(pbf_ctx* ctx) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    if (!ctx->buffersReady) return fail(ctx, PBF_ERR_STATE, "InitBuffers must run before InitCells");
    const PbfParameters& p = ctx->params;
    if (p.gridBufSize < 1 || p.gridBufSize > (1u << 30)) return fail(ctx, PBF_ERR_INVALID, "gridBufSize must be in [1, 2^30]");
    if (p.friendsCircles < 1 || p.friendsCircles > PBF_MAX_CIRCLES || p.particlesPerCircle < 1 ||
        p.particlesPerCircle > PBF_MAX_PER_CIRCLE)
        return fail(ctx, PBF_ERR_INVALID, "friendsCircles must be in [1, 8] and particlesPerCircle in [1, 64]");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    drop_graph(ctx);
    int rc;
    const size_t tableWords = (size_t)p.gridBufSize * (is_batch(ctx) ? ctx->sceneParams.size() : 1);
    if ((rc = dev_alloc(ctx, &ctx->cells, 2 * tableWords))) return rc;
    PBF_CUDA(ctx, cudaMemset(ctx->cells, 0xFF, 8 * tableWords));
    ctx->cellsWords = p.gridBufSize;
    ctx->listSlots = (int)(p.friendsCircles * p.particlesPerCircle);
    ctx->cellsN = ctx->n;
    ++ctx->epoch;
    if ((rc = dev_alloc(ctx, &ctx->list, (size_t)ctx->listSlots * ctx->n)) ||
        (rc = dev_alloc(ctx, &ctx->flat, (size_t)ctx->listSlots * ctx->n)) || (rc = dev_alloc(ctx, &ctx->meta, ctx->n)) ||
        (rc = dev_alloc(ctx, &ctx->taint, ctx->n)) || (rc = dev_alloc(ctx, &ctx->cellXYZ, ctx->n)) ||
        (rc = dev_alloc(ctx, &ctx->cellStart, tableWords)))
        return rc;
    PBF_CUDA(ctx, cudaMemset(ctx->meta, 0, 8 * (size_t)ctx->n));
    // taint marks are substep numbers from 1 on (the counter restarts with them); no cell start yet
    PBF_CUDA(ctx, cudaMemset(ctx->taint, 0, 4 * (size_t)ctx->n));
    PBF_CUDA(ctx, cudaMemset(ctx->errWord + 1, 0, sizeof(int)));
    PBF_CUDA(ctx, cudaMemset(ctx->cellStart, 0xFF, 4 * tableWords));
    apply_planes(ctx);
    ctx->cellsReady = true;
    ctx->kernelsReady = false;
    return PBF_OK;
}

int pbf_load_force_masks(pbf_ctx* ctx, const uint32_t* mask, int width, int height) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    if (!mask) {
        dev_free(ctx->maskDev);
        ctx->maskDev = nullptr;
        ctx->maskW = ctx->maskH = 0;
    } else {
        if (width < 1 || height < 1 || (uint64_t)width * (uint64_t)height > (1ull << 28))
            return fail(ctx, PBF_ERR_INVALID, "pbf_load_force_masks: width and height must be >= 1, at most 2^28 texels");
        const size_t texels = (size_t)width * height;
        if (int rc = dev_alloc(ctx, &ctx->maskDev, texels)) return rc;
        PBF_CUDA(ctx, cudaMemcpy(ctx->maskDev, mask, 4 * texels, cudaMemcpyHostToDevice));
        ctx->maskW = width;
        ctx->maskH = height;
    }
    ++ctx->epoch;
    drop_graph(ctx);
    apply_planes(ctx);
    return PBF_OK;
}

int pbf_set_force_quads(pbf_ctx* ctx, const PbfForceQuad* quads, int count) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    if (count < 0 || count > PBF_MAX_FORCE_QUADS || (count > 0 && !quads))
        return fail(ctx, PBF_ERR_INVALID, "pbf_set_force_quads: count must be 0 .. PBF_MAX_FORCE_QUADS with quads given");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    dev_free(ctx->quadsDev);
    ctx->quadsDev = nullptr;
    ctx->nquads = 0;
    if (count > 0) {
        std::vector<pbf::QuadDev> q(count);
        for (int k = 0; k < count; ++k) q[k] = quad_constants(quads[k]);
        if (int rc = dev_alloc(ctx, &ctx->quadsDev, (size_t)count)) return rc;
        PBF_CUDA(ctx, cudaMemcpy(ctx->quadsDev, q.data(), sizeof(pbf::QuadDev) * count, cudaMemcpyHostToDevice));
        ctx->nquads = count;
    }
    ++ctx->epoch;
    drop_graph(ctx);
    apply_planes(ctx);
    return PBF_OK;
}

// ---- state files: "PBFSTATE", version, N, sizeof(PbfParameters), the
// parameters, then positions, velocities (float4 each) and particle ids, in
// the current record order, little-endian as the host writes them.
namespace {
constexpr char kStateMagic[8] = {'P', 'B', 'F', 'S', 'T', 'A', 'T', 'E'};
constexpr uint32_t kStateVersion = 1;
}  // namespace

int pbf_save_state(pbf_ctx* ctx, const char* path) {
    if (!ctx || !path) return fail(ctx, PBF_ERR_INVALID, "pbf_save_state: NULL argument");
    if (!ctx->buffersReady) return fail(ctx, PBF_ERR_STATE, "InitBuffers has not run");
    const size_t n = (size_t)ctx->n;
    std::vector<float> pos(4 * n), vel(4 * n);
    std::vector<uint32_t> ids(n);
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    PBF_CUDA(ctx, cudaMemcpyAsync(pos.data(), ctx->pos[ctx->curPos], 16 * n, cudaMemcpyDeviceToHost, ctx->stream));
    PBF_CUDA(ctx, cudaMemcpyAsync(vel.data(), ctx->vel[ctx->curVel], 16 * n, cudaMemcpyDeviceToHost, ctx->stream));
    PBF_CUDA(ctx, cudaMemcpyAsync(ids.data(), ctx->ids, 4 * n, cudaMemcpyDeviceToHost, ctx->stream));
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(ctx, PBF_ERR_INVALID, std::string("pbf_save_state: cannot open ") + path);
    const uint32_t head[3] = {kStateVersion, (uint32_t)n, (uint32_t)sizeof(PbfParameters)};
    bool ok = std::fwrite(kStateMagic, 1, 8, f) == 8 && std::fwrite(head, 4, 3, f) == 3 &&
              std::fwrite(&ctx->params, sizeof(PbfParameters), 1, f) == 1 &&
              std::fwrite(pos.data(), 16, n, f) == n && std::fwrite(vel.data(), 16, n, f) == n &&
              std::fwrite(ids.data(), 4, n, f) == n;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return fail(ctx, PBF_ERR_INVALID, std::string("pbf_save_state: write failed: ") + path);
    return PBF_OK;
}

int pbf_load_state(pbf_ctx* ctx, const char* path) {
    if (!ctx || !path) return fail(ctx, PBF_ERR_INVALID, "pbf_load_state: NULL argument");
    if (!ctx->buffersReady) return fail(ctx, PBF_ERR_STATE, "InitBuffers has not run");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(ctx, PBF_ERR_INVALID, std::string("pbf_load_state: cannot open ") + path);
    char magic[8];
    uint32_t head[3];
    PbfParameters saved;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kStateMagic, 8) == 0 &&
              std::fread(head, 4, 3, f) == 3 && head[0] == kStateVersion && head[2] == sizeof(PbfParameters) &&
              std::fread(&saved, sizeof(PbfParameters), 1, f) == 1;
    if (!ok) { std::fclose(f); return fail(ctx, PBF_ERR_INVALID, std::string("pbf_load_state: not a state file: ") + path); }
    if ((int)head[1] != ctx->n) {
        std::fclose(f);
        return fail(ctx, PBF_ERR_INVALID, "pbf_load_state: the file holds " + std::to_string(head[1]) +
                                              " particles, the context " + std::to_string(ctx->n));
    }
    const size_t n = (size_t)ctx->n;
    std::vector<float> pos(4 * n), vel(4 * n);
    std::vector<uint32_t> ids(n);
    ok = std::fread(pos.data(), 16, n, f) == n && std::fread(vel.data(), 16, n, f) == n &&
         std::fread(ids.data(), 4, n, f) == n;
    std::fclose(f);
    if (!ok) return fail(ctx, PBF_ERR_INVALID, std::string("pbf_load_state: truncated file: ") + path);
    std::vector<uint8_t> seen(n, 0);
    for (uint32_t id : ids) {
        if (id >= n || seen[id]) return fail(ctx, PBF_ERR_INVALID, "pbf_load_state: particle ids are not a permutation");
        seen[id] = 1;
    }
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    PBF_CUDA(ctx, cudaMemcpyAsync(ctx->pos[ctx->curPos], pos.data(), 16 * n, cudaMemcpyHostToDevice, ctx->stream));
    PBF_CUDA(ctx, cudaMemcpyAsync(ctx->vel[ctx->curVel], vel.data(), 16 * n, cudaMemcpyHostToDevice, ctx->stream));
    PBF_CUDA(ctx, cudaMemcpyAsync(ctx->ids, ids.data(), 4 * n, cudaMemcpyHostToDevice, ctx->stream));
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return PBF_OK;
}

int pbf_render_camera(const float eye[3], const float at[3], const float up[3], float fovyDeg, int width, int height,
                      float pointSize, PbfCamera* cam) {
    if (!eye || !at || !up || !cam || width < 1 || height < 1 || !(fovyDeg > 0.0f && fovyDeg < 180.0f))
        return fail(nullptr, PBF_ERR_INVALID, "pbf_render_camera: bad arguments");
    const double PI = 3.14159265358979323846;
    double f[3] = {(double)at[0] - eye[0], (double)at[1] - eye[1], (double)at[2] - eye[2]};
    auto norm = [](double* v) {
        const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int k = 0; k < 3; ++k) v[k] /= l;
    };
    auto cross = [](const double* a, const double* b, double* o) {
        o[0] = a[1] * b[2] - a[2] * b[1]; o[1] = a[2] * b[0] - a[0] * b[2]; o[2] = a[0] * b[1] - a[1] * b[0];
    };
    norm(f);
    const double upd[3] = {up[0], up[1], up[2]};
    double s[3], v[3];
    cross(f, upd, s);
    norm(s);
    cross(s, f, v);
    const double e[3] = {eye[0], eye[1], eye[2]};
    auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    // glm::lookAt, column-major m[col * 4 + row]
    double mv[16] = {s[0], v[0], -f[0], 0, s[1], v[1], -f[1], 0, s[2], v[2], -f[2], 0, -dot(s, e), -dot(v, e), dot(f, e), 1};
    // inverse of the rigid transform: rotation transposed, then the eye
    double imv[16] = {s[0], s[1], s[2], 0, v[0], v[1], v[2], 0, -f[0], -f[1], -f[2], 0, e[0], e[1], e[2], 1};
    const double aspect = (double)width / (double)height, zn = 0.1, zf = 1000.0;
    const double th = std::tan(fovyDeg * PI / 180.0 / 2.0);
    double pr[16] = {0};
    pr[0] = 1.0 / (aspect * th);
    pr[5] = 1.0 / th;
    pr[10] = -(zf + zn) / (zf - zn);
    pr[11] = -1.0;
    pr[14] = -(2.0 * zf * zn) / (zf - zn);
    for (int k = 0; k < 16; ++k) {
        cam->modelView[k] = (float)mv[k];
        cam->invModelView[k] = (float)imv[k];
        cam->projection[k] = (float)pr[k];
    }
    cam->invFocalLen[0] = (float)(th * aspect);
    cam->invFocalLen[1] = (float)th;
    cam->depthRange[0] = 0.1f;
    cam->depthRange[1] = 1000.0f;
    cam->widthOfNearPlane = (float)(width / (2.0 * std::tan(0.5 * fovyDeg * PI / 180.0)));
    cam->pointSize = pointSize;
    cam->width = width;
    cam->height = height;
    return PBF_OK;
}

int pbf_render_frame(pbf_ctx* ctx, const PbfCamera* cam, int mode) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!cam || cam->width < 1 || cam->height < 1 || cam->width > 8192 || cam->height > 8192 || mode < 0 || mode > 2)
        return fail(ctx, PBF_ERR_INVALID, "pbf_render_frame: camera size must be 1..8192 and mode 0..2");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    pbf::RenderBuffers& r = ctx->render;
    const size_t pixels = (size_t)cam->width * cam->height;
    if (r.width != cam->width || r.height != cam->height || r.n != ctx->n) {
        free_render(ctx);
        const size_t n = (size_t)ctx->n;
        r.plan = pbf::make_sort_plan(ctx->n, 1u << 23);
        if ((rc = dev_alloc(ctx, &r.dkey, pixels)) || (rc = dev_alloc(ctx, &r.splat, pixels)) ||
            (rc = dev_alloc(ctx, &r.smooth, pixels)) || (rc = dev_alloc(ctx, &r.out, pixels)) ||
            (rc = dev_alloc(ctx, &r.vis, n)) || (rc = dev_alloc(ctx, &r.keys[0], n)) ||
            (rc = dev_alloc(ctx, &r.keys[1], n)) || (rc = dev_alloc(ctx, &r.perm[0], n)) ||
            (rc = dev_alloc(ctx, &r.perm[1], n)) || (rc = dev_alloc(ctx, &r.hist, r.plan.histWords)) ||
            (rc = dev_alloc(ctx, &r.cells, pbf::render_grid_words()))) {
            free_render(ctx);
            return rc;
        }
        r.width = cam->width;
        r.height = cam->height;
        r.n = ctx->n;
    }
    pbf::render_frame(*cam, mode, ctx->n, ctx->params.h, ctx->pos[ctx->curPos], r, ctx->stream);
    ctx->launches += pbf::render_launches(mode, r.plan);
    ctx->renderMode = mode;
    PBF_CUDA(ctx, cudaGetLastError());
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return PBF_OK;
}

int pbf_render_read(pbf_ctx* ctx, int which, float* rgba) {
    if (!ctx || !rgba) return fail(ctx, PBF_ERR_INVALID, "pbf_render_read: NULL argument");
    if (ctx->renderMode < 0) return fail(ctx, PBF_ERR_STATE, "pbf_render_frame has not run");
    const pbf::RenderBuffers& r = ctx->render;
    const float4* src = which == 0 ? r.out : which == 1 ? r.splat : which == 2 ? r.smooth : nullptr;
    if (!src || (which == 2 && ctx->renderMode != 0))
        return fail(ctx, PBF_ERR_INVALID, "pbf_render_read: which is 0, 1, or 2 after a mode 0 frame");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    PBF_CUDA(ctx, cudaMemcpyAsync(rgba, src, 16 * (size_t)r.width * r.height, cudaMemcpyDeviceToHost, ctx->stream));
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return PBF_OK;
}

int pbf_set_wave_position(pbf_ctx* ctx, float wavePos) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    if (!(wavePos == wavePos) || wavePos < 0.0f) return fail(ctx, PBF_ERR_INVALID, "pbf_set_wave_position: wavePos must be >= 0");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    if (!ctx->waveDev) {
        if (int rc = dev_alloc(ctx, &ctx->waveDev, 1)) return rc;
        drop_graph(ctx);  // the kernels now read the wall offset
        apply_planes(ctx);
    }
    ++ctx->epoch;
    // stream-ordered: steps enqueued before see the old wall, steps after the new one
    PBF_CUDA(ctx, cudaMemcpyAsync(ctx->waveDev, &wavePos, sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return PBF_OK;
}

// src/Runner.cpp:100-116
float pbf_wave_position(const PbfParameters* p, float waveTime) {
    if (!p) return 0.0f;
    const double push = (double)p->waveGenAmp * ((double)p->xMax - (double)p->xMin);
    const double t = (double)p->waveGenFreq * (double)waveTime;
    const double phase = std::pow(std::fmod(t, 1.0), (double)p->waveGenDuty);
    return (float)((1.0 - std::cos(2.0 * 3.14159265358979323846 * phase)) * push / 2.0);
}

int pbf_init_kernels(pbf_ctx* ctx) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    if (!ctx->buffersReady || !ctx->cellsReady) return fail(ctx, PBF_ERR_STATE, "InitBuffers and InitCells must run before InitKernels");
    int rc = validate(ctx, ctx->params);
    if (rc) return rc;
    if ((int)ctx->params.particleCount != ctx->n || ctx->cellsN != ctx->n)
        return fail(ctx, PBF_ERR_INVALID, "particleCount changed since InitBuffers or InitCells");
    if (ctx->params.gridBufSize != ctx->cellsWords ||
        (int)(ctx->params.friendsCircles * ctx->params.particlesPerCircle) != ctx->listSlots)
        return fail(ctx, PBF_ERR_INVALID, "gridBufSize or friend limits changed since InitCells");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    drop_graph(ctx);
    ++ctx->epoch;
    ctx->consts = pbf::make_consts(ctx->params, ctx->n);
    apply_planes(ctx);
    uint64_t keyRange = ctx->params.gridBufSize;
    if (is_batch(ctx)) {
        const size_t S = ctx->sceneParams.size();
        keyRange *= S;
        std::vector<pbf::SceneParams> table(S);
        for (size_t s = 0; s < S; ++s)
            table[s] = pbf::make_scene_params(ctx->sceneParams[s], (uint32_t)(s * ctx->params.gridBufSize));
        if ((rc = dev_alloc(ctx, &ctx->scenes, S))) return rc;
        PBF_CUDA(ctx, cudaMemcpy(ctx->scenes, table.data(), sizeof(pbf::SceneParams) * S, cudaMemcpyHostToDevice));
    }
    ctx->plan = pbf::make_sort_plan(ctx->n, (uint32_t)keyRange);
    if (ctx->plan.histWords != ctx->histWords) {
        if ((rc = dev_alloc(ctx, &ctx->hist, ctx->plan.histWords))) return rc;
        ctx->histWords = ctx->plan.histWords;
    }
    ctx->kernelsReady = true;
    return PBF_OK;
}

int pbf_set_params(pbf_ctx* ctx, const PbfParameters* params) {
    if (!ctx || !params) return fail(ctx, PBF_ERR_INVALID, "pbf_set_params: NULL argument");
    if (is_batch(ctx)) return fail(ctx, PBF_ERR_UNSUPPORTED, "pbf_set_params applies to single-scene contexts");
    int rc = validate(ctx, *params);
    if (rc) return rc;
    if (ctx->buffersReady && (int)params->particleCount != ctx->n)
        return fail(ctx, PBF_ERR_INVALID, "pbf_set_params cannot change particleCount; re-run InitBuffers");
    if (ctx->cellsReady && (params->gridBufSize != ctx->cellsWords ||
                            (int)(params->friendsCircles * params->particlesPerCircle) != ctx->listSlots))
        return fail(ctx, PBF_ERR_INVALID, "pbf_set_params cannot change gridBufSize or friend limits; re-run InitCells");
    ctx->params = *params;
    ++ctx->epoch;
    if (ctx->kernelsReady) {
        drop_graph(ctx);
        ctx->consts = pbf::make_consts(ctx->params, ctx->n);
        apply_planes(ctx);
    }
    return PBF_OK;
}

int pbf_set_pause(pbf_ctx* ctx, int paused) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    if ((paused ? 1 : 0) != ctx->paused) ++ctx->epoch;
    ctx->paused = paused ? 1 : 0;
    return PBF_OK;
}

int pbf_step_async(pbf_ctx* ctx, int substeps) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (substeps < 0) return fail(ctx, PBF_ERR_INVALID, "substeps must be >= 0");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    StageClock clock{ctx, {}};
    if (ctx->stageTiming) std::fill(ctx->stageMs.begin(), ctx->stageMs.end(), 0.0f);
    for (int k = 0; k < substeps; ++k) {
        const bool graphOk = ctx->useGraph && !ctx->paused && !ctx->stageTiming;
        if (graphOk) {
            if (!ctx->graph.exec || ctx->graph.pos != ctx->curPos)
                if ((rc = capture_graph(ctx, false))) return rc;
            PBF_CUDA(ctx, cudaGraphLaunch(ctx->graph.exec, ctx->stream));
            // the replayed substep has the captured buffer roles
            ctx->keysIdx = ctx->plan.passes & 1;
            ctx->curPred = 1;
            ctx->launches += ctx->graph.kernels;
        } else {
            if ((rc = enqueue_substep(ctx, ctx->stageTiming ? &clock : nullptr))) return rc;
        }
        ctx->stepped = true;
    }
    if (ctx->stageTiming) return clock.finish();
    return PBF_OK;
}

int pbf_step_read_async(pbf_ctx* ctx, int substeps, float* pos, float* vel) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (substeps < 1) return fail(ctx, PBF_ERR_INVALID, "pbf_step_read_async: substeps must be >= 1");
    if (ctx->stageTiming) {  // the trackers time whole substeps: no overlap
        if ((rc = pbf_step_async(ctx, substeps))) return rc;
        return pbf_read_state_async(ctx, pos, vel, nullptr);
    }
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    if (substeps > 1 && (rc = pbf_step_async(ctx, substeps - 1))) return rc;
    if (pos) {
        if (!ctx->copyStream) PBF_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copyStream, cudaStreamNonBlocking));
        if (!ctx->evPosReady) PBF_CUDA(ctx, cudaEventCreateWithFlags(&ctx->evPosReady, cudaEventDisableTiming));
        if (!ctx->evCopyDone) PBF_CUDA(ctx, cudaEventCreateWithFlags(&ctx->evCopyDone, cudaEventDisableTiming));
        if (!ctx->evVelHead) PBF_CUDA(ctx, cudaEventCreateWithFlags(&ctx->evVelHead, cudaEventDisableTiming));
    }
    ctx->readPos = pos;
    ctx->readVel = vel;
    // the last substep with its copies: a captured graph when both
    // destinations are page-locked (a graph's copy nodes keep their addresses)
    const bool graphOk = ctx->useGraph && !ctx->paused && (!pos || page_locked(pos)) && (!vel || page_locked(vel));
    if (graphOk) {
        pbf_ctx::StepGraph& g = ctx->readGraph;
        if (!g.exec || g.pos != ctx->curPos || g.host[0] != pos || g.host[1] != vel) rc = capture_graph(ctx, true);
        if (rc == PBF_OK) {
            const cudaError_t e = cudaGraphLaunch(g.exec, ctx->stream);
            if (e != cudaSuccess) rc = fail(ctx, PBF_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
        }
        if (rc == PBF_OK) {  // the replayed substep has the captured buffer roles, as in pbf_step_async
            ctx->keysIdx = ctx->plan.passes & 1;
            ctx->curPred = 1;
            ctx->launches += g.kernels;
        }
    } else {
        rc = enqueue_substep(ctx, nullptr);
    }
    ctx->readPos = nullptr;
    ctx->readVel = nullptr;
    if (rc) return rc;
    ctx->stepped = true;
    return PBF_OK;
}

int pbf_synchronize(pbf_ctx* ctx) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    PBF_CUDA(ctx, cudaGetLastError());
    return read_error_word(ctx);
}

int pbf_step(pbf_ctx* ctx, int substeps) {
    int rc = pbf_step_async(ctx, substeps);
    if (rc) return rc;
    return pbf_synchronize(ctx);
}

int pbf_read_state(pbf_ctx* ctx, float* pos, float* vel, float* pred) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    if (!ctx->buffersReady) return fail(ctx, PBF_ERR_STATE, "InitBuffers has not run");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = 16 * (size_t)ctx->n;
    if (pos) PBF_CUDA(ctx, cudaMemcpyAsync(pos, ctx->pos[ctx->curPos], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    if (vel) PBF_CUDA(ctx, cudaMemcpyAsync(vel, ctx->vel[ctx->curVel], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    if (pred) PBF_CUDA(ctx, cudaMemcpyAsync(pred, ctx->pred[ctx->curPred], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return PBF_OK;
}

int pbf_write_state_async(pbf_ctx* ctx, const float* pos, const float* vel) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    if (!ctx->buffersReady) return fail(ctx, PBF_ERR_STATE, "InitBuffers has not run");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = 16 * (size_t)ctx->n;
    if (pos) {
        PBF_CUDA(ctx, cudaMemcpyAsync(ctx->pos[ctx->curPos], pos, bytes, cudaMemcpyHostToDevice, ctx->stream));
        // the written records become particles 0 .. N-1
        iota_kernel<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, ctx->ids);
        PBF_CUDA(ctx, cudaGetLastError());
    }
    if (vel) PBF_CUDA(ctx, cudaMemcpyAsync(ctx->vel[ctx->curVel], vel, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return PBF_OK;
}

int pbf_write_state(pbf_ctx* ctx, const float* pos, const float* vel) {
    int rc = pbf_write_state_async(ctx, pos, vel);
    if (rc) return rc;
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return PBF_OK;
}

int pbf_read_state_async(pbf_ctx* ctx, float* pos, float* vel, float* pred) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    if (!ctx->buffersReady) return fail(ctx, PBF_ERR_STATE, "InitBuffers has not run");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = 16 * (size_t)ctx->n;
    if (pos) PBF_CUDA(ctx, cudaMemcpyAsync(pos, ctx->pos[ctx->curPos], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    if (vel) PBF_CUDA(ctx, cudaMemcpyAsync(vel, ctx->vel[ctx->curVel], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    if (pred) PBF_CUDA(ctx, cudaMemcpyAsync(pred, ctx->pred[ctx->curPred], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return PBF_OK;
}

int pbf_device_positions(pbf_ctx* ctx, void** dptr) {
    if (!ctx || !dptr) return fail(ctx, PBF_ERR_INVALID, "pbf_device_positions: NULL argument");
    if (!ctx->buffersReady) return fail(ctx, PBF_ERR_STATE, "InitBuffers has not run");
    *dptr = ctx->pos[ctx->curPos];
    return PBF_OK;
}

int pbf_get_stream(pbf_ctx* ctx, void** stream) {
    if (!ctx || !stream) return fail(ctx, PBF_ERR_INVALID, "pbf_get_stream: NULL argument");
    *stream = (void*)ctx->stream;
    return PBF_OK;
}

int pbf_sort_state(pbf_ctx* ctx, const float* pred, uint32_t* keys, uint32_t* perm, uint32_t* cells) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!pred) return fail(ctx, PBF_ERR_INVALID, "pbf_sort_state: pred is NULL");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    const int n = ctx->n;
    const uint32_t grid = (uint32_t)(ctx->params.gridBufSize * (is_batch(ctx) ? ctx->sceneParams.size() : 1));
    float4* dPred = nullptr;
    uint32_t *k[2] = {nullptr, nullptr}, *pm[2] = {nullptr, nullptr}, *dCells = nullptr, *dHist = nullptr;
    auto cleanup = [&] {
        cudaFree(dPred); cudaFree(k[0]); cudaFree(k[1]); cudaFree(pm[0]); cudaFree(pm[1]);
        cudaFree(dCells); cudaFree(dHist);
    };
    cudaError_t e = cudaSuccess;
    if ((e = cudaMalloc((void**)&dPred, 16 * (size_t)n)) || (e = cudaMalloc((void**)&k[0], 4 * (size_t)n)) ||
        (e = cudaMalloc((void**)&k[1], 4 * (size_t)n)) || (e = cudaMalloc((void**)&pm[0], 4 * (size_t)n)) ||
        (e = cudaMalloc((void**)&pm[1], 4 * (size_t)n)) || (e = cudaMalloc((void**)&dCells, 8 * (size_t)grid)) ||
        (e = cudaMalloc((void**)&dHist, 4 * ctx->plan.histWords))) {
        cleanup();
        return fail(ctx, PBF_ERR_CUDA, std::string("pbf_sort_state: ") + cudaGetErrorString(e));
    }
    cudaStream_t s = ctx->stream;
    auto keep = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };  // the first error of the sequence
    keep(cudaMemcpyAsync(dPred, pred, 16 * (size_t)n, cudaMemcpyHostToDevice, s));
    keep(cudaMemsetAsync(dCells, 0xFF, 8 * (size_t)grid, s));
    pbf::launch_compute_keys(ctx->consts, batch_of(ctx), dPred, k[0], pm[0], s);
    const int r = pbf::launch_radix_sort(ctx->plan, k, pm, dHist, nullptr, nullptr, nullptr, nullptr, s);
    pbf::launch_update_cells(n, k[r], dCells, grid, nullptr, s);
    const uint32_t nKeys = ((uint32_t)n + 2047u) / 2048u * 2048u;
    if (keys) keep(cudaMemcpyAsync(keys, k[r], 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    if (perm) keep(cudaMemcpyAsync(perm, pm[r], 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    if (cells) keep(cudaMemcpyAsync(cells, dCells, 8 * (size_t)grid, cudaMemcpyDeviceToHost, s));
    keep(cudaStreamSynchronize(s));
    if (e == cudaSuccess) e = cudaGetLastError();
    cleanup();
    if (e != cudaSuccess) return fail(ctx, PBF_ERR_CUDA, std::string("pbf_sort_state: ") + cudaGetErrorString(e));
    // The reference sorts IntCeil(N, 2048) keys, the tail padded with
    // 2147483646 (radixsort.cl:17), which sorts after every cell key.
    for (uint32_t i = (uint32_t)n; i < nKeys; ++i) {
        if (keys) keys[i] = 2147483646u;
        if (perm) perm[i] = i;
    }
    return PBF_OK;
}

int pbf_read_sort(pbf_ctx* ctx, uint32_t* keys, uint32_t* perm, uint32_t* cells) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!ctx->stepped) return fail(ctx, PBF_ERR_STATE, "no substep has run yet");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    const int n = ctx->n;
    cudaStream_t s = ctx->stream;
    const uint32_t* k = ctx->keys[ctx->keysIdx];
    const uint32_t tableKeys = ctx->cellsWords * (uint32_t)(is_batch(ctx) ? ctx->sceneParams.size() : 1);
    if (keys) PBF_CUDA(ctx, cudaMemcpyAsync(keys, k, 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    if (perm) PBF_CUDA(ctx, cudaMemcpyAsync(perm, ctx->perm[ctx->keysIdx], 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    if (cells) {  // the substep's table, rebuilt in the (empty) table and cleared again
        pbf::launch_update_cells(n, k, ctx->cells, tableKeys, ctx->errWord, s);
        PBF_CUDA(ctx, cudaMemcpyAsync(cells, ctx->cells, 8 * (size_t)tableKeys, cudaMemcpyDeviceToHost, s));
        pbf::launch_reset_cells(n, k, ctx->cells, tableKeys, ctx->errWord, s);
    }
    PBF_CUDA(ctx, cudaStreamSynchronize(s));
    PBF_CUDA(ctx, cudaGetLastError());
    const uint32_t nKeys = ((uint32_t)n + 2047u) / 2048u * 2048u;
    for (uint32_t i = (uint32_t)n; i < nKeys; ++i) {
        if (keys) keys[i] = 2147483646u;
        if (perm) perm[i] = i;
    }
    return PBF_OK;
}

int pbf_read_friends(pbf_ctx* ctx, uint32_t* counts, uint32_t* list, int list_slots) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!ctx->stepped) return fail(ctx, PBF_ERR_STATE, "no substep has run yet");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    const int n = ctx->n;
    std::vector<uint2> meta(n);
    PBF_CUDA(ctx, cudaMemcpyAsync(meta.data(), ctx->meta, 8 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
    // the kept friends of every particle in order: the flat rows the passes walk
    const int slots = list ? std::min(list_slots, ctx->listSlots) : 0;
    std::vector<uint32_t> rows((size_t)std::max(slots, 0) * n);
    if (slots > 0)
        PBF_CUDA(ctx, cudaMemcpyAsync(rows.data(), ctx->flat, 4 * rows.size(), cudaMemcpyDeviceToHost, ctx->stream));
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < n; ++i) {
        const uint64_t m = (uint64_t)meta[i].x | ((uint64_t)meta[i].y << 32);
        const int keptL = (int)(m >> 56) & 0xF, keptD = (int)(m >> 60) & 0xF;
        uint32_t nl = 0, nd = 0;
        for (int k = 0; k < keptL; ++k) {
            const uint32_t cnt = (uint32_t)(m >> (7 * k)) & 0x7Fu;
            nl += cnt;
            if (k < keptD) nd += cnt;
        }
        for (int t = 0; t < slots && t < (int)nl; ++t) list[(size_t)t * n + i] = rows[(size_t)t * n + i];
        if (counts) { counts[2 * i] = nl; counts[2 * i + 1] = nd; }
    }
    return PBF_OK;
}

int pbf_enable_stage_timing(pbf_ctx* ctx, int enable) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    const bool was = ctx->stageTiming;
    ctx->stageTiming = enable != 0;
    ctx->stageNames.clear();
    ctx->stageMs.clear();
    if (ctx->stageTiming && !was) {
        ctx->trackers.clear();
        PBF_CUDA(ctx, cudaSetDevice(ctx->device));
        if (!ctx->timingAnchor) PBF_CUDA(ctx, cudaEventCreate(&ctx->timingAnchor));
        PBF_CUDA(ctx, cudaEventRecord(ctx->timingAnchor, ctx->stream));
    }
    return PBF_OK;
}

int pbf_enable_nvtx(pbf_ctx* ctx, int enable) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    ctx->nvtx = enable != 0;
    return PBF_OK;
}

int pbf_perf_trackers(pbf_ctx* ctx, PbfPerfTracker* out, int capacity, int* count) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    const int k = (int)ctx->trackers.size();
    if (count) *count = k;
    if (out)
        for (int i = 0; i < std::min(k, capacity); ++i) out[i] = ctx->trackers[i];
    return PBF_OK;
}

int pbf_perf_export_json(pbf_ctx* ctx, char* buf, size_t capacity, size_t* length) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    std::string s = "{\"trackers\": [";
    double total = 0.0;
    char line[256];
    for (size_t i = 0; i < ctx->trackers.size(); ++i) {
        const PbfPerfTracker& t = ctx->trackers[i];
        std::snprintf(line, sizeof line,
                      "%s{\"eventName\": \"%s\", \"time_start\": %llu, \"time_end\": %llu, \"total_time\": %.6f, "
                      "\"last_time\": %.6f}",
                      i ? ", " : "", t.eventName, (unsigned long long)t.time_start, (unsigned long long)t.time_end,
                      t.total_time, t.last_time);
        s += line;
        total += t.total_time;
    }
    std::snprintf(line, sizeof line, "], \"total_time\": %.6f, \"unit\": \"ms\"}", total);
    s += line;
    if (length) *length = s.size() + 1;
    if (buf && capacity) std::snprintf(buf, capacity, "%s", s.c_str());
    return PBF_OK;
}

int pbf_stage_timings(pbf_ctx* ctx, float* ms, int capacity, int* count, char* names, size_t names_len) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    const int k = (int)ctx->stageNames.size();
    if (count) *count = k;
    if (ms)
        for (int i = 0; i < std::min(k, capacity); ++i) ms[i] = ctx->stageMs[i];
    if (names && names_len) {
        std::string joined;
        for (int i = 0; i < k; ++i) { if (i) joined += '\n'; joined += ctx->stageNames[i]; }
        std::snprintf(names, names_len, "%s", joined.c_str());
    }
    return PBF_OK;
}

int pbf_launch_count(pbf_ctx* ctx, uint64_t* count) {
    if (!ctx || !count) return fail(ctx, PBF_ERR_INVALID, "pbf_launch_count: NULL argument");
    *count = ctx->launches;
    return PBF_OK;
}

int pbf_get_launch_shape(pbf_ctx* ctx, int* blocks) {
    if (!ctx || !blocks) return fail(ctx, PBF_ERR_INVALID, "pbf_get_launch_shape: NULL argument");
    const pbf::LaunchShape& s = ctx->shape;
    blocks[0] = s.friends; blocks[1] = s.scaling; blocks[2] = s.delta; blocks[3] = s.viscosity; blocks[4] = s.vorticity;
    blocks[5] = s.friendsAlgorithm;
    blocks[6] = s.balance;
    blocks[7] = s.persistent;
    return PBF_OK;
}

int pbf_set_launch_shape(pbf_ctx* ctx, const int* blocks) {
    if (!ctx || !blocks) return fail(ctx, PBF_ERR_INVALID, "pbf_set_launch_shape: NULL argument");
    for (int k = 0; k < 5; ++k)
        if (blocks[k] < 32 || blocks[k] > pbf::kMaxBlock || blocks[k] % 32)
            return fail(ctx, PBF_ERR_INVALID, "block sizes must be multiples of 32 in [32, 512]");
    if (blocks[5] < 0 || blocks[5] > 2) return fail(ctx, PBF_ERR_INVALID, "the friends algorithm is 0, 1 or 2");
    if (blocks[6] != 0 && blocks[6] != 1) return fail(ctx, PBF_ERR_INVALID, "the balance flag is 0 or 1");
    if (blocks[7] != 0 && blocks[7] != 1) return fail(ctx, PBF_ERR_INVALID, "the persistent flag is 0 or 1");
    ctx->shape.friends = blocks[0]; ctx->shape.scaling = blocks[1]; ctx->shape.delta = blocks[2];
    ctx->shape.viscosity = blocks[3]; ctx->shape.vorticity = blocks[4]; ctx->shape.friendsAlgorithm = blocks[5];
    ctx->shape.balance = blocks[6];
    ctx->shape.persistent = blocks[7];
    drop_graph(ctx);
    return PBF_OK;
}

// Times `trial_substeps` substeps from the current state with every candidate
// block size and keeps, for each neighbour kernel, the fastest.  The state is
// saved before and restored after every trial, so the simulation continues
// from where it was; every block size gives bit-identical results.
int pbf_autotune(pbf_ctx* ctx, int trial_substeps, int* blocks_out) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (trial_substeps < 1) return fail(ctx, PBF_ERR_INVALID, "pbf_autotune: trial_substeps must be >= 1");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const size_t n = (size_t)ctx->n;
    float4 *savePos = nullptr, *saveVel = nullptr;
    float* saveDensity = nullptr;
    uint32_t *saveKeys = nullptr, *saveIds = nullptr;
    auto release = [&] {
        cudaFree(savePos); cudaFree(saveVel); cudaFree(saveDensity); cudaFree(saveKeys); cudaFree(saveIds);
    };
    if (cudaMalloc((void**)&savePos, 16 * n) || cudaMalloc((void**)&saveVel, 16 * n) ||
        cudaMalloc((void**)&saveDensity, 4 * n) || cudaMalloc((void**)&saveKeys, 4 * n) ||
        cudaMalloc((void**)&saveIds, 4 * n)) {
        release();
        cudaGetLastError();
        return fail(ctx, PBF_ERR_CUDA, "pbf_autotune: cannot allocate the state copy");
    }
    const int pos0 = ctx->curPos, vel0 = ctx->curVel, pred0 = ctx->curPred, keys0 = ctx->keysIdx;
    const bool stepped0 = ctx->stepped, timing0 = ctx->stageTiming;
    const uint64_t launches0 = ctx->launches;
    const pbf::LaunchShape shape0 = ctx->shape;
    const std::vector<PbfPerfTracker> trackers0 = ctx->trackers;  // trials do not count as steps
    // the trials step the state (and permute the particle records and their
    // ids); the copy taken here is put back after each of them
    auto copy_state = [&](bool back) {
        struct { void* live; void* saved; size_t bytes; } parts[5] = {
            {ctx->pos[pos0], savePos, 16 * n}, {ctx->vel[vel0], saveVel, 16 * n},
            {ctx->density, saveDensity, 4 * n}, {ctx->keys[keys0], saveKeys, 4 * n}, {ctx->ids, saveIds, 4 * n}};
        cudaError_t err = cudaSuccess;
        for (const auto& q : parts) {
            const cudaError_t e1 = back ? cudaMemcpyAsync(q.live, q.saved, q.bytes, cudaMemcpyDeviceToDevice, ctx->stream)
                                        : cudaMemcpyAsync(q.saved, q.live, q.bytes, cudaMemcpyDeviceToDevice, ctx->stream);
            if (err == cudaSuccess) err = e1;
        }
        return err;
    };
    if (cudaError_t e0 = copy_state(false)) {
        cudaStreamSynchronize(ctx->stream);
        release();
        return fail(ctx, PBF_ERR_CUDA, std::string("pbf_autotune: state copy: ") + cudaGetErrorString(e0));
    }
    cudaError_t restoreErr = cudaSuccess;
    auto restore = [&] {
        ctx->curPos = pos0; ctx->curVel = vel0; ctx->curPred = pred0; ctx->keysIdx = keys0;
        const cudaError_t e1 = copy_state(true);
        if (restoreErr == cudaSuccess) restoreErr = e1;
    };
    const char* names[5] = {"buildFriendsList", "computeScaling", "computeDelta", "applyViscosity", "applyVorticity"};
    const int candidates[4] = {64, 128, 256, 512};
    // friends: best over block size x algorithm; the solver passes: best
    // block size per balance setting, then the balance setting with the
    // smaller sum
    float friendsMs = 1e30f;
    int friendsBlock = shape0.friends, algorithm = shape0.friendsAlgorithm;
    float solverMs[2][4];
    int solverBlock[2][4];
    for (int bal = 0; bal < 2; ++bal)
        for (int q = 0; q < 4; ++q) { solverMs[bal][q] = 1e30f; solverBlock[bal][q] = 256; }
    ctx->stageTiming = true;
    for (int trial = 0; trial < 24; ++trial) {
        // block size x friends algorithm (3) x balanced thread map (2)
        const int cand = candidates[trial % 4], algo = (trial / 4) % 3, bal = trial / 12;
        ctx->shape = pbf::LaunchShape{cand, cand, cand, cand, cand, algo, bal, 0};
        ctx->stageNames.clear();
        ctx->stageMs.clear();
        StageClock clock{ctx, {}};
        for (int k = 0; k < trial_substeps && rc == PBF_OK; ++k) rc = enqueue_substep(ctx, &clock);
        if (rc == PBF_OK) rc = clock.finish();
        restore();
        if (rc != PBF_OK) break;
        for (int q = 0; q < 5; ++q)
            for (size_t k = 0; k < ctx->stageNames.size(); ++k) {
                if (ctx->stageNames[k] != names[q]) continue;
                const float ms = ctx->stageMs[k];
                if (q == 0 && ms < friendsMs) { friendsMs = ms; friendsBlock = cand; algorithm = algo; }
                if (q > 0 && ms < solverMs[bal][q - 1]) { solverMs[bal][q - 1] = ms; solverBlock[bal][q - 1] = cand; }
            }
    }
    float sum[2] = {0.0f, 0.0f};
    for (int bal = 0; bal < 2; ++bal)
        for (int q = 0; q < 4; ++q) sum[bal] += solverMs[bal][q];
    const int balance = sum[1] <= sum[0] ? 1 : 0;
    int choice[5] = {friendsBlock, solverBlock[balance][0], solverBlock[balance][1], solverBlock[balance][2],
                     solverBlock[balance][3]};
    // then one block per tile against a persistent grid walking the tiles,
    // with that shape: the smaller sum of the five neighbour stages (the
    // better of two trials each, alternated)
    float persistMs[2] = {1e30f, 1e30f};
    for (int trial = 0; trial < 4 && rc == PBF_OK; ++trial) {
        const int pers = trial & 1;
        ctx->shape = pbf::LaunchShape{choice[0], choice[1], choice[2], choice[3], choice[4], algorithm, balance, pers};
        ctx->stageNames.clear();
        ctx->stageMs.clear();
        StageClock clock{ctx, {}};
        for (int k = 0; k < trial_substeps && rc == PBF_OK; ++k) rc = enqueue_substep(ctx, &clock);
        if (rc == PBF_OK) rc = clock.finish();
        restore();
        if (rc != PBF_OK) break;
        float ms = 0.0f;
        for (int q = 0; q < 5; ++q)
            for (size_t k = 0; k < ctx->stageNames.size(); ++k)
                if (ctx->stageNames[k] == names[q]) ms += ctx->stageMs[k];
        persistMs[pers] = std::min(persistMs[pers], ms);
    }
    const int persistent = persistMs[1] < persistMs[0] ? 1 : 0;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) e = restoreErr;
    release();
    ctx->trackers = trackers0;
    ctx->stageTiming = timing0;
    ctx->stageNames.clear();
    ctx->stageMs.clear();
    ctx->stepped = stepped0;
    ctx->launches = launches0;
    drop_graph(ctx);
    if (rc != PBF_OK) { ctx->shape = shape0; return rc; }
    if (e != cudaSuccess) { ctx->shape = shape0; return fail(ctx, PBF_ERR_CUDA, std::string("pbf_autotune: ") + cudaGetErrorString(e)); }
    ctx->shape = pbf::LaunchShape{choice[0], choice[1], choice[2], choice[3], choice[4], algorithm, balance, persistent};
    if (blocks_out) {
        for (int q = 0; q < 5; ++q) blocks_out[q] = choice[q];
        blocks_out[5] = algorithm;
        blocks_out[6] = balance;
        blocks_out[7] = persistent;
    }
    return read_error_word(ctx);
}

int pbf_read_ids(pbf_ctx* ctx, uint32_t* ids) {
    if (!ctx || !ids) return fail(ctx, PBF_ERR_INVALID, "pbf_read_ids: NULL argument");
    if (!ctx->buffersReady) return fail(ctx, PBF_ERR_STATE, "InitBuffers has not run");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    PBF_CUDA(ctx, cudaMemcpyAsync(ids, ctx->ids, 4 * (size_t)ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
    PBF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return PBF_OK;
}

int pbf_rollout_forward(pbf_ctx* ctx, int substeps, int checkpoint_every) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (is_batch(ctx)) return fail(ctx, PBF_ERR_UNSUPPORTED, "rollouts run on single-scene contexts");
    if (ctx->paused) return fail(ctx, PBF_ERR_STATE, "rollouts need an unpaused simulation");
    if (ctx->nquads > 0) return fail(ctx, PBF_ERR_UNSUPPORTED, "rollouts do not differentiate force planes");
    if (ctx->params.completeNeighbours)
        return fail(ctx, PBF_ERR_UNSUPPORTED, "rollouts follow the reference's neighbour sets (completeNeighbours 0)");
    if (substeps < 1 || checkpoint_every < 1) return fail(ctx, PBF_ERR_INVALID, "substeps and checkpoint_every must be >= 1");
    if (ctx->params.simIterations < 1 || ctx->params.simIterations > 64)
        return fail(ctx, PBF_ERR_INVALID, "rollouts need 1..64 solver iterations");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    const int segments = (substeps + checkpoint_every - 1) / checkpoint_every;
    for (auto& k : ctx->ckpt) { dev_free(k.pos); dev_free(k.vel); dev_free(k.ids); }
    ctx->ckpt.assign(segments, pbf_ctx::Checkpoint{});
    for (int sgm = 0; sgm < segments; ++sgm) {
        if ((rc = save_checkpoint(ctx, ctx->ckpt[sgm]))) return rc;
        const int len = std::min(checkpoint_every, substeps - sgm * checkpoint_every);
        if ((rc = pbf_step_async(ctx, len))) return rc;
    }
    if ((rc = save_checkpoint(ctx, ctx->ckptEnd))) return rc;
    ctx->rollSubsteps = substeps;
    ctx->rollEvery = checkpoint_every;
    ctx->rollEpoch = ctx->epoch;
    return pbf_synchronize(ctx);
}

int pbf_rollout_backward(pbf_ctx* ctx, const float* dL_dx, float* dL_dv0, float* dL_dvisc, float* dL_dg) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!dL_dx) return fail(ctx, PBF_ERR_INVALID, "pbf_rollout_backward: dL_dx is NULL");
    if (ctx->ckpt.empty() || ctx->rollSubsteps < 1) return fail(ctx, PBF_ERR_STATE, "pbf_rollout_forward has not run");
    // the recomputed segments must be the substeps the forward pass took
    if (ctx->rollEpoch != ctx->epoch)
        return fail(ctx, PBF_ERR_STATE,
                    "the buffers, parameters, pause, force planes or wave wall changed since pbf_rollout_forward");
    PBF_CUDA(ctx, cudaSetDevice(ctx->device));
    if ((rc = ensure_tape(ctx))) return rc;
    drop_step_graph(ctx);
    const int n = ctx->n, iters = (int)ctx->params.simIterations, every = ctx->rollEvery;
    const size_t v4 = 16 * (size_t)n;
    cudaStream_t s = ctx->stream;
    pbf::AdjointBuffers ab = ctx->adj;  // adjoint_substep swaps its pointers
    PBF_CUDA(ctx, cudaMemcpyAsync(ctx->adjById, dL_dx, v4, cudaMemcpyHostToDevice, s));
    pbf::scatter_by_id(n, ctx->ckptEnd.ids, ctx->adjById, ab.xb, s);
    PBF_CUDA(ctx, cudaMemsetAsync(ab.vb, 0, v4, s));
    PBF_CUDA(ctx, cudaMemsetAsync(ab.scalars, 0, 16, s));
    ctx->launches += 1;
    const int segments = (int)ctx->ckpt.size();
    for (int sgm = segments - 1; sgm >= 0 && rc == PBF_OK; --sgm) {
        if ((rc = load_checkpoint(ctx, ctx->ckpt[sgm]))) break;
        const int len = std::min(every, ctx->rollSubsteps - sgm * every);
        if (ctx->useGraph) {
            rc = run_segment_graph(ctx, len, ab);
        } else {
            for (int k = 0; k < len && rc == PBF_OK; ++k) rc = enqueue_substep(ctx, nullptr, &ctx->tapes[k]);
            for (int k = len - 1; k >= 0 && rc == PBF_OK; --k) {
                pbf::adjoint_substep(ctx->consts, ctx->tapes[k], ab, s);
                ctx->launches += pbf::adjoint_launches(iters);
            }
        }
    }
    if (rc) return rc;
    pbf::gather_to_id(n, ctx->ckpt[0].ids, ab.vb, ctx->adjById, s);
    ctx->launches += 1;
    if (dL_dv0) PBF_CUDA(ctx, cudaMemcpyAsync(dL_dv0, ctx->adjById, v4, cudaMemcpyDeviceToHost, s));
    float sc[4] = {0, 0, 0, 0};
    PBF_CUDA(ctx, cudaMemcpyAsync(sc, ab.scalars, 16, cudaMemcpyDeviceToHost, s));
    if ((rc = load_checkpoint(ctx, ctx->ckptEnd))) return rc;
    PBF_CUDA(ctx, cudaStreamSynchronize(s));
    PBF_CUDA(ctx, cudaGetLastError());
    if (dL_dvisc) *dL_dvisc = sc[0];
    if (dL_dg) { dL_dg[0] = sc[1]; dL_dg[1] = sc[2]; dL_dg[2] = sc[3]; }
    return read_error_word(ctx);
}

int pbf_use_graph(pbf_ctx* ctx, int enable) {
    if (!ctx) return fail(nullptr, PBF_ERR_INVALID, "NULL context");
    ctx->useGraph = enable != 0;
    if (!ctx->useGraph) drop_graph(ctx);
    return PBF_OK;
}

}  // extern "C"
