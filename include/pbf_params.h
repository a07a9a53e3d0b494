/*
 * pbf_params.h — scenario parameters of the PBF substep pipeline.
 *
 * PbfParameters keeps the field order, types and meaning of the reference's
 * `struct Parameters` (src/Parameters.hpp:5-56; the kernel-side copy is
 * assets/kernels/parameters.hpp) so that a caller holding a filled
 * `Parameters` can hand its bytes over unchanged: the prefix up to and
 * including `EnableCachedBuffers` is layout-identical.  New fields are only
 * appended after it.
 *
 * Reference semantics kept verbatim, including the misspelled names
 * (`garvity`, `surfaceTenstionK`, `surfaceTenstionDist`):
 *   - mass is implicitly 1;
 *   - `garvity` is a scalar applied along -y (predict_positions.cl:13) unless
 *     the appended gravity vector is enabled;
 *   - `friendsCircles` / `particlesPerCircle` are forced to 5 / 50 and
 *     `h_2 = h*h` by the loader (src/ParamUtils.cpp:97-99);
 *   - xMin..zMax are never read by the reference kernels; here they bound the
 *     box clamp when `boxClamp` is set.
 */
#ifndef PBF_PARAMS_H
#define PBF_PARAMS_H

#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct PbfParameters {
    /* ---- prefix identical to src/Parameters.hpp:5-56 ---- */
    int          resetSimOnChange;
    unsigned int particleCount;
    float        xMin, xMax, yMin, yMax, zMin, zMax;
    float        waveGenAmp, waveGenFreq, waveGenDuty;
    float        timeStep;
    unsigned int simIterations;
    unsigned int subSteps;
    float        h;
    float        restDensity;
    float        epsilon;
    float        garvity;
    float        vorticityFactor;
    float        viscosityFactor;
    float        surfaceTenstionK;
    float        surfaceTenstionDist;
    unsigned int friendsCircles;
    unsigned int particlesPerCircle;
    unsigned int gridBufSize;
    float        setupSpacing;
    unsigned int segmentSize;
    unsigned int sortIterations;
    float        particleRenderSize;
    float        h_2;
    bool         EnableCachedBuffers;
    /* ---- appended fields (not in the reference) ---- */
    /* 0: gravity is (0, -garvity, 0) exactly as the reference;
       1: gravity is (gravityX, gravityY, gravityZ). */
    int          gravityVectorEnable;
    float        gravityX, gravityY, gravityZ;
    /* 1: clamp pred + delta_p to [xMin,xMax]x[yMin,yMax]x[zMin,zMax] inside
       the delta-p stage, after the position update is formed and before the
       delta is taken.  0: no clamp (the reference's behaviour). */
    int          boxClamp;
    /* 1: a neighbour at distance exactly 0 contributes nothing to the density,
       delta-p, viscosity and vorticity sums.  0: it is summed as in the
       reference, where r / |r| is 0/0 and the particle's state becomes NaN
       (compute_scaling.cl:76-83, compute_delta.cl:142-146). */
    int          zeroDistanceGuard;
    /* 0: the four neighbour passes evaluate the reference kernels in strict
       IEEE FP32, bit-identical to the oracle.  1: relaxed FP32 in those
       passes, as the reference's own -cl-fast-relaxed-math -cl-mad-enable
       build (src/Simulation.cpp:160): one hardware reciprocal square root
       per pair in place of a square root and three divisions, and fused
       multiply-adds.  Keys, sort, cell table and friend lists stay exact;
       one substep stays within 1e-5 relative of the exact result. */
    int          relaxedMath;
    /* 0: the reference's neighbour sets: the density pass keeps the friend
       circles up to 60 % of the friends, the other passes up to 50 %
       (compute_scaling.cl:50, compute_delta.cl:100), and the density leaves
       out the particle itself.  1: physically complete sets: every friend
       circle in every pass, and the density includes the particle's own
       W(0) term, added first. */
    int          completeNeighbours;
} PbfParameters;

/* One force plane of the delta-p stage: BouncePointQuad's arguments
   (compute_delta.cl:1-42), which the reference hard-codes as 14 calls
   (compute_delta.cl:169-182).  The quad is B + s E0 + t E1 for s, t in
   [0, 1]; a point that reaches it from the inside is moved onto it where the
   force mask texel (t * 512, maskYOffset + s * maskHeight) is non-zero. */
typedef struct PbfForceQuad {
    float   B[3], E0[3], E1[3];
    int32_t maskYOffset, maskHeight;
} PbfForceQuad;

/* The camera of the reference's particle renderer (src/visual/visual.cpp:108-127,
   src/ZPR.cpp:32-37), as data.  Matrices are column-major, as glm hands them
   to OpenGL.  depthRange is the (near, far) that fluid_depth_smoothing.fs and
   fluid_final_render.fs linearise depth with (0.1, 1000 in the reference). */
typedef struct PbfCamera {
    float modelView[16];
    float invModelView[16];
    float projection[16];
    float invFocalLen[2];
    float depthRange[2];
    float widthOfNearPlane;
    float pointSize;         /* Params.particleRenderSize */
    int32_t width, height;   /* pixels, each at most 8192 */
} PbfCamera;

/* The initial block of a scenario file (`.par` keys BlockDims, BlockOrigin,
   Jitter, Seed; the spacing is SmoothLen x SetupSpacing, as the reference's
   CreateParticles spaces its lattice).  The reference's loader reports these
   keys as unknown and skips them, so the files stay readable by it. */
typedef struct PbfScene {
    int32_t  blockDims[3];
    float    blockOrigin[3];
    float    jitter;
    uint64_t seed;
} PbfScene;

/* Largest number of force planes. */
#define PBF_MAX_FORCE_QUADS        64

/* Largest friend-circle configuration the kernels accept. */
#define PBF_MAX_CIRCLES            8
#define PBF_MAX_PER_CIRCLE         64
/* Largest particle count: the reference's sort limit _N = 1<<23
   (assets/kernels/hesp.hpp:77) times 8. */
#define PBF_MAX_PARTICLES          (1u << 26)

#ifdef __cplusplus
}
#endif

#endif /* PBF_PARAMS_H */
