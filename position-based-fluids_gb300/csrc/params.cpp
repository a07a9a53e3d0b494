// params.cpp — scenario parameters: the `.par` loader and the initial-state
// generators.  Host code only; compiled with -ffp-contract=off so that the
// generated positions are bit-identical on every host.

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <iostream>
#include <random>
#include <sstream>
#include <string>

#include "pbf_capi.h"
#include "pbf_internal.h"

namespace {

// The loader's computed fields (src/ParamUtils.cpp:97-99).
void apply_computed_fields(PbfParameters* p) {
    p->h_2 = p->h * p->h;
    p->friendsCircles = 5;
    p->particlesPerCircle = 50;
}

}  // namespace

extern "C" int pbf_default_parameters(PbfParameters* out) {
    if (!out) return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_default_parameters: out is NULL");
    std::memset(out, 0, sizeof(*out));
    apply_computed_fields(out);
    return PBF_OK;
}

// Same grammar and error behaviour as LoadParameters (src/ParamUtils.cpp:24-100).
extern "C" int pbf_load_parameters(const char* text, PbfParameters* p, int* unknown) {
    if (!text || !p) return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_load_parameters: NULL argument");
    int nUnknown = 0;
    std::istringstream in{std::string(text)};
    std::string line, key;
    while (std::getline(in, line)) {
        // A line read up to end-of-input without a newline leaves the stream
        // not good(); the reference reports it and stops (ParamUtils.cpp:34-38).
        if (!in.good()) {
            std::cerr << "Error parsing parameters file" << std::endl;
            break;
        }
        line.erase(std::find(line.begin(), line.end(), '#'), line.end());
        if (line.empty()) continue;
        std::transform(line.begin(), line.end(), line.begin(), [](unsigned char c) { return (char)std::tolower(c); });
        std::istringstream fields(line);
        if (!(fields >> key)) {
            std::cerr << "Unable to read parameter" << std::endl;
            continue;
        }
        if (key == "resetsimonchange") fields >> p->resetSimOnChange;
        else if (key == "particlecount") fields >> p->particleCount;
        else if (key == "xmin") fields >> p->xMin;
        else if (key == "xmax") fields >> p->xMax;
        else if (key == "ymin") fields >> p->yMin;
        else if (key == "ymax") fields >> p->yMax;
        else if (key == "zmin") fields >> p->zMin;
        else if (key == "zmax") fields >> p->zMax;
        else if (key == "wavegenamp") fields >> p->waveGenAmp;
        else if (key == "wavegenfreq") fields >> p->waveGenFreq;
        else if (key == "wavegenduty") fields >> p->waveGenDuty;
        else if (key == "timestep") fields >> p->timeStep;
        else if (key == "simiterations") fields >> p->simIterations;
        else if (key == "substeps") fields >> p->subSteps;
        else if (key == "smoothlen") fields >> p->h;
        else if (key == "gridbuffersize") fields >> p->gridBufSize;
        else if (key == "restdensity") fields >> p->restDensity;
        else if (key == "epsilon") fields >> p->epsilon;
        else if (key == "garvity") fields >> p->garvity;
        else if (key == "vorticityfactor") fields >> p->vorticityFactor;
        else if (key == "viscosityfactor") fields >> p->viscosityFactor;
        else if (key == "surfacetenstionk") fields >> p->surfaceTenstionK;
        else if (key == "surfacetenstiondist") fields >> p->surfaceTenstionDist;
        else if (key == "setupspacing") fields >> p->setupSpacing;
        else if (key == "segmentsize") fields >> p->segmentSize;
        else if (key == "sortiterations") fields >> p->sortIterations;
        else if (key == "particlerendersize") fields >> p->particleRenderSize;
        else if (key == "enablecachedbuffers") fields >> p->EnableCachedBuffers;
        // Keys added by this library.
        else if (key == "gravityx") { fields >> p->gravityX; p->gravityVectorEnable = 1; }
        else if (key == "gravityy") { fields >> p->gravityY; p->gravityVectorEnable = 1; }
        else if (key == "gravityz") { fields >> p->gravityZ; p->gravityVectorEnable = 1; }
        else if (key == "boxclamp") fields >> p->boxClamp;
        else if (key == "zerodistanceguard") fields >> p->zeroDistanceGuard;
        else if (key == "relaxedmath") fields >> p->relaxedMath;
        else if (key == "completeneighbours") fields >> p->completeNeighbours;
        else if (key == "blockdims" || key == "blockorigin" || key == "jitter" || key == "seed") {
            // scene keys (pbf_load_scene)
        } else {
            std::cerr << "Unknown parameter " << key << std::endl << "Leaving it out." << std::endl;
            ++nUnknown;
        }
    }
    apply_computed_fields(p);
    if (unknown) *unknown = nUnknown;
    return PBF_OK;
}

// The scene keys of a `.par` file: BlockDims nx ny nz, BlockOrigin x y z,
// Jitter j, Seed s.  Other keys are left to pbf_load_parameters.
extern "C" int pbf_load_scene(const char* text, PbfScene* scene) {
    if (!text || !scene) return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_load_scene: NULL argument");
    std::memset(scene, 0, sizeof(*scene));
    std::istringstream in{std::string(text)};
    std::string line, key;
    bool dims = false;
    while (std::getline(in, line)) {
        line.erase(std::find(line.begin(), line.end(), '#'), line.end());
        std::transform(line.begin(), line.end(), line.begin(), [](unsigned char c) { return (char)std::tolower(c); });
        std::istringstream fields(line);
        if (!(fields >> key)) continue;
        if (key == "blockdims") dims = (bool)(fields >> scene->blockDims[0] >> scene->blockDims[1] >> scene->blockDims[2]);
        else if (key == "blockorigin") fields >> scene->blockOrigin[0] >> scene->blockOrigin[1] >> scene->blockOrigin[2];
        else if (key == "jitter") fields >> scene->jitter;
        else if (key == "seed") fields >> scene->seed;
    }
    if (!dims || scene->blockDims[0] < 1 || scene->blockDims[1] < 1 || scene->blockDims[2] < 1)
        return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_load_scene: no valid BlockDims line");
    return PBF_OK;
}

// The scene's particles: a BlockDims lattice at spacing SmoothLen x
// SetupSpacing (the reference's spacing, src/Simulation.cpp:77) from
// BlockOrigin, jittered by U(-Jitter, Jitter) from Seed (pbf_scene_block).
extern "C" int pbf_scene_positions(const PbfParameters* p, const PbfScene* s, float* pos) {
    if (!p || !s || !pos) return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_scene_positions: NULL argument");
    return pbf_scene_block(s->blockDims[0], s->blockDims[1], s->blockDims[2], p->h * p->setupSpacing,
                           s->blockOrigin[0], s->blockOrigin[1], s->blockOrigin[2], s->jitter, s->seed, pos);
}

// Simulation::CreateParticles (src/Simulation.cpp:71-101): a cube of
// ceil(cbrt(N)) particles per axis at spacing h*setupSpacing, index i mapped
// to (x, y, z) = ((i/P) % P, i % P, (i/P^2) % P).
extern "C" int pbf_reference_lattice(const PbfParameters* p, float* pos) {
    if (!p || !pos) return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_reference_lattice: NULL argument");
    const unsigned N = p->particleCount;
    const int P = (int)std::ceil(std::pow((double)N, 1 / 3.0));
    const float d = p->h * p->setupSpacing;
    const float offX = (1.0f - P * d) / 2.0f;
    const float offY = 0.3f;
    const float offZ = (1.0f - P * d) / 2.0f;
    for (unsigned i = 0; i < N; ++i) {
        unsigned x = ((unsigned)(i / std::pow((double)P, 1.0)) % P);
        unsigned y = ((unsigned)(i / std::pow((double)P, 0.0)) % P);
        unsigned z = ((unsigned)(i / std::pow((double)P, 2.0)) % P);
        pos[4 * (size_t)i + 0] = offX + x * d;
        pos[4 * (size_t)i + 1] = offY + y * d;
        pos[4 * (size_t)i + 2] = offZ + z * d;
        pos[4 * (size_t)i + 3] = 0.0f;
    }
    return PBF_OK;
}

// Jittered block lattice used by the dam-break scenarios.  The uniform draw
// takes the top 53 bits of each 64-bit Mersenne Twister output, so the values
// do not depend on the standard library's distribution classes.
extern "C" int pbf_scene_block(int nx, int ny, int nz, float spacing, float ox, float oy, float oz,
                               float jitter, uint64_t seed, float* pos) {
    if (!pos || nx <= 0 || ny <= 0 || nz <= 0)
        return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_scene_block: bad arguments");
    std::mt19937_64 rng(seed);
    const double s = spacing, j = jitter;
    const double o[3] = {ox, oy, oz};
    size_t i = 0;
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix, ++i) {
                const int idx[3] = {ix, iy, iz};
                for (int c = 0; c < 3; ++c) {
                    double u = (double)(rng() >> 11) * 0x1.0p-53;  // [0, 1)
                    pos[4 * i + c] = (float)(o[c] + idx[c] * s + (2.0 * u - 1.0) * j);
                }
                pos[4 * i + 3] = 0.0f;
            }
    return PBF_OK;
}

// Double dam break: two blocks of n/2 particles each (the second takes the
// odd one), aspect 1:2:1 in x:y:z, standing on the floor in opposite x/z
// corners of a 2:1:1 box whose volume is n * spacing^3 / fill.  Each block is
// a lattice of a x 2a x a sites with a the smallest integer holding its
// particles, filled x fastest, then z, then y, so only its top layer can be
// partial.  Jitter as in pbf_scene_block (one std::mt19937_64 stream for both
// blocks).  box receives xMin, xMax, yMin, yMax, zMin, zMax.
extern "C" int pbf_scene_double_dam_break(int n, float spacing, float fill, float jitter, uint64_t seed,
                                          float* pos, float* box) {
    if (!pos || !box || n < 2 || !(spacing > 0.0f) || !(fill > 0.0f) || !(fill <= 1.0f))
        return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_scene_double_dam_break: bad arguments");
    const double s = spacing;
    const double side = std::cbrt((double)n * s * s * s / fill / 2.0);  // box is 2*side x side x side
    const double bx[6] = {0.0, 2.0 * side, 0.0, side, 0.0, side};
    for (int k = 0; k < 6; ++k) box[k] = (float)bx[k];
    std::mt19937_64 rng(seed);
    size_t out = 0;
    for (int b = 0; b < 2; ++b) {
        const int count = b == 0 ? n / 2 : n - n / 2;
        int a = 1;
        while ((long long)a * (2 * a) * a < count) ++a;
        // block 0 at the low x/z corner, block 1 at the high one, half a spacing from the walls
        const double ox = b == 0 ? 0.5 * s : bx[1] - (a - 0.5) * s;
        const double oz = b == 0 ? 0.5 * s : bx[5] - (a - 0.5) * s;
        const double oy = 0.5 * s;
        int placed = 0;
        for (int iy = 0; iy < 2 * a && placed < count; ++iy)
            for (int iz = 0; iz < a && placed < count; ++iz)
                for (int ix = 0; ix < a && placed < count; ++ix, ++placed, ++out) {
                    const double o[3] = {ox + ix * s, oy + iy * s, oz + iz * s};
                    for (int c = 0; c < 3; ++c) {
                        const double u = (double)(rng() >> 11) * 0x1.0p-53;
                        pos[4 * out + c] = (float)(o[c] + (2.0 * u - 1.0) * jitter);
                    }
                    pos[4 * out + 3] = 0.0f;
                }
    }
    return PBF_OK;
}
