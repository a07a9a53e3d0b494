// pbf_oracle.cpp — TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference's per-substep PBF pipeline
// (Simulation::Step, src/Simulation.cpp:554-621, and the OpenCL kernels in
// assets/kernels/*.cl).  It is the checker for the CUDA path: the tests, the
// smoke check and the benchmark's CPU-baseline leg call it; the product never
// does.
//
// Arithmetic contract.  Every floating-point expression follows the
// evaluation order of the kernel source it restates, one IEEE operation at a
// time, with no fused multiply-add (this file is compiled with
// -ffp-contract=off).  sqrt and division are IEEE.  The OpenCL built-ins are
// given one fixed meaning here and in the CUDA kernels:
//   dot(a,b)       = (a.x*b.x + a.y*b.y) + a.z*b.z
//   cross(a,b)     = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x)
//   fast_length(a) = sqrt(dot(a,a))
//   convert_int(x) = truncation toward zero, saturating, NaN -> 0
//   max(0, x)      = fmax
// Compile-time constants are formed as src/Simulation.cpp:179-180 forms them:
// the double value printed with 6 significant digits, read back as float.
// The circle truncation, the 50-per-circle cap, self exclusion and the hash
// modulo are the reference's.  Two semantics are fixed where the reference is
// racy or silent: applyViscosity reads the pre-pass velocities of every
// neighbour (Jacobi; the reference updates in place while neighbours read,
// apply_viscosity.cl:46,81), and an optional box clamp is applied to the
// updated position in computeDelta before the delta is taken.  With the
// optional zero-distance guard a neighbour at distance exactly 0 is left out
// of the four solver sums (the reference divides 0 by 0 there).
//
// Templated on the scalar type: float is the parity oracle, double is the
// FP64 oracle used to state error bounds.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>
#include <omp.h>

#include "../include/pbf_params.h"
#include "noise_sin.hpp"

namespace {

template <typename T> struct V3 { T x, y, z; };
template <typename T> struct V4 { T x, y, z, w; };

template <typename T> inline V3<T> xyz(const V4<T>& a) { return {a.x, a.y, a.z}; }
template <typename T> inline V3<T> sub(const V3<T>& a, const V3<T>& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T> inline V3<T> add(const V3<T>& a, const V3<T>& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T> inline V3<T> scale(T s, const V3<T>& a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename T> inline T dot(const V3<T>& a, const V3<T>& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <typename T> inline V3<T> cross(const V3<T>& a, const V3<T>& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T> inline T fast_length(const V3<T>& a) { return std::sqrt(dot(a, a)); }

// convert_int with round-toward-zero; saturating and NaN -> 0 so that the
// result is defined for every input.
template <typename T> inline int convert_int_rtz(T v) {
    if (v != v) return 0;
    if (v >= (T)2147483647.0) return 2147483647;
    if (v <= (T)-2147483648.0) return (-2147483647 - 1);
    return (int)v;
}

// utilities.cl:69-77, in unsigned arithmetic (the same bits as the OpenCL
// int shifts, without C++'s signed-shift rules).
inline uint32_t expand_bits(int xi) {
    uint32_t x = (uint32_t)xi;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

// utilities.cl:79-87: Morton number of the cell, modulo the hash size.
inline uint32_t grid_hash(int cx, int cy, int cz, uint32_t grid) {
    int m = (int)(expand_bits(cx) | (expand_bits(cy) << 1) | (expand_bits(cz) << 2));
    return (uint32_t)(m % (int)grid);
}

// Simulation.cpp:179-180 streams the double value with std::showpoint and the
// default precision (6 significant digits) into a "-D...f" float literal.
float six_digit_literal(double v) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.6g", v);
    return std::strtof(buf, nullptr);
}

const uint32_t kEmpty = 0xFFFFFFFFu;          // END_OF_CELL_LIST (-1)
const uint32_t kPadKey = 2147483647u - 1u;     // radixsort.cl:17

template <typename T> struct Consts {
    T dt, h, h2, minR, hMinusMinR, poly6, gradSpiky, poly6q, rho0, eps, K, visc, vort;
    T gx, gy, gz, lo[3], hi[3];
    int clamp, guard;
    int complete;  // completeNeighbours: every circle in every pass, self in the density
    int circles, perCircle;
    uint32_t grid;
};

template <typename T> Consts<T> make_consts(const PbfParameters& p) {
    Consts<T> c;
    const double PI = 3.14159265358979323846;
    float poly6 = six_digit_literal(315.0f / (64.0f * PI * std::pow((double)p.h, 9.0)));
    float grad = six_digit_literal(45.0f / (PI * std::pow((double)p.h, 6.0)));
    // compute_delta.cl:81-82: q_2 = pow(dist*h, 2), poly6_q = pow(h_2 - q_2, 3),
    // taken in double and rounded once to float.
    float qh = p.surfaceTenstionDist * p.h;
    float q2 = (float)((double)qh * (double)qh);
    float d = p.h_2 - q2;
    float poly6q = (float)((double)d * (double)d * (double)d);
    float minR = 0.3f * p.h;  // build_friends_list.cl:32
    c.dt = p.timeStep; c.h = p.h; c.h2 = p.h_2; c.minR = minR; c.hMinusMinR = (T)(p.h - minR);
    c.poly6 = poly6; c.gradSpiky = grad; c.poly6q = poly6q;
    c.rho0 = p.restDensity; c.eps = p.epsilon; c.K = p.surfaceTenstionK;
    c.visc = p.viscosityFactor; c.vort = p.vorticityFactor;
    if (p.gravityVectorEnable) { c.gx = p.gravityX; c.gy = p.gravityY; c.gz = p.gravityZ; }
    else { c.gx = 0.0f; c.gy = -p.garvity; c.gz = 0.0f; }
    c.lo[0] = p.xMin; c.lo[1] = p.yMin; c.lo[2] = p.zMin;
    c.hi[0] = p.xMax; c.hi[1] = p.yMax; c.hi[2] = p.zMax;
    c.clamp = p.boxClamp;
    c.guard = p.zeroDistanceGuard;
    c.complete = p.completeNeighbours;
    c.circles = (int)p.friendsCircles; c.perCircle = (int)p.particlesPerCircle;
    c.grid = p.gridBufSize;
    return c;
}

inline uint32_t int_ceil(uint32_t n, uint32_t d) { return ((n + d - 1) / d) * d; }

// ---------------------------------------------------------------- sort --
// radixsort.cl:61-115 (histogram), :224-308 (scan + paste, restated as one
// exclusive scan over the [digit][group][item] layout), :165-218 (reorder),
// driven as Simulation.cpp:466-520: 6 passes of 5 bits over 2048 virtual
// processors, each owning a contiguous run of n/2048 keys.
void reference_radix_sort(std::vector<uint32_t>& keys, std::vector<uint32_t>& perm) {
    const int ITEMS = 128, GROUPS = 16, BITS = 5, TOTALBITS = 30, RADIX = 1 << BITS;
    const int PASSES = TOTALBITS / BITS, VP = ITEMS * GROUPS;
    const size_t n = keys.size();
    const size_t size = n / VP;
    std::vector<uint32_t> hist((size_t)RADIX * VP), outK(n), outP(n);
    for (int pass = 0; pass < PASSES; ++pass) {
        const int shift = pass * BITS;
        std::fill(hist.begin(), hist.end(), 0u);
        for (int vp = 0; vp < VP; ++vp)
            for (size_t i = vp * size; i < (vp + 1) * size; ++i)
                hist[(size_t)((keys[i] >> shift) & (RADIX - 1)) * VP + vp]++;
        uint32_t run = 0;
        for (size_t k = 0; k < hist.size(); ++k) { uint32_t v = hist[k]; hist[k] = run; run += v; }
        for (int vp = 0; vp < VP; ++vp)
            for (size_t i = vp * size; i < (vp + 1) * size; ++i) {
                uint32_t& pos = hist[(size_t)((keys[i] >> shift) & (RADIX - 1)) * VP + vp];
                outK[pos] = keys[i];
                outP[pos] = perm[i];
                ++pos;
            }
        keys.swap(outK);
        perm.swap(outP);
    }
}

// ------------------------------------------------------------ simulation --
template <typename T> struct State {
    int n = 0;
    uint32_t nKeys = 0;
    std::vector<V4<T>> pos, vel, pred, predP, omega;
    std::vector<T> density, lambda;
    std::vector<uint32_t> keys, perm, cells;
    // friends: [i][circle][slot] plus [i][circle] counts (the reference keeps
    // the same content as counts[circle][N] + idx[circle][slot][N],
    // build_friends_list.cl:1-21).
    std::vector<int32_t> friends;
    std::vector<int32_t> fcount;
};

template <typename T>
uint32_t cell_hash_of(const V4<T>& p, const Consts<T>& c, int& cx, int& cy, int& cz) {
    // radixsort.cl:11-13 / build_friends_list.cl:43
    cx = convert_int_rtz<T>(p.x / c.h);
    cy = convert_int_rtz<T>(p.y / c.h);
    cz = convert_int_rtz<T>(p.z / c.h);
    return grid_hash(cx, cy, cz, c.grid);
}

// predict_positions.cl:8-17
template <typename T> void predict(State<T>& s, const Consts<T>& c, bool paused) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s.n; ++i) {
        V4<T> v = s.vel[i];
        if (!paused) {
            v.x = v.x + c.dt * c.gx;
            v.y = v.y + c.dt * c.gy;
            v.z = v.z + c.dt * c.gz;
            s.vel[i] = v;
        }
        const V4<T>& p = s.pos[i];
        s.pred[i] = {p.x + c.dt * v.x, p.y + c.dt * v.y, p.z + c.dt * v.z, p.w + c.dt * v.w};
    }
}

// radixsort.cl:1-20 (computeKeys), the sort, then radixsort.cl:22-37
// (sortParticles: positions and predictions gathered by the permutation;
// velocities are not permuted, Simulation.cpp:523-535).
template <typename T> void sort_particles(State<T>& s, const Consts<T>& c) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < (int)s.nKeys; ++i) {
        if (i < s.n) { int x, y, z; s.keys[i] = cell_hash_of(s.pred[i], c, x, y, z); }
        else s.keys[i] = kPadKey;
        s.perm[i] = (uint32_t)i;
    }
    reference_radix_sort(s.keys, s.perm);
    std::vector<V4<T>> pos2(s.n), pred2(s.n);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s.n; ++i) { pos2[i] = s.pos[s.perm[i]]; pred2[i] = s.pred[s.perm[i]]; }
    s.pos.swap(pos2);
    s.pred.swap(pred2);
}

// update_cells.cl:6-25 (applied to a table that holds END_OF_CELL_LIST).
template <typename T> void update_cells(State<T>& s) {
    const int N = s.n;
    for (int i = 0; i < N; ++i) {
        uint32_t k = s.keys[i];
        if (i > 0) {
            uint32_t kp = s.keys[i - 1];
            if (kp != k) { s.cells[2 * (size_t)k] = (uint32_t)i; s.cells[2 * (size_t)kp + 1] = (uint32_t)(i - 1); }
            if (i == N - 1) s.cells[2 * (size_t)k + 1] = (uint32_t)i;
        } else {
            s.cells[2 * (size_t)k] = (uint32_t)i;
        }
    }
}

// reset_grid.cl:6-14
template <typename T> void reset_grid(State<T>& s) {
    for (int i = 0; i < s.n; ++i) { s.cells[2 * (size_t)s.keys[i]] = kEmpty; s.cells[2 * (size_t)s.keys[i] + 1] = kEmpty; }
}

// build_friends_list.cl:29-102
template <typename T> void build_friends(State<T>& s, const Consts<T>& c) {
    const int C = c.circles, P = c.perCircle, N = s.n;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < N; ++i) {
        int32_t* cnt = &s.fcount[(size_t)i * C];
        int32_t* lst = &s.friends[(size_t)i * C * P];
        for (int k = 0; k < C; ++k) cnt[k] = 0;
        V3<T> pi = xyz(s.pred[i]);
        int cx, cy, cz;
        cell_hash_of(s.pred[i], c, cx, cy, cz);
        for (int x = -1; x <= 1; ++x)
            for (int y = -1; y <= 1; ++y)
                for (int z = -1; z <= 1; ++z) {
                    uint32_t hsh = grid_hash(cx + x, cy + y, cz + z, c.grid);
                    uint32_t start = s.cells[2 * (size_t)hsh], end = s.cells[2 * (size_t)hsh + 1];
                    if (start == kEmpty) continue;
                    // The reference loops to `end` unbounded; with one particle
                    // the end stays END_OF_CELL_LIST.  Bounded here by N-1.
                    uint32_t last = std::min<uint32_t>(end, (uint32_t)(N - 1));
                    for (uint32_t j = start; j <= last; ++j) {
                        if ((int)j == i) continue;
                        V3<T> r = sub(pi, xyz(s.pred[j]));
                        T r2 = dot(r, r);
                        if (r2 >= c.h2) continue;
                        T adj = std::fmax((T)0, (std::sqrt(r2) - c.minR) / c.hMinusMinR);
                        int circ = std::min(convert_int_rtz<T>(adj * adj * adj * (T)C), C - 1);
                        if (cnt[circ] >= P) continue;
                        lst[circ * P + cnt[circ]++] = (int32_t)j;
                    }
                }
    }
}

// Circles kept by a pass with the given threshold (compute_scaling.cl:47-54
// with 0.6f, compute_delta.cl:97-104 and the XSPH / vorticity kernels with
// 0.5f).  Returns the number of leading circles processed.
inline int circles_kept(const int32_t* cnt, int C, float threshold) {
    int total = 0;
    for (int k = 0; k < C; ++k) total += cnt[k];
    int processed = 0, kept = 0;
    for (int k = 0; k < C; ++k) {
        if (((float)processed) / total > threshold) continue;
        processed += cnt[k];
        kept = k + 1;
    }
    return kept;
}

// compute_scaling.cl:27-112, then pack_data.cl (pred.w = lambda).
template <typename T> void compute_scaling(State<T>& s, const Consts<T>& c) {
    const int C = c.circles, P = c.perCircle;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s.n; ++i) {
        const int32_t* cnt = &s.fcount[(size_t)i * C];
        const int32_t* lst = &s.friends[(size_t)i * C * P];
        V3<T> pi = xyz(s.pred[i]);
        // complete neighbour sets count the particle itself first: d = h^2 - 0
        T density_sum = c.complete ? c.h2 * c.h2 * c.h2 : (T)0, grad_sum_k = 0;
        V3<T> grad_sum_k_i = {0, 0, 0};
        int kept = (c.complete ? C : circles_kept(cnt, C, 0.6f));
        for (int k = 0; k < kept; ++k)
            for (int f = 0; f < cnt[k]; ++f) {
                V3<T> r = sub(pi, xyz(s.pred[lst[k * P + f]]));
                T r2 = dot(r, r);
                if (r2 < c.h2 && (!c.guard || r2 > (T)0)) {
                    T rl = std::sqrt(r2);
                    T hr = c.h - rl;
                    T sc = c.gradSpiky * hr * hr;
                    V3<T> g = {(sc * r.x) / rl, (sc * r.y) / rl, (sc * r.z) / rl};
                    T d = c.h2 - r2;
                    density_sum += d * d * d;
                    grad_sum_k += dot(g, g);
                    grad_sum_k_i = add(grad_sum_k_i, g);
                }
            }
        density_sum *= c.poly6;
        s.density[i] = density_sum;
        grad_sum_k += dot(grad_sum_k_i, grad_sum_k_i);
        T constraint = (density_sum / c.rho0) - (T)1;
        s.lambda[i] = (T)-1 * constraint / (grad_sum_k / (c.rho0 * c.rho0) + c.eps);
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s.n; ++i) { V4<T> p = s.pred[i]; p.w = s.lambda[i]; s.predP[i] = p; }
}

// ---- force planes (compute_delta.cl:1-42, 157-182), as data ----
static std::vector<PbfForceQuad> g_quads;
static std::vector<uint32_t> g_fmask;
static int g_fmaskW = 0, g_fmaskH = 0;
static float g_wave = 0.0f;  // the wave generator's moving wall: xMin + g_wave

template <typename T> T noise_sin(T x) { return (T)std::sin(x); }
template <> float noise_sin<float>(float x) { return noise_sinf_ref(x); }

// compute_delta.cl:157-161: 1.0 (a double literal) + (3 + sin + sin + sin) h 0.03f.
template <typename T> T plane_edge_offset(const Consts<T>& c, V3<T> f) {
    const T nx = f.x * (T)5 / c.h, ny = f.y * (T)5 / c.h, nz = f.z * (T)5 / c.h;
    const T x = (T)3 + noise_sin(nx) + noise_sin(ny) + noise_sin(nz);
    return (T)(1.0 + (double)(x * c.h * (T)0.03f));
}

// BouncePointQuad (compute_delta.cl:1-42).
template <typename T> V3<T> bounce_point_quad(V3<T> prev, V3<T> next, const PbfForceQuad& q, T edge) {
    const V3<T> B = {(T)q.B[0], (T)q.B[1], (T)q.B[2]}, E0 = {(T)q.E0[0], (T)q.E0[1], (T)q.E0[2]},
                E1 = {(T)q.E1[0], (T)q.E1[1], (T)q.E1[2]};
    const T a = dot(E0, E0), b = dot(E0, E1), c = dot(E1, E1);
    const T invdet = (T)(1.0 / (double)(a * c - b * b));
    const V3<T> cr = {E0.y * E1.z - E0.z * E1.y, E0.z * E1.x - E0.x * E1.z, E0.x * E1.y - E0.y * E1.x};
    const T cl = std::sqrt(dot(cr, cr));
    const V3<T> n = {cr.x / cl, cr.y / cl, cr.z / cl};
    const V3<T> ro = {n.x * edge, n.y * edge, n.z * edge};
    const V3<T> D = {B.x - next.x, B.y - next.y, B.z - next.z};
    const T e = dot(E1, D), d = dot(E0, D);
    const T s = invdet * (b * e - c * d), t = invdet * (b * d - a * e);
    if ((s < 0) || (s > 1) || (t < 0) || (t > 1)) return next;
    const V3<T> pp = {((B.x + E0.x * s) + E1.x * t) + ro.x, ((B.y + E0.y * s) + E1.y * t) + ro.y,
                      ((B.z + E0.z * s) + E1.z * t) + ro.z};
    const V3<T> dP = {next.x - pp.x, next.y - pp.y, next.z - pp.z};
    if (dot(n, dP) > 0) return next;
    const T nv = dot(n, V3<T>{prev.x - next.x, prev.y - next.y, prev.z - next.z});
    if (std::sqrt(dot(dP, dP)) > edge + nv) return next;
    if (g_fmask.empty()) return next;
    // (int2)(t * 512.0, maskYOffset + s * maskHeight), clamped to the edge
    int tx = (int)((double)t * 512.0);
    int sy = (int)((T)q.maskYOffset + s * (T)q.maskHeight);
    tx = std::min(std::max(tx, 0), g_fmaskW - 1);
    sy = std::min(std::max(sy, 0), g_fmaskH - 1);
    if (g_fmask[(size_t)sy * g_fmaskW + tx] == 0u) return next;
    return pp;
}

// compute_delta.cl:54-185 (with the force planes of oracle_set_force_planes), then
// update_predicted.cl (pred += delta).  The clamp, when enabled, bounds
// `future` to the box before the delta is formed.
// `mask` (may be NULL): per particle, which coordinates the clamp moved, two
// bits per axis (1: to the lower bound, 2: to the upper bound).
template <typename T> void compute_delta(State<T>& s, const Consts<T>& c, uint8_t* mask = nullptr) {
    const int C = c.circles, P = c.perCircle;
    const T negG = -c.gradSpiky;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s.n; ++i) {
        const int32_t* cnt = &s.fcount[(size_t)i * C];
        const int32_t* lst = &s.friends[(size_t)i * C * P];
        V4<T> pi = s.predP[i];
        V3<T> sum = {0, 0, 0};
        int kept = (c.complete ? C : circles_kept(cnt, C, 0.5f));
        for (int k = 0; k < kept; ++k)
            for (int f = 0; f < cnt[k]; ++f) {
                V4<T> pj = s.predP[lst[k * P + f]];
                V3<T> r = {pi.x - pj.x, pi.y - pj.y, pi.z - pj.z};
                T r2 = dot(r, r);
                if (r2 < c.h2 && (!c.guard || r2 > (T)0)) {
                    T rl = std::sqrt(r2);
                    T hr = c.h - rl;
                    V3<T> g = {(r.x / rl) * hr * hr, (r.y / rl) * hr * hr, (r.z / rl) * hr * hr};
                    T d = c.h2 - r2;
                    T p6 = d * d * d;
                    T rq = p6 / c.poly6q;
                    T scorr = c.K * rq * rq * rq * rq;
                    T a = pi.w + pj.w + scorr;
                    sum = add(sum, scale(a, g));
                }
            }
        V3<T> dp = {(negG * sum.x) / c.rho0, (negG * sum.y) / c.rho0, (negG * sum.z) / c.rho0};
        V3<T> fut = {pi.x + dp.x, pi.y + dp.y, pi.z + dp.z};
        if (!g_quads.empty()) {
            const V3<T> prev = {s.pos[i].x, s.pos[i].y, s.pos[i].z};
            const T edge = plane_edge_offset(c, fut);
            for (const PbfForceQuad& q : g_quads) fut = bounce_point_quad(prev, fut, q, edge);
        }
        if (c.clamp) {  // comparisons, so that -0.0 and NaN pass through unchanged
            T lo[3] = {c.lo[0], c.lo[1], c.lo[2]};
            if (g_wave != 0.0f) lo[0] = (T)((float)c.lo[0] + g_wave);
            if (mask) {
                T* f = &fut.x;
                uint8_t m = 0;
                for (int k = 0; k < 3; ++k) m |= (uint8_t)((f[k] < lo[k] ? 1 : (f[k] > c.hi[k] ? 2 : 0)) << (2 * k));
                mask[i] = m;
            }
            fut.x = fut.x < lo[0] ? lo[0] : (fut.x > c.hi[0] ? c.hi[0] : fut.x);
            fut.y = fut.y < lo[1] ? lo[1] : (fut.y > c.hi[1] ? c.hi[1] : fut.y);
            fut.z = fut.z < lo[2] ? lo[2] : (fut.z > c.hi[2] ? c.hi[2] : fut.z);
        } else if (mask) {
            mask[i] = 0;
        }
        V3<T> delta = {fut.x - pi.x, fut.y - pi.y, fut.z - pi.z};
        s.pred[i] = {pi.x + delta.x, pi.y + delta.y, pi.z + delta.z, pi.w + (T)0};
    }
}

// update_velocities.cl:11-14 (after pack_data with the density).
template <typename T> void update_velocities(State<T>& s, const Consts<T>& c) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s.n; ++i) {
        V4<T>& p = s.pred[i];
        p.w = s.density[i];
        V4<T>& v = s.vel[i];
        v.x = (p.x - s.pos[i].x) / c.dt;
        v.y = (p.y - s.pos[i].y) / c.dt;
        v.z = (p.z - s.pos[i].z) / c.dt;
        s.pos[i] = {p.x, p.y, p.z, fast_length(V3<T>{v.x, v.y, v.z})};
    }
}

// apply_viscosity.cl:12-86, reading the pre-pass velocities (Jacobi).
template <typename T> void apply_viscosity(State<T>& s, const Consts<T>& c) {
    const int C = c.circles, P = c.perCircle;
    const T negG = -c.gradSpiky;
    std::vector<V4<T>> vold(s.vel);
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s.n; ++i) {
        const int32_t* cnt = &s.fcount[(size_t)i * C];
        const int32_t* lst = &s.friends[(size_t)i * C * P];
        V4<T> pi = s.pred[i], vi = vold[i];
        V3<T> vs = {0, 0, 0}, om = {0, 0, 0};
        int kept = (c.complete ? C : circles_kept(cnt, C, 0.5f));
        for (int k = 0; k < kept; ++k)
            for (int f = 0; f < cnt[k]; ++f) {
                int j = lst[k * P + f];
                V4<T> pj = s.pred[j], vj = vold[j];
                V3<T> r = {pi.x - pj.x, pi.y - pj.y, pi.z - pj.z};
                T r2 = r.x * r.x + r.y * r.y + r.z * r.z;
                if (r2 < c.h2 && (!c.guard || r2 > (T)0)) {
                    if (std::fabs(pj.w) > (T)1e-8f) {
                        V3<T> v = {vj.x - vi.x, vj.y - vi.y, vj.z - vi.z};
                        T d = c.h2 - r2;
                        T rl = std::sqrt(r2);
                        T hr = c.h - rl;
                        V3<T> g = {(r.x / rl) * hr * hr, (r.y / rl) * hr * hr, (r.z / rl) * hr * hr};
                        om = add(om, cross(v, g));
                        T d3 = d * d * d;
                        vs = add(vs, V3<T>{v.x * d3, v.y * d3, v.z * d3});
                    }
                }
            }
        vs = {vs.x * c.poly6, vs.y * c.poly6, vs.z * c.poly6};
        s.vel[i] = {vi.x + c.visc * vs.x, vi.y + c.visc * vs.y, vi.z + c.visc * vs.z, vi.w + c.visc * (T)0};
        s.omega[i] = {om.x * negG, om.y * negG, om.z * negG, (T)0};
    }
}

// apply_vorticity.cl:12-86
template <typename T> void apply_vorticity(State<T>& s, const Consts<T>& c) {
    const int C = c.circles, P = c.perCircle;
    const T negG = -c.gradSpiky;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s.n; ++i) {
        const int32_t* cnt = &s.fcount[(size_t)i * C];
        const int32_t* lst = &s.friends[(size_t)i * C * P];
        V4<T> pi = s.pred[i];
        V3<T> eta = {0, 0, 0};
        int kept = (c.complete ? C : circles_kept(cnt, C, 0.5f));
        for (int k = 0; k < kept; ++k)
            for (int f = 0; f < cnt[k]; ++f) {
                int j = lst[k * P + f];
                V4<T> pj = s.pred[j];
                V3<T> r = {pi.x - pj.x, pi.y - pj.y, pi.z - pj.z};
                T r2 = r.x * r.x + r.y * r.y + r.z * r.z;
                if (r2 < c.h2 && (!c.guard || r2 > (T)0)) {
                    if (std::fabs(pj.w) > (T)1e-8f) {
                        T rl = std::sqrt(r2);
                        T hr = c.h - rl;
                        V3<T> g = {(r.x / rl) * hr * hr, (r.y / rl) * hr * hr, (r.z / rl) * hr * hr};
                        T ol = fast_length(xyz(s.omega[j]));
                        eta = add(eta, scale(ol, g));
                    }
                }
            }
        eta = {eta.x * negG, eta.y * negG, eta.z * negG};
        T l = fast_length(eta);
        if (l > 0) eta = {eta.x / l, eta.y / l, eta.z / l};
        V3<T> cr = cross(eta, xyz(s.omega[i]));
        V3<T> force = scale(c.vort, cr);
        V3<T> vv = {force.x * c.dt, force.y * c.dt, force.z * c.dt};
        V4<T>& v = s.vel[i];
        v = {v.x + vv.x, v.y + vv.y, v.z + vv.z, v.w + (T)0};
    }
}

}  // namespace

// Optional outputs of the last substep (any pointer may be NULL).
typedef struct OracleDebug {
    uint32_t* keys;      // IntCeil(N, 2048) sorted keys
    uint32_t* perm;      // IntCeil(N, 2048) permutation
    uint32_t* cells;     // 2 * gridBufSize, after updateCells (before reset)
    uint32_t* counts;    // 2 * N: entries used by scaling / by delta, XSPH, vorticity
    uint32_t* list;      // list_slots * N, slot-major, circle-major order
    int       list_slots;
    float*    density;   // N (last iteration)
    float*    lambda;    // N (last iteration)
    float*    omega;     // 4 * N
} OracleDebug;

namespace {

int check(const PbfParameters* p, int n) {
    if (!p || n <= 0) return -1;
    if (p->friendsCircles < 1 || p->friendsCircles > PBF_MAX_CIRCLES) return -1;
    if (p->particlesPerCircle < 1 || p->particlesPerCircle > PBF_MAX_PER_CIRCLE) return -1;
    if (p->gridBufSize < 1 || p->gridBufSize > (1u << 30)) return -1;
    if (!(p->h > 0) || !(p->timeStep > 0)) return -1;
    return 0;
}

template <typename T>
int run_steps(const PbfParameters* p, int n, T* pos, T* vel, T* pred, int substeps,
                     int paused, uint32_t* keys_state, int nthreads, OracleDebug* dbg) {
    if (check(p, n) || substeps < 0) return -1;
    if (nthreads > 0) omp_set_num_threads(nthreads);
    Consts<T> c = make_consts<T>(*p);
    State<T> s;
    s.n = n;
    s.nKeys = int_ceil((uint32_t)n, 2048u);
    s.pos.resize(n); s.vel.resize(n); s.pred.resize(n); s.predP.resize(n); s.omega.resize(n);
    std::memcpy(s.pos.data(), pos, sizeof(T) * 4 * n);
    std::memcpy(s.vel.data(), vel, sizeof(T) * 4 * n);
    s.density.assign(n, 0); s.lambda.assign(n, 0);
    s.keys.assign(s.nKeys, 0); s.perm.assign(s.nKeys, 0);
    if (keys_state) std::memcpy(s.keys.data(), keys_state, 4 * s.nKeys);
    s.cells.assign(2 * (size_t)p->gridBufSize, kEmpty);
    s.friends.assign((size_t)n * c.circles * c.perCircle, 0);
    s.fcount.assign((size_t)n * c.circles, 0);
    for (int step = 0; step < substeps; ++step) {
        const bool last = step == substeps - 1;
        predict(s, c, paused != 0);
        if (!paused) sort_particles(s, c);
        update_cells(s);
        if (last && dbg && dbg->cells) std::memcpy(dbg->cells, s.cells.data(), 8 * (size_t)p->gridBufSize);
        if (last && dbg && dbg->keys) std::memcpy(dbg->keys, s.keys.data(), 4 * (size_t)s.nKeys);
        if (last && dbg && dbg->perm) std::memcpy(dbg->perm, s.perm.data(), 4 * (size_t)s.nKeys);
        build_friends(s, c);
        reset_grid(s);
        for (unsigned it = 0; it < p->simIterations; ++it) {
            compute_scaling(s, c);
            compute_delta(s, c);
        }
        update_velocities(s, c);
        apply_viscosity(s, c);
        apply_vorticity(s, c);
    }
    std::memcpy(pos, s.pos.data(), sizeof(T) * 4 * n);
    std::memcpy(vel, s.vel.data(), sizeof(T) * 4 * n);
    if (pred) std::memcpy(pred, s.pred.data(), sizeof(T) * 4 * n);
    if (keys_state) std::memcpy(keys_state, s.keys.data(), 4 * s.nKeys);
    if (dbg && substeps > 0) {
        const int C = c.circles, P = c.perCircle;
        for (int i = 0; i < n; ++i) {
            const int32_t* cnt = &s.fcount[(size_t)i * C];
            const int32_t* lst = &s.friends[(size_t)i * C * P];
            int kl = (c.complete ? C : circles_kept(cnt, C, 0.6f)), kd = (c.complete ? C : circles_kept(cnt, C, 0.5f));
            uint32_t nl = 0, nd = 0, slot = 0;
            for (int k = 0; k < C; ++k) {
                if (k < kl) nl += cnt[k];
                if (k < kd) nd += cnt[k];
            }
            if (dbg->counts) { dbg->counts[2 * i] = nl; dbg->counts[2 * i + 1] = nd; }
            if (dbg->list)
                for (int k = 0; k < kl; ++k)
                    for (int f = 0; f < cnt[k]; ++f, ++slot)
                        if ((int)slot < dbg->list_slots) dbg->list[(size_t)slot * n + i] = (uint32_t)lst[k * P + f];
            if (dbg->density) dbg->density[i] = (float)s.density[i];
            if (dbg->lambda) dbg->lambda[i] = (float)s.lambda[i];
            if (dbg->omega)
                for (int q = 0; q < 4; ++q) dbg->omega[4 * i + q] = (float)(&s.omega[i].x)[q];
        }
    }
    return 0;
}


// ============================================================ rollouts ==
// Gradients of a rollout over a fixed neighbour structure.  An FP32 forward
// (identical to the pipeline above) records, per substep, the sort
// permutation, the friend lists and which coordinates the box clamp moved.
// The same function with that structure frozen is then evaluated in FP64
// ("replay"), and its exact gradient is taken by reverse accumulation through
// the substeps.  The replay is smooth in the inputs: the support test
// r^2 < h^2 switches terms that vanish with their first derivative at r = h.

struct Structure {
    std::vector<uint32_t> perm;    // sorted index k came from index perm[k]
    std::vector<int32_t> counts;   // N x C friends per circle
    std::vector<int32_t> start;    // N + 1 offsets into list
    std::vector<int32_t> list;     // the kept-for-density circles, circle-major
    std::vector<uint8_t> mask;     // iterations x N clamp masks
};

struct RolloutRecord {
    PbfParameters params;
    int n = 0;
    std::vector<Structure> steps;
};

template <typename T> struct Tape {
    std::vector<V4<T>> xs;               // sorted positions before the update
    std::vector<std::vector<V4<T>>> q;   // (p^t, lambda^t), t < iterations
    std::vector<V4<T>> pI;               // final predictions, w = density of the last pass
    std::vector<V4<T>> v2, omega;        // velocities before XSPH, vorticity
};

// The reference's truncation (rollouts use the reference's neighbour sets).
inline void kept_circles(const int32_t* cnt, int C, int& keptL, int& keptD) {
    keptL = circles_kept(cnt, C, 0.6f);
    keptD = circles_kept(cnt, C, 0.5f);
}

// Friends of i used by a pass keeping `kept` circles: list[start[i] .. +m).
inline int kept_count(const int32_t* cnt, int kept) {
    int m = 0;
    for (int k = 0; k < kept; ++k) m += cnt[k];
    return m;
}

// k(r) = (h - |r|)^2 r / |r| and the adjoint of its argument.
template <typename T> inline V3<T> kvec(const V3<T>& r, T rl, T h) {
    T hr = h - rl;
    return {r.x / rl * hr * hr, r.y / rl * hr * hr, r.z / rl * hr * hr};
}
template <typename T> inline V3<T> kvec_adj(const V3<T>& r, T rl, T h, const V3<T>& kb) {
    T f = (h - rl) * (h - rl) / rl;
    T fp = -(h - rl) * (h + rl) / (rl * rl);
    T s = fp * dot(kb, r) / rl;
    return {f * kb.x + s * r.x, f * kb.y + s * r.y, f * kb.z + s * r.z};
}

template <typename T> inline bool support(const Consts<T>& c, T r2) { return r2 < c.h2 && (!c.guard || r2 > (T)0); }

template <typename T> void atomic_add3(V4<T>& a, const V3<T>& v) {
#pragma omp atomic
    a.x += v.x;
#pragma omp atomic
    a.y += v.y;
#pragma omp atomic
    a.z += v.z;
}

// One substep of the frozen-structure function in T.  x, v: in/out (state in
// the order of the previous substep on entry, sorted order on exit); ids
// follows the permutation.  With a tape, the intermediate values are kept.
template <typename T>
void replay_substep(const Structure& st, const Consts<T>& c, int iters, std::vector<V4<T>>& x, std::vector<V4<T>>& v,
                    std::vector<uint32_t>& ids, Tape<T>* tape) {
    const int N = (int)x.size(), C = c.circles;
    std::vector<V4<T>> p0(N), xs(N), p(N);
    std::vector<uint32_t> ids2(N);
    for (int i = 0; i < N; ++i) {
        V4<T> v1 = {v[i].x + c.dt * c.gx, v[i].y + c.dt * c.gy, v[i].z + c.dt * c.gz, 0};
        p0[i] = {x[i].x + c.dt * v1.x, x[i].y + c.dt * v1.y, x[i].z + c.dt * v1.z, 0};
    }
    for (int k = 0; k < N; ++k) { xs[k] = x[st.perm[k]]; p[k] = p0[st.perm[k]]; ids2[k] = ids[st.perm[k]]; }
    ids.swap(ids2);
    std::vector<T> lam(N), rho(N);
    if (tape) { tape->xs = xs; tape->q.assign(iters, {}); }
    const T negG = -c.gradSpiky;
    for (int t = 0; t < iters; ++t) {
#pragma omp parallel for schedule(dynamic, 64)
        for (int i = 0; i < N; ++i) {
            const int32_t* cnt = &st.counts[(size_t)i * C];
            int kl, kd;
            kept_circles(cnt, C, kl, kd);
            const int m = kept_count(cnt, kl);
            T ds = 0, gsk = 0;
            V3<T> S = {0, 0, 0};
            for (int f = 0; f < m; ++f) {
                const int j = st.list[st.start[i] + f];
                V3<T> r = sub(xyz(p[i]), xyz(p[j]));
                T r2 = dot(r, r);
                if (!support(c, r2)) continue;
                T rl = std::sqrt(r2);
                V3<T> g = scale(c.gradSpiky, kvec(r, rl, c.h));
                T d = c.h2 - r2;
                ds += d * d * d;
                gsk += dot(g, g);
                S = add(S, g);
            }
            rho[i] = ds * c.poly6;
            T D = gsk + dot(S, S);
            lam[i] = -(rho[i] / c.rho0 - 1) / (D / (c.rho0 * c.rho0) + c.eps);
        }
        if (tape) {
            tape->q[t].resize(N);
            for (int i = 0; i < N; ++i) tape->q[t][i] = {p[i].x, p[i].y, p[i].z, lam[i]};
        }
        std::vector<V4<T>> pn(N);
#pragma omp parallel for schedule(dynamic, 64)
        for (int i = 0; i < N; ++i) {
            const int32_t* cnt = &st.counts[(size_t)i * C];
            int kl, kd;
            kept_circles(cnt, C, kl, kd);
            const int m = kept_count(cnt, kd);
            V3<T> sum = {0, 0, 0};
            for (int f = 0; f < m; ++f) {
                const int j = st.list[st.start[i] + f];
                V3<T> r = sub(xyz(p[i]), xyz(p[j]));
                T r2 = dot(r, r);
                if (!support(c, r2)) continue;
                T rl = std::sqrt(r2);
                T W = (c.h2 - r2) * (c.h2 - r2) * (c.h2 - r2);
                T rq = W / c.poly6q;
                T a = lam[i] + lam[j] + c.K * rq * rq * rq * rq;
                sum = add(sum, scale(a, kvec(r, rl, c.h)));
            }
            V3<T> fut = {p[i].x + negG * sum.x / c.rho0, p[i].y + negG * sum.y / c.rho0, p[i].z + negG * sum.z / c.rho0};
            const uint8_t mk = st.mask[(size_t)t * N + i];
            T* f = &fut.x;
            for (int k = 0; k < 3; ++k) {
                const int b = (mk >> (2 * k)) & 3;
                if (b == 1) f[k] = c.lo[k];
                else if (b == 2) f[k] = c.hi[k];
            }
            pn[i] = {fut.x, fut.y, fut.z, 0};
        }
        p.swap(pn);
    }
    std::vector<V4<T>> v2(N), v3(N), om(N);
    for (int i = 0; i < N; ++i) {
        v2[i] = {(p[i].x - xs[i].x) / c.dt, (p[i].y - xs[i].y) / c.dt, (p[i].z - xs[i].z) / c.dt, 0};
        p[i].w = iters > 0 ? rho[i] : 0;
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < N; ++i) {
        const int32_t* cnt = &st.counts[(size_t)i * C];
        int kl, kd;
        kept_circles(cnt, C, kl, kd);
        const int m = kept_count(cnt, kd);
        V3<T> vs = {0, 0, 0}, o = {0, 0, 0};
        for (int f = 0; f < m; ++f) {
            const int j = st.list[st.start[i] + f];
            V3<T> r = sub(xyz(p[i]), xyz(p[j]));
            T r2 = dot(r, r);
            if (!support(c, r2) || !(std::fabs(p[j].w) > (T)1e-8f)) continue;
            T rl = std::sqrt(r2);
            V3<T> u = sub(xyz(v2[j]), xyz(v2[i]));
            T d = c.h2 - r2;
            vs = add(vs, scale(d * d * d, u));
            o = add(o, cross(u, kvec(r, rl, c.h)));
        }
        v3[i] = {v2[i].x + c.visc * c.poly6 * vs.x, v2[i].y + c.visc * c.poly6 * vs.y, v2[i].z + c.visc * c.poly6 * vs.z, 0};
        om[i] = {negG * o.x, negG * o.y, negG * o.z, 0};
    }
    std::vector<V4<T>> v4(N);
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < N; ++i) {
        const int32_t* cnt = &st.counts[(size_t)i * C];
        int kl, kd;
        kept_circles(cnt, C, kl, kd);
        const int m = kept_count(cnt, kd);
        V3<T> eta = {0, 0, 0};
        for (int f = 0; f < m; ++f) {
            const int j = st.list[st.start[i] + f];
            V3<T> r = sub(xyz(p[i]), xyz(p[j]));
            T r2 = dot(r, r);
            if (!support(c, r2) || !(std::fabs(p[j].w) > (T)1e-8f)) continue;
            T rl = std::sqrt(r2);
            eta = add(eta, scale(fast_length(xyz(om[j])), kvec(r, rl, c.h)));
        }
        eta = scale(negG, eta);
        T l = fast_length(eta);
        V3<T> Nn = l > 0 ? scale((T)1 / l, eta) : V3<T>{0, 0, 0};
        V3<T> fv = scale(c.vort * c.dt, cross(Nn, xyz(om[i])));
        v4[i] = {v3[i].x + fv.x, v3[i].y + fv.y, v3[i].z + fv.z, 0};
    }
    if (tape) { tape->pI = p; tape->v2 = v2; tape->omega = om; }
    x = p;
    for (auto& q : x) q.w = 0;
    v = v4;
}

// Reverse accumulation through one substep of the frozen-structure function.
// xb, vb: adjoints of the substep's output (sorted order) on entry, of its
// input (previous order) on exit.  cb, gb accumulate dL/d visc and dL/d g.
template <typename T>
void adjoint_substep(const Structure& st, const Consts<T>& c, int iters, const Tape<T>& tp, std::vector<V4<T>>& xb,
                     std::vector<V4<T>>& vb, T& cb, T gb[3]) {
    const int N = (int)xb.size(), C = c.circles;
    const T negG = -c.gradSpiky, G = c.gradSpiky;
    const std::vector<V4<T>>& p = tp.pI;
    std::vector<V4<T>> pb(N, V4<T>{0, 0, 0, 0}), omb(N, V4<T>{0, 0, 0, 0}), v2b(N, V4<T>{0, 0, 0, 0});
    // vorticity: v4 = v3 + dt*vort*(N x omega_i), N = eta/|eta|, eta = -G sum |om_j| k_ij
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < N; ++i) {
        const int32_t* cnt = &st.counts[(size_t)i * C];
        int kl, kd;
        kept_circles(cnt, C, kl, kd);
        const int m = kept_count(cnt, kd);
        V3<T> eta = {0, 0, 0};
        for (int f = 0; f < m; ++f) {
            const int j = st.list[st.start[i] + f];
            V3<T> r = sub(xyz(p[i]), xyz(p[j]));
            T r2 = dot(r, r);
            if (!support(c, r2) || !(std::fabs(p[j].w) > (T)1e-8f)) continue;
            eta = add(eta, scale(fast_length(xyz(tp.omega[j])), kvec(r, std::sqrt(r2), c.h)));
        }
        eta = scale(negG, eta);
        T l = fast_length(eta);
        if (!(l > 0)) continue;
        V3<T> Nn = scale((T)1 / l, eta);
        V3<T> ub = scale(c.vort * c.dt, xyz(vb[i]));
        V3<T> oi = xyz(tp.omega[i]);
        V3<T> Nb = cross(oi, ub);
        atomic_add3(omb[i], cross(ub, Nn));
        V3<T> etab = scale((T)1 / l, sub(Nb, scale(dot(Nn, Nb), Nn)));
        for (int f = 0; f < m; ++f) {
            const int j = st.list[st.start[i] + f];
            V3<T> r = sub(xyz(p[i]), xyz(p[j]));
            T r2 = dot(r, r);
            if (!support(c, r2) || !(std::fabs(p[j].w) > (T)1e-8f)) continue;
            T rl = std::sqrt(r2);
            V3<T> k = kvec(r, rl, c.h);
            V3<T> oj = xyz(tp.omega[j]);
            T ol = fast_length(oj);
            if (ol > 0) atomic_add3(omb[j], scale(negG * dot(etab, k) / ol, oj));
            V3<T> rb = kvec_adj(r, rl, c.h, scale(negG * ol, etab));
            atomic_add3(pb[i], rb);
            atomic_add3(pb[j], scale((T)-1, rb));
        }
    }
    // XSPH + omega: v3 = v2 + visc*POLY6*sum (v2_j - v2_i) W_ij; omega = -G sum (v2_j - v2_i) x k_ij
    T cacc = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : cacc)
    for (int i = 0; i < N; ++i) {
        const int32_t* cnt = &st.counts[(size_t)i * C];
        int kl, kd;
        kept_circles(cnt, C, kl, kd);
        const int m = kept_count(cnt, kd);
        V3<T> v3b = xyz(vb[i]), ob = xyz(omb[i]);
        atomic_add3(v2b[i], v3b);
        for (int f = 0; f < m; ++f) {
            const int j = st.list[st.start[i] + f];
            V3<T> r = sub(xyz(p[i]), xyz(p[j]));
            T r2 = dot(r, r);
            if (!support(c, r2) || !(std::fabs(p[j].w) > (T)1e-8f)) continue;
            T rl = std::sqrt(r2);
            V3<T> u = sub(xyz(tp.v2[j]), xyz(tp.v2[i]));
            T d = c.h2 - r2;
            T w = c.poly6 * d * d * d;
            V3<T> k = kvec(r, rl, c.h);
            cacc += w * dot(v3b, u);
            V3<T> ub = add(scale(c.visc * w, v3b), scale(negG, cross(k, ob)));
            atomic_add3(v2b[j], ub);
            atomic_add3(v2b[i], scale((T)-1, ub));
            T Wb = c.visc * c.poly6 * dot(v3b, u);
            V3<T> rb = scale(Wb * (T)-6 * d * d, r);
            rb = add(rb, kvec_adj(r, rl, c.h, scale(negG, cross(ob, u))));
            atomic_add3(pb[i], rb);
            atomic_add3(pb[j], scale((T)-1, rb));
        }
    }
    cb += cacc;
    // velocities: v2 = (p^I - xs)/dt, x' = p^I
    std::vector<V4<T>> xsb(N);
    for (int i = 0; i < N; ++i) {
        pb[i] = {pb[i].x + xb[i].x + v2b[i].x / c.dt, pb[i].y + xb[i].y + v2b[i].y / c.dt,
                 pb[i].z + xb[i].z + v2b[i].z / c.dt, 0};
        xsb[i] = {-v2b[i].x / c.dt, -v2b[i].y / c.dt, -v2b[i].z / c.dt, 0};
    }
    // solver iterations, last first
    for (int t = iters - 1; t >= 0; --t) {
        const std::vector<V4<T>>& q = tp.q[t];
        std::vector<V4<T>> pbt(N, V4<T>{0, 0, 0, 0});
        std::vector<T> lb(N, 0);
#pragma omp parallel for schedule(dynamic, 64)
        for (int i = 0; i < N; ++i) {
            V3<T> fb = xyz(pb[i]);
            const uint8_t mk = st.mask[(size_t)t * N + i];
            T* f = &fb.x;
            for (int k = 0; k < 3; ++k)
                if ((mk >> (2 * k)) & 3) f[k] = 0;
            atomic_add3(pbt[i], fb);
            const int32_t* cnt = &st.counts[(size_t)i * C];
            int kl, kd;
            kept_circles(cnt, C, kl, kd);
            const int m = kept_count(cnt, kd);
            for (int f2 = 0; f2 < m; ++f2) {
                const int j = st.list[st.start[i] + f2];
                V3<T> r = sub(xyz(q[i]), xyz(q[j]));
                T r2 = dot(r, r);
                if (!support(c, r2)) continue;
                T rl = std::sqrt(r2);
                T d = c.h2 - r2;
                T W = d * d * d;
                T rq = W / c.poly6q;
                T a = q[i].w + q[j].w + c.K * rq * rq * rq * rq;
                V3<T> k = kvec(r, rl, c.h);
                T ab = negG / c.rho0 * dot(fb, k);
#pragma omp atomic
                lb[i] += ab;
#pragma omp atomic
                lb[j] += ab;
                T sW = ab * (T)4 * c.K * rq * rq * rq / c.poly6q;
                V3<T> rb = scale(sW * (T)-6 * d * d, r);
                rb = add(rb, kvec_adj(r, rl, c.h, scale(negG / c.rho0 * a, fb)));
                atomic_add3(pbt[i], rb);
                atomic_add3(pbt[j], scale((T)-1, rb));
            }
        }
#pragma omp parallel for schedule(dynamic, 64)
        for (int i = 0; i < N; ++i) {
            const int32_t* cnt = &st.counts[(size_t)i * C];
            int kl, kd;
            kept_circles(cnt, C, kl, kd);
            const int m = kept_count(cnt, kl);
            T ds = 0, gsk = 0;
            V3<T> S = {0, 0, 0};
            for (int f = 0; f < m; ++f) {
                const int j = st.list[st.start[i] + f];
                V3<T> r = sub(xyz(q[i]), xyz(q[j]));
                T r2 = dot(r, r);
                if (!support(c, r2)) continue;
                T rl = std::sqrt(r2);
                V3<T> g = scale(G, kvec(r, rl, c.h));
                T d = c.h2 - r2;
                ds += d * d * d;
                gsk += dot(g, g);
                S = add(S, g);
            }
            T rho = ds * c.poly6, D = gsk + dot(S, S);
            T den = D / (c.rho0 * c.rho0) + c.eps, Cc = rho / c.rho0 - 1;
            T Cb = -lb[i] / den, Db = lb[i] * Cc / (den * den) / (c.rho0 * c.rho0);
            T rhob = Cb / c.rho0;
            for (int f = 0; f < m; ++f) {
                const int j = st.list[st.start[i] + f];
                V3<T> r = sub(xyz(q[i]), xyz(q[j]));
                T r2 = dot(r, r);
                if (!support(c, r2)) continue;
                T rl = std::sqrt(r2);
                T d = c.h2 - r2;
                V3<T> g = scale(G, kvec(r, rl, c.h));
                V3<T> rb = scale(rhob * c.poly6 * (T)-6 * d * d, r);
                V3<T> gb = scale((T)2 * Db, add(g, S));
                rb = add(rb, kvec_adj(r, rl, c.h, scale(G, gb)));
                atomic_add3(pbt[i], rb);
                atomic_add3(pbt[j], scale((T)-1, rb));
            }
        }
        pb.swap(pbt);
    }
    // unsort, then predict: p0 = x + dt (v + dt g)
    std::vector<V4<T>> xo(N), vo(N);
    for (int k = 0; k < N; ++k) {
        const uint32_t i = st.perm[k];
        xo[i] = {xsb[k].x + pb[k].x, xsb[k].y + pb[k].y, xsb[k].z + pb[k].z, 0};
        vo[i] = {c.dt * pb[k].x, c.dt * pb[k].y, c.dt * pb[k].z, 0};
        gb[0] += c.dt * c.dt * pb[k].x;
        gb[1] += c.dt * c.dt * pb[k].y;
        gb[2] += c.dt * c.dt * pb[k].z;
    }
    xb.swap(xo);
    vb.swap(vo);
}

Structure record_structure(const State<float>& s, const std::vector<uint8_t>& masks, int C) {
    Structure st;
    const int N = s.n;
    st.perm.assign(s.perm.begin(), s.perm.begin() + N);
    st.counts.assign(s.fcount.begin(), s.fcount.end());
    st.start.assign(N + 1, 0);
    const int P = (int)(s.friends.size() / ((size_t)N * C));
    for (int i = 0; i < N; ++i) {
        int kl, kd;
        kept_circles(&s.fcount[(size_t)i * C], C, kl, kd);
        st.start[i + 1] = st.start[i] + kept_count(&s.fcount[(size_t)i * C], kl);
    }
    st.list.resize(st.start[N]);
    for (int i = 0; i < N; ++i) {
        int kl, kd, o = st.start[i];
        kept_circles(&s.fcount[(size_t)i * C], C, kl, kd);
        for (int k = 0; k < kl; ++k)
            for (int f = 0; f < s.fcount[(size_t)i * C + k]; ++f) st.list[o++] = s.friends[((size_t)i * C + k) * P + f];
    }
    st.mask = masks;
    return st;
}

}  // namespace

extern "C" {

// One or more reference Steps in FP32.  pos, vel: 4*n floats, in/out.
// pred (4*n, may be NULL) receives the predicted positions after the last
// step.  keys_state (IntCeil(n,2048), may be NULL) carries the sorted keys
// between calls, needed only for paused steps (which skip the sort).
int oracle_step_f32(const PbfParameters* p, int n, float* pos, float* vel, float* pred,
                    int substeps, int paused, uint32_t* keys_state, int nthreads, OracleDebug* dbg) {
    return run_steps<float>(p, n, pos, vel, pred, substeps, paused, keys_state, nthreads, dbg);
}

// The same pipeline in FP64 (constants are the FP32 literals, promoted).
int oracle_step_f64(const PbfParameters* p, int n, double* pos, double* vel, double* pred,
                    int substeps, int nthreads) {
    return run_steps<double>(p, n, pos, vel, pred, substeps, 0, nullptr, nthreads, nullptr);
}

// Keys, sort and cell table from given predicted positions (FP32):
// computeKeys, the 6-pass radix sort and updateCells.
int oracle_sort_f32(const PbfParameters* p, int n, const float* pred,
                    uint32_t* keys, uint32_t* perm, uint32_t* cells) {
    if (check(p, n)) return -1;
    Consts<float> c = make_consts<float>(*p);
    State<float> s;
    s.n = n;
    s.nKeys = int_ceil((uint32_t)n, 2048u);
    s.pred.resize(n);
    std::memcpy(s.pred.data(), pred, 16 * (size_t)n);
    s.keys.assign(s.nKeys, 0); s.perm.assign(s.nKeys, 0);
    for (uint32_t i = 0; i < s.nKeys; ++i) {
        if ((int)i < n) { int x, y, z; s.keys[i] = cell_hash_of(s.pred[i], c, x, y, z); }
        else s.keys[i] = kPadKey;
        s.perm[i] = i;
    }
    reference_radix_sort(s.keys, s.perm);
    s.cells.assign(2 * (size_t)p->gridBufSize, kEmpty);
    update_cells(s);
    if (keys) std::memcpy(keys, s.keys.data(), 4 * (size_t)s.nKeys);
    if (perm) std::memcpy(perm, s.perm.data(), 4 * (size_t)s.nKeys);
    if (cells) std::memcpy(cells, s.cells.data(), 8 * (size_t)p->gridBufSize);
    return 0;
}

// The compile-time constants the kernels see (POLY6_FACTOR, GRAD_SPIKY_FACTOR,
// poly6(q)), for tests of the host-side derivation.
int oracle_constants(const PbfParameters* p, float* poly6, float* grad_spiky, float* poly6_q) {
    if (!p) return -1;
    Consts<float> c = make_consts<float>(*p);
    if (poly6) *poly6 = c.poly6;
    if (grad_spiky) *grad_spiky = c.gradSpiky;
    if (poly6_q) *poly6_q = c.poly6q;
    return 0;
}

// ---- rollouts over a fixed neighbour structure ----

// FP32 forward of `substeps` substeps (identical to oracle_step_f32),
// recording the structure of each.  pos, vel: in/out; ids (n, may be NULL)
// receives the original index of each final particle.  Returns a handle for
// the replay / gradient calls (free with oracle_rollout_free), NULL on error.
void* oracle_rollout_record(const PbfParameters* p, int n, float* pos, float* vel, int substeps, uint32_t* ids,
                            int nthreads) {
    if (check(p, n) || substeps < 1 || p->completeNeighbours) return nullptr;  // the reference's sets only
    if (nthreads > 0) omp_set_num_threads(nthreads);
    Consts<float> c = make_consts<float>(*p);
    auto* rec = new RolloutRecord();
    rec->params = *p;
    rec->n = n;
    State<float> s;
    s.n = n;
    s.nKeys = int_ceil((uint32_t)n, 2048u);
    s.pos.resize(n); s.vel.resize(n); s.pred.resize(n); s.predP.resize(n); s.omega.resize(n);
    std::memcpy(s.pos.data(), pos, 16 * (size_t)n);
    std::memcpy(s.vel.data(), vel, 16 * (size_t)n);
    s.density.assign(n, 0); s.lambda.assign(n, 0);
    s.keys.assign(s.nKeys, 0); s.perm.assign(s.nKeys, 0);
    s.cells.assign(2 * (size_t)p->gridBufSize, kEmpty);
    s.friends.assign((size_t)n * c.circles * c.perCircle, 0);
    s.fcount.assign((size_t)n * c.circles, 0);
    std::vector<uint32_t> idv(n);
    for (int i = 0; i < n; ++i) idv[i] = (uint32_t)i;
    std::vector<uint8_t> masks((size_t)p->simIterations * n, 0);
    for (int step = 0; step < substeps; ++step) {
        predict(s, c, false);
        sort_particles(s, c);
        std::vector<uint32_t> id2(n);
        for (int k = 0; k < n; ++k) id2[k] = idv[s.perm[k]];
        idv.swap(id2);
        update_cells(s);
        build_friends(s, c);
        reset_grid(s);
        for (unsigned it = 0; it < p->simIterations; ++it) {
            compute_scaling(s, c);
            compute_delta(s, c, masks.data() + (size_t)it * n);
        }
        update_velocities(s, c);
        apply_viscosity(s, c);
        apply_vorticity(s, c);
        rec->steps.push_back(record_structure(s, masks, c.circles));
    }
    std::memcpy(pos, s.pos.data(), 16 * (size_t)n);
    std::memcpy(vel, s.vel.data(), 16 * (size_t)n);
    if (ids) std::memcpy(ids, idv.data(), 4 * (size_t)n);
    return rec;
}

void oracle_rollout_free(void* handle) { delete static_cast<RolloutRecord*>(handle); }

// The frozen-structure rollout in FP64 from pos0 / vel0 (4n doubles each,
// original particle order) with gravity vector g (3 doubles) and
// viscosityFactor *visc (NULL: the recorded values).  Writes the final positions by original
// index to pos_by_id (4n, may be NULL) and returns the loss
// mean_{i,axis} (x_final - target)^2 against target_by_id (4n, may be NULL).
extern "C++" {
template <typename T>
static Consts<T> replay_consts(const RolloutRecord& rec, const double* g, const double* visc) {
    Consts<T> c = make_consts<T>(rec.params);
    if (g) { c.gx = (T)g[0]; c.gy = (T)g[1]; c.gz = (T)g[2]; }
    if (visc) c.visc = (T)*visc;
    return c;
}

template <typename T>
static double replay(const RolloutRecord& rec, const double* g, const double* visc, const double* pos0,
                     const double* vel0, const double* target_by_id, double* pos_by_id,
                     std::vector<Tape<T>>* tapes, std::vector<V4<T>>* xFinal,
                     std::vector<uint32_t>* idsFinal) {
    Consts<T> c = replay_consts<T>(rec, g, visc);
    const int n = rec.n;
    std::vector<V4<T>> x(n), v(n);
    for (int i = 0; i < n; ++i) {
        x[i] = {(T)pos0[4 * i], (T)pos0[4 * i + 1], (T)pos0[4 * i + 2], (T)pos0[4 * i + 3]};
        v[i] = {(T)vel0[4 * i], (T)vel0[4 * i + 1], (T)vel0[4 * i + 2], (T)vel0[4 * i + 3]};
    }
    std::vector<uint32_t> ids(n);
    for (int i = 0; i < n; ++i) ids[i] = (uint32_t)i;
    if (tapes) tapes->assign(rec.steps.size(), {});
    for (size_t k = 0; k < rec.steps.size(); ++k)
        replay_substep(rec.steps[k], c, (int)rec.params.simIterations, x, v, ids, tapes ? &(*tapes)[k] : nullptr);
    double loss = 0;
    for (int k = 0; k < n; ++k) {
        const uint32_t id = ids[k];
        const double px = x[k].x, py = x[k].y, pz = x[k].z;
        if (pos_by_id) { pos_by_id[4 * id] = px; pos_by_id[4 * id + 1] = py; pos_by_id[4 * id + 2] = pz; pos_by_id[4 * id + 3] = 0; }
        if (target_by_id) {
            const double* tg = target_by_id + 4 * (size_t)id;
            loss += (px - tg[0]) * (px - tg[0]) + (py - tg[1]) * (py - tg[1]) + (pz - tg[2]) * (pz - tg[2]);
        }
    }
    if (xFinal) *xFinal = x;
    if (idsFinal) *idsFinal = ids;
    return loss / (3.0 * n);
}

// Reverse pass in T after a replay in T; dL/dx from the replay's own final
// positions, or from dl_dx_by_id (4n doubles, original order) when given.
template <typename T>
static double grad(const RolloutRecord& rec, const double* g, const double* visc, const double* pos0,
                   const double* vel0, const double* target_by_id, const double* dl_dx_by_id, double* dv0,
                   double* dvisc, double* dg) {
    std::vector<Tape<T>> tapes;
    std::vector<V4<T>> x;
    std::vector<uint32_t> ids;
    const double loss = replay<T>(rec, g, visc, pos0, vel0, target_by_id, nullptr, &tapes, &x, &ids);
    Consts<T> c = replay_consts<T>(rec, g, visc);
    const int n = rec.n;
    std::vector<V4<T>> xb(n), vb(n, V4<T>{0, 0, 0, 0});
    for (int k = 0; k < n; ++k) {
        if (dl_dx_by_id) {
            const double* d = dl_dx_by_id + 4 * (size_t)ids[k];
            xb[k] = {(T)d[0], (T)d[1], (T)d[2], 0};
        } else {
            const double* tg = target_by_id + 4 * (size_t)ids[k];
            const double s = 2.0 / (3.0 * n);
            xb[k] = {(T)(s * ((double)x[k].x - tg[0])), (T)(s * ((double)x[k].y - tg[1])),
                     (T)(s * ((double)x[k].z - tg[2])), 0};
        }
    }
    T cb = 0, gb[3] = {0, 0, 0};
    for (size_t k = rec.steps.size(); k-- > 0;)
        adjoint_substep(rec.steps[k], c, (int)rec.params.simIterations, tapes[k], xb, vb, cb, gb);
    if (dv0)
        for (int i = 0; i < n; ++i) {
            dv0[4 * i] = vb[i].x; dv0[4 * i + 1] = vb[i].y; dv0[4 * i + 2] = vb[i].z; dv0[4 * i + 3] = vb[i].w;
        }
    if (dvisc) *dvisc = cb;
    if (dg) for (int k = 0; k < 3; ++k) dg[k] = gb[k];
    return loss;
}

}  // extern "C++"

double oracle_rollout_replay_f64(void* handle, const double* g, const double* visc, const double* pos0,
                                 const double* vel0, const double* target_by_id, double* pos_by_id) {
    return replay<double>(*static_cast<RolloutRecord*>(handle), g, visc, pos0, vel0, target_by_id, pos_by_id, nullptr,
                          nullptr, nullptr);
}

// Loss and its exact gradient (FP64) with respect to the initial velocities
// (dv0, 4n doubles, original order), viscosityFactor (dvisc) and the gravity
// vector (dg, 3 doubles), at gravity g / viscosityFactor *visc (NULL: as
// recorded).
double oracle_rollout_grad_f64(void* handle, const double* g, const double* visc, const double* pos0,
                               const double* vel0, const double* target_by_id, double* dv0, double* dvisc, double* dg) {
    return grad<double>(*static_cast<RolloutRecord*>(handle), g, visc, pos0, vel0, target_by_id, nullptr, dv0, dvisc,
                        dg);
}

// The same replay and reverse pass evaluated in FP32, serially: the size of
// the gradient error that FP32 arithmetic alone gives, in a fixed summation
// order.  dl_dx_by_id may be NULL (dL/dx from the FP32 replay and target).
double oracle_rollout_grad_f32(void* handle, const double* pos0, const double* vel0, const double* target_by_id,
                               const double* dl_dx_by_id, double* dv0, double* dvisc, double* dg) {
    return grad<float>(*static_cast<RolloutRecord*>(handle), nullptr, nullptr, pos0, vel0, target_by_id, dl_dx_by_id,
                       dv0, dvisc, dg);
}

// Morton hash of one cell (utilities.cl:84-87).
uint32_t oracle_grid_hash(int x, int y, int z, uint32_t grid) { return grid_hash(x, y, z, grid); }

int oracle_max_threads(void) { return omp_get_max_threads(); }

// Force planes for every later step (count 0 removes them) and their mask
// (NULL: the empty mask).  Process-wide state of the oracle.
int oracle_set_force_planes(const PbfForceQuad* quads, int count, const uint32_t* mask, int w, int h) {
    if (count < 0 || (count > 0 && !quads)) return -1;
    g_quads.assign(quads, quads + count);
    if (mask && w > 0 && h > 0) {
        g_fmask.assign(mask, mask + (size_t)w * h);
        g_fmaskW = w;
        g_fmaskH = h;
    } else {
        g_fmask.clear();
        g_fmaskW = g_fmaskH = 0;
    }
    return 0;
}

// The wave generator's moving wall for every later step: the box clamp's low
// x bound is xMin + wavePos.
void oracle_set_wave_position(float wavePos) { g_wave = wavePos; }

// ---- headless render: the reference's particle shaders restated ----
// particles.vs + particles_color.fs (splat), vis_scan.cms, grid_build.cms,
// fluid_depth_smoothing.fs, fluid_final_render.fs; the orders the shaders
// leave to the hardware fixed as the library fixes them (equal depths: the
// last drawn wins; a bucket's chain in decreasing particle index).
namespace render {
struct V4 { float x, y, z, w; };
static V4 mat_mul(const float* m, float x, float y, float z, float w) {
    return {((m[0] * x + m[4] * y) + m[8] * z) + m[12] * w, ((m[1] * x + m[5] * y) + m[9] * z) + m[13] * w,
            ((m[2] * x + m[6] * y) + m[10] * z) + m[14] * w, ((m[3] * x + m[7] * y) + m[11] * z) + m[15] * w};
}
static float dot3(float ax, float ay, float az, float bx, float by, float bz) { return (ax * bx + ay * by) + az * bz; }
static float gmax(float x, float y) { return x < y ? y : x; }
static float gmin(float x, float y) { return y < x ? y : x; }
static float gclamp(float x, float a, float b) { return gmin(gmax(x, a), b); }
static int to_int(float v) {  // truncation, saturating, NaN -> 0
    if (v != v) return 0;
    if (v >= 2147483648.0f) return 2147483647;
    if (v <= -2147483648.0f) return (-2147483647 - 1);
    return (int)v;
}
static uint32_t expand(int xi) {
    uint32_t x = (uint32_t)xi;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}
static const uint32_t kBuckets = 2048u * 2048u;
static uint32_t bucket(int x, int y, int z) {
    const int m = (int)(expand(x) | (expand(y) << 1) | (expand(z) << 2));
    return (uint32_t)(m % (int)kBuckets);
}
struct Sprite { float ex, ey, ez, xw, yw, s; };
static bool sprite(const PbfCamera& cam, const float* p, Sprite& sp) {
    const V4 e = mat_mul(cam.modelView, p[0], p[1], p[2], 1.0f);
    const V4 c = mat_mul(cam.projection, e.x, e.y, e.z, e.w);
    if (!(c.w > 0.0f)) return false;
    const float nx = c.x / c.w, ny = c.y / c.w, nz = c.z / c.w;
    if (!(std::fabs(nx) <= 1.0f && std::fabs(ny) <= 1.0f && std::fabs(nz) <= 1.0f)) return false;
    float s = cam.widthOfNearPlane * cam.pointSize / c.w;
    s = std::fmin(std::fmax(s, 1.0f), 1024.0f);
    const float hw = 0.5f * (float)cam.width, hh = 0.5f * (float)cam.height;
    sp = {e.x, e.y, e.z, nx * hw + hw, ny * hh + hh, s};
    return true;
}
struct Frag { float nx, ny, nz, depth; };
static bool fragment(const PbfCamera& cam, const Sprite& sp, int i, int j, Frag& f) {
    const float pcx = 0.5f + (((float)i + 0.5f) - sp.xw) / sp.s;
    const float pcy = 0.5f - (((float)j + 0.5f) - sp.yw) / sp.s;
    f.nx = pcx * 2.0f + -1.0f;
    f.ny = pcy * 2.0f + -1.0f;
    const float mag = f.nx * f.nx + f.ny * f.ny;
    if (mag > 1.0f) return false;
    f.nz = std::sqrt(1.0f - mag);
    const V4 c = mat_mul(cam.projection, sp.ex + f.nx * cam.pointSize, sp.ey + f.ny * cam.pointSize,
                         sp.ez + f.nz * cam.pointSize, 1.0f);
    const float ndc = c.z / c.w;
    if (ndc < -1.0f) return false;
    f.depth = ((1.0f * ndc + 0.0f) + 1.0f) / 2.0f;
    return f.depth <= 1.0f;
}
static float hsv_channel(float h, float k, float s, float v) {
    const float x = h + k;
    const float fr = x - std::floor(x);
    const float p = std::fabs(fr * 6.0f - 3.0f);
    const float q = gclamp(p - 1.0f, 0.0f, 1.0f);
    return v * (1.0f * (1.0f - s) + q * s);
}
static V4 pixel_world(const PbfCamera& cam, int i, int j, float z) {
    const float nearv = cam.depthRange[0], farv = cam.depthRange[1];
    const float lz = nearv / (farv - z * (farv - nearv)) * farv;
    const float u = (((float)i + 0.5f) / (float)cam.width * 2.0f - 1.0f) * cam.invFocalLen[0];
    const float v = (((float)j + 0.5f) / (float)cam.height * 2.0f - 1.0f) * cam.invFocalLen[1];
    return mat_mul(cam.invModelView, u * lz, v * lz, -lz, 1.0f);
}
static void normalize3(float& x, float& y, float& z) {
    const float l = std::sqrt(dot3(x, y, z, x, y, z));
    x = x / l; y = y / l; z = z / l;
}
static float pow50(float x) {
    if (!(x >= 0.0f)) return std::nanf("");
    const float x2 = x * x, x4 = x2 * x2, x8 = x4 * x4, x16 = x8 * x8, x32 = x16 * x16;
    return (x32 * x16) * x2;
}
}  // namespace render

// The frame of pbf_render_frame: splat, smooth (mode 0 only) and out
// receive width x height float4 images (row 0 at the bottom); any may be NULL.
int oracle_render(const PbfCamera* camp, int mode, int n, float h, const float* pos, float* splat, float* smooth,
                  float* out) {
    using namespace render;
    if (!camp || n < 1 || !pos || mode < 0 || mode > 2) return -1;
    const PbfCamera& cam = *camp;
    const int W = cam.width, H = cam.height;
    const size_t pixels = (size_t)W * H;
    std::vector<float> depth(pixels, 2.0f);
    std::vector<int64_t> winner(pixels, -1);
    for (int p = 0; p < n; ++p) {  // draw order
        Sprite sp;
        if (!sprite(cam, pos + 4 * (size_t)p, sp)) continue;
        const int i0 = std::max(0, (int)std::ceil(sp.xw - sp.s * 0.5f - 0.5f));
        const int i1 = std::min(W - 1, (int)std::ceil(sp.xw + sp.s * 0.5f - 0.5f) - 1);
        const int j0 = std::max(0, (int)std::ceil(sp.yw - sp.s * 0.5f - 0.5f));
        const int j1 = std::min(H - 1, (int)std::ceil(sp.yw + sp.s * 0.5f - 0.5f) - 1);
        for (int j = j0; j <= j1; ++j)
            for (int i = i0; i <= i1; ++i) {
                Frag f;
                if (!fragment(cam, sp, i, j, f)) continue;
                const size_t k = (size_t)j * W + i;
                if (f.depth <= depth[k]) { depth[k] = f.depth; winner[k] = p; }  // LEQUAL
            }
    }
    std::vector<float> sc(4 * pixels, 0.0f);
    for (size_t k = 0; k < pixels; ++k) {
        if (winner[k] < 0) continue;
        const int p = (int)winner[k], i = (int)(k % W), j = (int)(k / W);
        float* c = &sc[4 * k];
        if (mode == 0) { c[0] = depth[k]; c[1] = (float)p; c[2] = 0.0f; c[3] = 1.0f; continue; }
        Sprite sp;
        Frag f{};
        sprite(cam, pos + 4 * (size_t)p, sp);
        fragment(cam, sp, i, j, f);
        const float cosA = gclamp(dot3(f.nx, f.ny, f.nz, 1.0f, 1.0f, 1.0f), 0.0f, 1.0f);
        float r, g, b;
        if (mode == 1) {
            const float v = pos[4 * (size_t)p + 3] / 20.0f;
            r = v; g = v; b = 1.0f;
        } else {
            const float hue = (float)p / (float)n * 0.7f;
            r = hsv_channel(hue, 1.0f, 0.9f, 0.9f);
            g = hsv_channel(hue, 2.0f / 3.0f, 0.9f, 0.9f);
            b = hsv_channel(hue, 1.0f / 3.0f, 0.9f, 0.9f);
        }
        c[0] = r * cosA; c[1] = g * cosA; c[2] = b * cosA; c[3] = 1.0f * cosA;
    }
    if (splat) std::memcpy(splat, sc.data(), 16 * pixels);
    if (mode != 0) {
        if (out) std::memcpy(out, sc.data(), 16 * pixels);
        return 0;
    }
    // visible particles and their buckets
    std::vector<uint8_t> vis((size_t)n, 0);
    for (size_t k = 0; k < pixels; ++k) {
        const uint32_t x = (uint32_t)(sc[4 * k + 1] + 0.5f);
        if (x < (uint32_t)n) vis[x] = 1;
    }
    std::vector<std::vector<int>> chains;
    std::vector<int32_t> slot(kBuckets, -1);
    for (int p = 0; p < n; ++p) {
        if (!vis[p]) continue;
        const float* q = pos + 4 * (size_t)p;
        const uint32_t b = bucket(to_int(q[0] / h), to_int(q[1] / h), to_int(q[2] / h));
        if (slot[b] < 0) { slot[b] = (int32_t)chains.size(); chains.emplace_back(); }
        chains[slot[b]].push_back(p);
    }
    auto sample = [&](float wx, float wy, float wz, float& density, float& gx, float& gy, float& gz) {
        const float h2 = h * h;
        density = 0.0f; gx = gy = gz = 0.0f;
        const int cx = to_int(wx / h), cy = to_int(wy / h), cz = to_int(wz / h);
        for (int iz = -1; iz <= 1; ++iz)
            for (int iy = -1; iy <= 1; ++iy)
                for (int ix = -1; ix <= 1; ++ix) {
                    const int32_t sl = slot[bucket(cx + ix, cy + iy, cz + iz)];
                    if (sl < 0) continue;
                    const std::vector<int>& ch = chains[sl];
                    for (size_t t = ch.size(); t-- > 0;) {
                        const float* pp = pos + 4 * (size_t)ch[t];
                        const float dx = pp[0] - wx, dy = pp[1] - wy, dz = pp[2] - wz;
                        const float r2 = dot3(dx, dy, dz, dx, dy, dz);
                        if (r2 < h2) {
                            const float d = h2 - r2;
                            gx = gx + dx * d * d;
                            gy = gy + dy * d * d;
                            gz = gz + dz * d * d;
                            density = density + d * d * d;
                        }
                    }
                }
        density = density * 1.0f;
        gx = gx * -6.0f; gy = gy * -6.0f; gz = gz * -6.0f;
    };
    std::vector<float> sm(4 * pixels, 0.0f);
#pragma omp parallel for schedule(dynamic, 64)
    for (long long kk = 0; kk < (long long)pixels; ++kk) {
        const size_t k = (size_t)kk;
        const int i = (int)(k % W), j = (int)(k / W);
        const float z = sc[4 * k];
        if (z == 1.0f) continue;
        const render::V4 m = pixel_world(cam, i, j, z);
        float nx = cam.invModelView[12] - m.x, ny = cam.invModelView[13] - m.y, nz = cam.invModelView[14] - m.z;
        normalize3(nx, ny, nz);
        float tp = 0.0f, sx = m.x, sy = m.y, sz = m.z, density, gx = 0.0f, gy = 0.0f, gz = 0.0f;
        for (int it = 0; it < 2; ++it) {
            sample(sx, sy, sz, density, gx, gy, gz);
            const float dd = density - 1.0f;
            const float ga = dot3(nx, ny, nz, gx, gy, gz);
            tp += dd / ga;
            sx = m.x + tp * nx; sy = m.y + tp * ny; sz = m.z + tp * nz;
        }
        const render::V4 vs = mat_mul(cam.modelView, sx, sy, sz, 1.0f);
        const render::V4 c = mat_mul(cam.projection, vs.x, vs.y, vs.z, 1.0f);
        const float ndc = c.z / c.w;
        if (ndc < -1.0f) continue;
        normalize3(gx, gy, gz);
        float* r = &sm[4 * k];
        r[0] = ((1.0f * ndc + 0.0f) + 1.0f) / 2.0f; r[1] = gx; r[2] = gy; r[3] = gz;
    }
    if (smooth) std::memcpy(smooth, sm.data(), 16 * pixels);
    if (!out) return 0;
    std::vector<float> fo(4 * pixels, 0.0f);
    const int di[5] = {0, 1, -1, 0, 0}, dj[5] = {0, 0, 0, 1, -1};
    for (size_t k = 0; k < pixels; ++k) {
        const int i = (int)(k % W), j = (int)(k / W);
        bool discard = false;
        for (int q = 0; q < 5 && !discard; ++q) {
            const int a = i + di[q], b = j + dj[q];
            const float z = (a >= 0 && a < W && b >= 0 && b < H) ? sm[4 * ((size_t)b * W + a)] : 0.0f;
            discard = (z == 1.0f);
        }
        if (discard) continue;
        const float* s = &sm[4 * k];
        const render::V4 w = pixel_world(cam, i, j, s[0]);
        float ex = cam.invModelView[12] - w.x, ey = cam.invModelView[13] - w.y, ez = cam.invModelView[14] - w.z;
        normalize3(ex, ey, ez);
        const float lx = 0.0f, ly = 1.0f, lz = 0.0f;
        float hx = lx + ex, hy = ly + ey, hz = lz + ez;
        normalize3(hx, hy, hz);
        const float diff = gclamp(dot3(lx, ly, lz, s[1], s[2], s[3]), 0.0f, 1.0f);
        const float spec = gmax(0.0f, pow50(dot3(s[1], s[2], s[3], hx, hy, hz)));
        float* r = &fo[4 * k];
        r[0] = 0.0f * diff + 1.0f * spec; r[1] = 0.0f * diff + 1.0f * spec; r[2] = 0.5f * diff + 1.0f * spec; r[3] = 1.0f;
    }
    std::memcpy(out, fo.data(), 16 * pixels);
    return 0;
}

// The force planes' noise sine, for the tests.
float oracle_noise_sinf(float x) { return noise_sinf_ref(x); }

// A scenario file read as the reference's LoadParameters reads it
// (src/ParamUtils.cpp:24-100): '#' starts a comment, keys are
// case-insensitive, each line's first word names a field and the next is
// its value, the computed fields are set at the end (:97-99).  The keys the
// benchmark's scenario files add are read too: the gravity vector, BoxClamp,
// ZeroDistanceGuard, RelaxedMath, CompleteNeighbours, and the initial block
// (BlockDims, BlockOrigin, Jitter, Seed).  `p` keeps the values of fields the
// text does not name.  Returns the number of unknown keys.
int oracle_load_scenario(const char* text, PbfParameters* p, int* dims, float* origin, float* jitter,
                         uint64_t* seed) {
    std::string all(text), line;
    size_t at = 0;
    int unknown = 0;
    while (at < all.size()) {
        const size_t nl = all.find('\n', at);
        line = all.substr(at, nl == std::string::npos ? std::string::npos : nl - at);
        at = nl == std::string::npos ? all.size() : nl + 1;
        line.erase(std::find(line.begin(), line.end(), '#'), line.end());
        for (char& ch : line) ch = (char)std::tolower((unsigned char)ch);
        char key[64];
        int used = 0;
        if (std::sscanf(line.c_str(), " %63s%n", key, &used) != 1) continue;
        const char* v = line.c_str() + used;
        const std::string k(key);
        auto F = [&](float& f) { std::sscanf(v, "%f", &f); };
        auto U = [&](unsigned& u) { std::sscanf(v, "%u", &u); };
        auto I = [&](int& i) { std::sscanf(v, "%d", &i); };
        if (k == "resetsimonchange") I(p->resetSimOnChange);
        else if (k == "particlecount") U(p->particleCount);
        else if (k == "xmin") F(p->xMin);
        else if (k == "xmax") F(p->xMax);
        else if (k == "ymin") F(p->yMin);
        else if (k == "ymax") F(p->yMax);
        else if (k == "zmin") F(p->zMin);
        else if (k == "zmax") F(p->zMax);
        else if (k == "wavegenamp") F(p->waveGenAmp);
        else if (k == "wavegenfreq") F(p->waveGenFreq);
        else if (k == "wavegenduty") F(p->waveGenDuty);
        else if (k == "timestep") F(p->timeStep);
        else if (k == "simiterations") U(p->simIterations);
        else if (k == "substeps") U(p->subSteps);
        else if (k == "smoothlen") F(p->h);
        else if (k == "gridbuffersize") U(p->gridBufSize);
        else if (k == "restdensity") F(p->restDensity);
        else if (k == "epsilon") F(p->epsilon);
        else if (k == "garvity") F(p->garvity);
        else if (k == "vorticityfactor") F(p->vorticityFactor);
        else if (k == "viscosityfactor") F(p->viscosityFactor);
        else if (k == "surfacetenstionk") F(p->surfaceTenstionK);
        else if (k == "surfacetenstiondist") F(p->surfaceTenstionDist);
        else if (k == "setupspacing") F(p->setupSpacing);
        else if (k == "segmentsize") U(p->segmentSize);
        else if (k == "sortiterations") U(p->sortIterations);
        else if (k == "particlerendersize") F(p->particleRenderSize);
        else if (k == "enablecachedbuffers") { int b = 0; I(b); p->EnableCachedBuffers = b != 0; }
        else if (k == "gravityx") { F(p->gravityX); p->gravityVectorEnable = 1; }
        else if (k == "gravityy") { F(p->gravityY); p->gravityVectorEnable = 1; }
        else if (k == "gravityz") { F(p->gravityZ); p->gravityVectorEnable = 1; }
        else if (k == "boxclamp") I(p->boxClamp);
        else if (k == "zerodistanceguard") I(p->zeroDistanceGuard);
        else if (k == "relaxedmath") I(p->relaxedMath);
        else if (k == "completeneighbours") I(p->completeNeighbours);
        else if (k == "blockdims") std::sscanf(v, "%d %d %d", &dims[0], &dims[1], &dims[2]);
        else if (k == "blockorigin") std::sscanf(v, "%f %f %f", &origin[0], &origin[1], &origin[2]);
        else if (k == "jitter") std::sscanf(v, "%f", jitter);
        else if (k == "seed") { unsigned long long sd = 0; std::sscanf(v, "%llu", &sd); *seed = sd; }
        else ++unknown;
    }
    p->h_2 = p->h * p->h;
    p->friendsCircles = 5;
    p->particlesPerCircle = 50;
    return unknown;
}

// The benchmark scenes' initial block: nx x ny x nz particles at `spacing`
// from the origin, x fastest, each coordinate moved by U(-jitter, jitter)
// drawn from a 64-bit Mersenne Twister seeded with `seed` (53 bits of each
// draw, in double, rounded once to float).
int oracle_scene_block(int nx, int ny, int nz, float spacing, const float* origin, float jitter, uint64_t seed,
                       float* pos) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || !pos) return -1;
    std::mt19937_64 rng(seed);
    size_t i = 0;
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix, ++i) {
                const int idx[3] = {ix, iy, iz};
                for (int c = 0; c < 3; ++c) {
                    const double u = (double)(rng() >> 11) / 9007199254740992.0;
                    pos[4 * i + c] = (float)((double)origin[c] + idx[c] * (double)spacing + (2.0 * u - 1.0) * (double)jitter);
                }
                pos[4 * i + 3] = 0.0f;
            }
    return 0;
}

}  // extern "C"
