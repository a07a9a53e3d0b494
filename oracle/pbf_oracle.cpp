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
#include <vector>
#include <omp.h>

#include "../include/pbf_params.h"

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
        T density_sum = 0, grad_sum_k = 0;
        V3<T> grad_sum_k_i = {0, 0, 0};
        int kept = circles_kept(cnt, C, 0.6f);
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

// compute_delta.cl:54-185 (with the force planes the identity), then
// update_predicted.cl (pred += delta).  The clamp, when enabled, bounds
// `future` to the box before the delta is formed.
template <typename T> void compute_delta(State<T>& s, const Consts<T>& c) {
    const int C = c.circles, P = c.perCircle;
    const T negG = -c.gradSpiky;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < s.n; ++i) {
        const int32_t* cnt = &s.fcount[(size_t)i * C];
        const int32_t* lst = &s.friends[(size_t)i * C * P];
        V4<T> pi = s.predP[i];
        V3<T> sum = {0, 0, 0};
        int kept = circles_kept(cnt, C, 0.5f);
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
        if (c.clamp) {  // comparisons, so that -0.0 and NaN pass through unchanged
            fut.x = fut.x < c.lo[0] ? c.lo[0] : (fut.x > c.hi[0] ? c.hi[0] : fut.x);
            fut.y = fut.y < c.lo[1] ? c.lo[1] : (fut.y > c.hi[1] ? c.hi[1] : fut.y);
            fut.z = fut.z < c.lo[2] ? c.lo[2] : (fut.z > c.hi[2] ? c.hi[2] : fut.z);
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
        int kept = circles_kept(cnt, C, 0.5f);
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
        int kept = circles_kept(cnt, C, 0.5f);
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
            int kl = circles_kept(cnt, C, 0.6f), kd = circles_kept(cnt, C, 0.5f);
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

// Morton hash of one cell (utilities.cl:84-87).
uint32_t oracle_grid_hash(int x, int y, int z, uint32_t grid) { return grid_hash(x, y, z, grid); }

int oracle_max_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
