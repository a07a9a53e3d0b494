// pbf_kernels.cu — the per-substep PBF stages on sm_103a.
//
// Arithmetic contract (shared with the CPU oracle): this file is compiled
// with --fmad=false, IEEE division and IEEE sqrt, so every float operation
// below is one correctly rounded IEEE operation, evaluated in the order of
// the reference kernel it stands for.  With the same inputs the results are
// bit-identical to a strict IEEE evaluation of the reference's kernels.
//   dot(a,b)       = (a.x*b.x + a.y*b.y) + a.z*b.z
//   cross(a,b)     = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x)
//   fast_length(a) = sqrtf(dot(a,a))
//   convert_int    = __float2int_rz (truncating, saturating, NaN -> 0)
//
// Data layout in device memory (N particles, all arrays dense):
//   pos, pred, vel, omega : float4[N]  (16-byte records, coalesced 128-bit I/O)
//   keys, perm            : uint32[N]
//   cells                 : uint2[gridBufSize]  (start, inclusive end)
//   list                  : uint32[circles * perCircle][N]: friend s of circle
//                           c of particle i at row c*perCircle + s (the
//                           reference's friends layout, build_friends_list.cl:
//                           1-21); a warp of consecutive particles reads one
//                           row coalesced.
//   flat                  : uint32[circles * perCircle][N]: particle i's
//                           friends in summation order, the t-th in row t;
//                           recorded by the first density pass of a substep
//                           and walked by the passes after it.
//   meta                  : uint2[N] per particle: 7-bit friend count of each
//                           of up to 8 circles (bits 0-55), the circles the
//                           density pass keeps (bits 56-59) and the circles
//                           the other passes keep (bits 60-63).

#include <cuda_runtime.h>
#include <cstdint>

#include "pbf_device.cuh"
#include "pbf_internal.h"

namespace pbf {
namespace {

constexpr int kBlock = 256;

inline unsigned blocks_for(int n, int block = kBlock) { return (unsigned)((n + block - 1) / block); }

// Scene values of particle i: from the batch table, or DevConsts for a
// single scene.
__device__ __forceinline__ uint32_t key_base(const Batch& b, int i) {
    return b.scenes ? b.scenes[b.sceneOf[i]].keyBase : 0u;
}

// ------------------------------------------------------------- predict --
// predict_positions.cl:8-17 fused with computeKeys (radixsort.cl:7-19).
__global__ void predict_keys_kernel(DevConsts c, Batch b, const float4* __restrict__ pos, float4* __restrict__ vel,
                                    float4* __restrict__ pred, uint32_t* __restrict__ keys,
                                    uint32_t* __restrict__ perm, int paused) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    float4 v = vel[i];
    float gx = c.gx, gy = c.gy, gz = c.gz;
    uint32_t base = 0;
    if (b.scenes) {
        const SceneParams& sp = b.scenes[b.sceneOf[i]];
        gx = sp.gx; gy = sp.gy; gz = sp.gz;
        base = sp.keyBase;
    }
    if (!paused) {
        v.x = v.x + c.dt * gx;
        v.y = v.y + c.dt * gy;
        v.z = v.z + c.dt * gz;
        vel[i] = v;
    }
    const float4 p = pos[i];
    const float4 q = make_float4(p.x + c.dt * v.x, p.y + c.dt * v.y, p.z + c.dt * v.z, p.w + c.dt * v.w);
    pred[i] = q;
    if (i == 0) *c.epoch += 1u;  // a new substep: earlier taint marks lapse
    if (!paused) {
        keys[i] = base + grid_hash(__float2int_rz(q.x / c.h), __float2int_rz(q.y / c.h), __float2int_rz(q.z / c.h), c.grid);
        perm[i] = (uint32_t)i;
    }
}

// radixsort.cl:1-20 alone (keys of given predicted positions, no padding).
__global__ void compute_keys_kernel(DevConsts c, Batch b, const float4* __restrict__ pred,
                                    uint32_t* __restrict__ keys, uint32_t* __restrict__ perm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const float4 q = pred[i];
    keys[i] = key_base(b, i) + grid_hash(__float2int_rz(q.x / c.h), __float2int_rz(q.y / c.h), __float2int_rz(q.z / c.h), c.grid);
    perm[i] = (uint32_t)i;
}

// radixsort.cl:22-37 (velocities are not permuted; they are recomputed
// before any read, update_velocities.cl:13).
// Particle ids (the original index of each record) follow the same
// permutation into idsOut.
__global__ void gather_sorted_kernel(int n, const uint32_t* __restrict__ perm, const float4* __restrict__ pos,
                                     const float4* __restrict__ pred, const uint32_t* __restrict__ ids,
                                     float4* __restrict__ posOut, float4* __restrict__ predOut,
                                     uint32_t* __restrict__ idsOut, int* err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t j = checked_index(perm[i], (uint32_t)n, err, kErrSortIndex);
    posOut[i] = pos[j];
    predOut[i] = pred[j];
    idsOut[i] = ids[j];
}

// --------------------------------------------------------------- cells --
// update_cells.cl:6-25 on a table that holds END_OF_CELL_LIST everywhere.
// cellStart (may be NULL) also receives each occupied cell's first particle;
// it is never reset (taint_around checks an entry against the keys).
__global__ void update_cells_kernel(int n, const uint32_t* __restrict__ keys, uint32_t* __restrict__ cells,
                                    uint32_t keyLimit, int* err, uint32_t* __restrict__ cellStart) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = checked_index(keys[i], keyLimit, err, kErrCellKey);
    if (i > 0) {
        const uint32_t kp = checked_index(keys[i - 1], keyLimit, err, kErrCellKey);
        if (kp != k) {
            cells[2 * (size_t)k] = (uint32_t)i;
            cells[2 * (size_t)kp + 1] = (uint32_t)(i - 1);
            if (cellStart) cellStart[k] = (uint32_t)i;
        }
        if (i == n - 1) cells[2 * (size_t)k + 1] = (uint32_t)i;
    } else {
        cells[2 * (size_t)k] = 0u;
        if (cellStart) cellStart[k] = 0u;
    }
}

// reset_grid.cl:6-14
__global__ void reset_cells_kernel(int n, const uint32_t* __restrict__ keys, uint2* __restrict__ cells,
                                   uint32_t keyLimit, int* err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    cells[checked_index(keys[i], keyLimit, err, kErrCellKey)] = make_uint2(kEmpty, kEmpty);
}

// Number of leading circles a pass keeps: circles are visited in order and
// skipped once processed/total exceeds the threshold (compute_scaling.cl:47-54
// with 0.6f; compute_delta.cl:97-104, apply_viscosity.cl:25-32 and
// apply_vorticity.cl:23-30 with 0.5f).
__device__ __forceinline__ int circles_kept(uint64_t cnt, int C, int total, float threshold) {
    int processed = 0, kept = 0;
    for (int k = 0; k < C; ++k) {
        if (((float)processed) / total > threshold) continue;
        processed += (int)byte_of(cnt, k);
        kept = k + 1;
    }
    return kept;
}

// One particle's friend circles as the candidates arrive (build_friends_list.cl:
// 58-95): r^2 < h^2, binned into circles by min(int(adj^3 * C), C-1) with
// adj = max(0, (r - 0.3h) / 0.7h), at most perCircle per circle (later ones
// are dropped, :79-83).  The circle is read off precomputed r^2 thresholds
// (DevConsts::circT): the same integer the sqrt / divide / cube / truncate
// sequence gives, without computing it.
//
// Narrow (at most 5 circles of at most 63): the counters are 6-bit fields of
// one word, so a candidate's slot, the test "inside and its circle not full",
// the store and the increment are a few 32-bit operations with no branch
// (the wide form's 64-bit counter arithmetic is longer).  Either form writes
// the same entries in the same order.
template <bool Narrow>
struct FriendCircles {
    const DevConsts& c;
    uint32_t* row0;     // this particle's entry of list row 0; row r is row0 + r * n
    uint32_t rowBytes;  // 4 n
    int n, i;
    float4 pi;
    uint64_t cnt = 0;   // wide: 8 circles x 8-bit counters
    uint32_t cnt6 = 0;  // narrow: 5 circles x 6-bit counters
    __device__ __forceinline__ FriendCircles(const DevConsts& cc, uint32_t* l, int i_, float4 p)
        : c(cc), row0(l + i_), rowBytes(4u * (uint32_t)cc.n), n(cc.n), i(i_), pi(p) {}
    __device__ __forceinline__ uint32_t count(int k) const {
        return Narrow ? (cnt6 >> (6 * k)) & 63u : byte_of(cnt, k);
    }
    __device__ __forceinline__ void consider(uint32_t j, const float4 pj) {
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        const float r2 = dot3(rx, ry, rz, rx, ry, rz);
        // thresholds past C-1 are +inf, so only the first C-1 decide
        int circ = (r2 >= c.circT[0]) + (r2 >= c.circT[1]) + (r2 >= c.circT[2]) + (r2 >= c.circT[3]);
        if (Narrow) {
            const uint32_t sh = 6u * (uint32_t)circ;
            const uint32_t k = (cnt6 >> sh) & 63u;
            const bool take = !(r2 >= c.h2) && (int)k < c.perCircle;  // NaN distances are taken, as in the scan
            const uint32_t row = (uint32_t)circ * (uint32_t)c.perCircle + k;
            if (take) *reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(row0) + (size_t)row * rowBytes) = j;
            cnt6 += take ? 1u << sh : 0u;
        } else {
            if (r2 >= c.h2) return;
            if (c.circles > 5) circ += (r2 >= c.circT[4]) + (r2 >= c.circT[5]) + (r2 >= c.circT[6]);
            const uint32_t k = byte_of(cnt, circ);
            if ((int)k >= c.perCircle) return;
            row0[(size_t)(circ * c.perCircle + (int)k) * n] = j;
            cnt += 1ull << (8 * circ);
        }
    }
    __device__ __forceinline__ void finish(uint2* meta) const {
        const int C = c.circles;
        int total = 0;
        uint64_t mt = 0, bytes = 0;
        for (int k = 0; k < C; ++k) {
            total += (int)count(k);
            mt |= (uint64_t)count(k) << (7 * k);
            bytes |= (uint64_t)count(k) << (8 * k);
        }
        mt |= (uint64_t)(c.complete ? C : circles_kept(bytes, C, total, 0.6f)) << 56;
        mt |= (uint64_t)(c.complete ? C : circles_kept(bytes, C, total, 0.5f)) << 60;
        meta[i] = make_uint2((uint32_t)mt, (uint32_t)(mt >> 32));
    }
};

// build_friends_list.cl:29-102 for particle i: one scan of the 27 neighbour
// cells in the reference's order (x, then y, then z offsets; particles of a
// cell in sorted order), self excluded, candidates read through L1 with U
// loads in flight.  The 27 hashes are formed from the three spread
// coordinates of each axis.
template <int U, typename FC>
__device__ __forceinline__ void friends_scan_global(const DevConsts& c, uint32_t base, const float4* __restrict__ pred,
                                                   const uint2* __restrict__ cells, int* __restrict__ err, FC& fc) {
    const int i = fc.i, n = c.n;
    const float4 pi = fc.pi;
    const int cx = __float2int_rz(pi.x / c.h), cy = __float2int_rz(pi.y / c.h), cz = __float2int_rz(pi.z / c.h);
    const bool pow2 = (c.grid & (c.grid - 1)) == 0;
    const uint32_t mask = c.grid - 1;
    const uint32_t exm = expand_bits(cx - 1), ex0 = expand_bits(cx), exp_ = expand_bits(cx + 1);
    const uint32_t eym = expand_bits(cy - 1) << 1, ey0 = expand_bits(cy) << 1, eyp = expand_bits(cy + 1) << 1;
    const uint32_t ezm = expand_bits(cz - 1) << 2, ez0 = expand_bits(cz) << 2, ezp = expand_bits(cz + 1) << 2;
    const uint32_t selfHash = pow2 ? ((ex0 | ey0 | ez0) & mask) : ((ex0 | ey0 | ez0) % c.grid);
    record_cell(c, i, pi, cx, cy, cz, base);
    auto scan = [&](uint32_t lo, uint32_t hi) {
        uint32_t j = lo;
        for (; j + (U - 1) <= hi; j += U) {
            float4 p[U];
#pragma unroll
            for (int u = 0; u < U; ++u) p[u] = __ldg(pred + j + u);
#pragma unroll
            for (int u = 0; u < U; ++u) fc.consider(j + u, p[u]);
        }
        for (; j <= hi; ++j) fc.consider(j, __ldg(pred + j));
    };
    for (int x = -1; x <= 1; ++x) {
        const uint32_t ex = x < 0 ? exm : (x > 0 ? exp_ : ex0);
        for (int y = -1; y <= 1; ++y) {
            const uint32_t exy = ex | (y < 0 ? eym : (y > 0 ? eyp : ey0));
            for (int z = -1; z <= 1; ++z) {
                const uint32_t m = exy | (z < 0 ? ezm : (z > 0 ? ezp : ez0));
                const uint32_t hm = pow2 ? (m & mask) : (m % c.grid);
                const uint2 range = cells[base + hm];
                if (range.x == kEmpty) continue;
                const uint32_t last = min(range.y, (uint32_t)(n - 1));
                if (range.x > last) { atomicOr(err, kErrCellTable); continue; }
                if (hm == selfHash && range.x <= (uint32_t)i && (uint32_t)i <= last) {
                    // the particle's own table entry: skip itself (build_friends_list.cl:62)
                    if ((uint32_t)i > range.x) scan(range.x, (uint32_t)i - 1);
                    if ((uint32_t)i < last) scan((uint32_t)i + 1, last);
                } else {
                    scan(range.x, last);
                }
            }
        }
    }
}

// One thread per particle, candidates through L1.
template <int U, bool Narrow>
__global__ void __launch_bounds__(kMaxBlock)
build_friends_kernel(DevConsts c, Batch b, const float4* __restrict__ pred, const uint2* __restrict__ cells,
                     uint32_t* __restrict__ list, uint2* __restrict__ meta, int* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    FriendCircles<Narrow> fc(c, list, i, pred[i]);
    friends_scan_global<U>(c, key_base(b, i), pred, cells, err, fc);
    fc.finish(meta);
}

// The same lists with the candidates streamed through shared memory, one
// block per brick of B x B x B cells (B^3 consecutive Morton numbers, so the
// brick's particles are one range of the sorted order).  The block stages the
// brick's (B+2)^3 halo of cells into shared memory with coalesced float4
// loads (every particle's 27 neighbour cells lie in it), then each thread
// scans its particle's 27 cells from there in the reference's order.  A
// particle whose cell is not the brick's (a key that aliases through the hash
// modulo), or a halo too large for the buffer, takes the per-particle scan
// through L1.  Needs a power-of-two GridBufferSize of at least B^3.
template <int B> struct BrickShape;
template <> struct BrickShape<4> { static constexpr int threads = 256, capacity = 2816; };  // 44 KB of float4

__device__ __forceinline__ uint32_t compact_bits(uint32_t x) {
    x &= 0x09249249u;
    x = (x ^ (x >> 2)) & 0x030C30C3u;
    x = (x ^ (x >> 4)) & 0x0300F00Fu;
    x = (x ^ (x >> 8)) & 0x030000FFu;
    x = (x ^ (x >> 16)) & 0x000003FFu;
    return x;
}

template <int B, bool Narrow>
__global__ void __launch_bounds__(BrickShape<B>::threads)
build_friends_brick_kernel(DevConsts c, const float4* __restrict__ pred, const uint2* __restrict__ cells,
                           uint32_t* __restrict__ list, uint2* __restrict__ meta, int* __restrict__ err) {
    constexpr int T = BrickShape<B>::threads, kCap = BrickShape<B>::capacity;
    constexpr int E = B + 2, kHalo = E * E * E, kCodes = B * B * B, kPerLane = (kHalo + 31) / 32;
    __shared__ uint32_t hStart[kHalo], hCount[kHalo], hOff[kHalo];
    __shared__ float4 staged[kCap];
    __shared__ uint32_t firstP, lastP, haloTotal;
    const int t = threadIdx.x, n = c.n;
    const uint32_t key0 = blockIdx.x * (uint32_t)kCodes;   // first key of the brick
    const uint32_t base = (key0 / c.grid) * c.grid;        // the scene's key offset
    const uint32_t m0 = key0 - base;                       // its Morton number
    const int bx = (int)compact_bits(m0), by = (int)compact_bits(m0 >> 1), bz = (int)compact_bits(m0 >> 2);
    if (t == 0) { firstP = 0xFFFFFFFFu; lastP = 0u; }
    __syncthreads();
    for (int q = t; q < kCodes; q += T) {  // the brick's particle range
        const uint2 r = cells[key0 + q];
        if (r.x != kEmpty) {
            atomicMin(&firstP, r.x);
            atomicMax(&lastP, min(r.y, (uint32_t)(n - 1)));
        }
    }
    const uint32_t mask = c.grid - 1;
    for (int h = t; h < kHalo; h += T) {
        const int hx = bx - 1 + h / (E * E), hy = by - 1 + (h / E) % E, hz = bz - 1 + h % E;
        const uint32_t m = expand_bits(hx) | (expand_bits(hy) << 1) | (expand_bits(hz) << 2);
        const uint2 range = cells[base + (m & mask)];
        uint32_t count = 0;
        if (range.x != kEmpty) {
            const uint32_t last = min(range.y, (uint32_t)(n - 1));
            if (range.x <= last) count = last - range.x + 1u;
            else atomicOr(err, kErrCellTable);
        }
        hStart[h] = range.x;
        hCount[h] = count;
    }
    __syncthreads();
    if (firstP == 0xFFFFFFFFu) return;  // an empty brick
    if (t < 32) {  // exclusive scan of the halo counts
        uint32_t v[kPerLane], s = 0;
#pragma unroll
        for (int k = 0; k < kPerLane; ++k) {
            const int h = kPerLane * t + k;
            v[k] = h < kHalo ? hCount[h] : 0u;
            s += v[k];
        }
        uint32_t incl = s;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (t >= d) incl += u;
        }
        uint32_t run = incl - s;
#pragma unroll
        for (int k = 0; k < kPerLane; ++k) {
            const int h = kPerLane * t + k;
            if (h < kHalo) hOff[h] = run;
            run += v[k];
        }
        if (t == 31) haloTotal = incl;
    }
    __syncthreads();
    const uint32_t total = haloTotal;
    const bool useSmem = total <= (uint32_t)kCap;
    if (useSmem) {
        for (uint32_t e = t; e < total; e += T) {
            int lo = 0;  // the halo cell holding staged entry e: the last with hOff <= e
#pragma unroll
            for (int s = 128; s > 0; s >>= 1)
                if (lo + s < kHalo && hOff[lo + s] <= e) lo += s;
            while (lo < kHalo - 1 && (hCount[lo] == 0 || hOff[lo] + hCount[lo] <= e)) ++lo;
            staged[e] = pred[hStart[lo] + (e - hOff[lo])];
        }
    }
    __syncthreads();
    for (uint32_t p = firstP + t; p <= lastP; p += T) {
        const int i = (int)p;
        FriendCircles<Narrow> fc(c, list, i, pred[i]);
        const int cx = __float2int_rz(fc.pi.x / c.h), cy = __float2int_rz(fc.pi.y / c.h), cz = __float2int_rz(fc.pi.z / c.h);
        const int lx = cx - bx, ly = cy - by, lz = cz - bz;
        if (useSmem && (unsigned)lx < (unsigned)B && (unsigned)ly < (unsigned)B && (unsigned)lz < (unsigned)B) {
            record_cell(c, i, fc.pi, cx, cy, cz, base);
            // staged entries [a, b) of one cell, candidates st + (k - off), two in flight, self skipped
            auto scanStaged = [&](uint32_t a, uint32_t b, uint32_t jOfA) {
                uint32_t k = a;
                for (; k + 1 < b; k += 2) {
                    const float4 p0 = staged[k], p1 = staged[k + 1];
                    fc.consider(jOfA + (k - a), p0);
                    fc.consider(jOfA + (k + 1 - a), p1);
                }
                if (k < b) fc.consider(jOfA + (k - a), staged[k]);
            };
#pragma unroll 1
            for (int x = 0; x < 3; ++x)
#pragma unroll 1
                for (int y = 0; y < 3; ++y)
#pragma unroll
                    for (int z = 0; z < 3; ++z) {
                        const int h = (lx + x) * (E * E) + (ly + y) * E + (lz + z);
                        const uint32_t cnt = hCount[h], off = hOff[h], st = hStart[h];
                        if ((uint32_t)i - st < cnt) {  // the particle's own range: skip itself
                            const uint32_t self = off + ((uint32_t)i - st);
                            scanStaged(off, self, st);
                            scanStaged(self + 1, off + cnt, (uint32_t)i + 1);
                        } else {
                            scanStaged(off, off + cnt, st);
                        }
                    }
        } else {
            friends_scan_global<2>(c, base, pred, cells, err, fc);
        }
        fc.finish(meta);
    }
}

// The same lists, built warp-cooperatively.  A warp takes its 32 particles
// run by run (a run: consecutive particles in one cell of one scene, which
// share the 27-cell candidate sequence).  Lanes take 32 candidates of the
// run's sequence at a time, in order (the candidate of lane L follows that of
// lane L-1), and every run member tests all 32: its accepted candidates are
// appended to their circles in sequence order, with ranks from the circle
// counts and match_any, so the lists equal those of the per-particle scan
// while every lane stays busy.  Circle counts saturate at perCircle.
__global__ void __launch_bounds__(kMaxBlock)
build_friends_warp_kernel(DevConsts c, Batch b, const float4* __restrict__ pred, const uint2* __restrict__ cells,
                          uint32_t* __restrict__ list, uint2* __restrict__ meta, int* __restrict__ err) {
    constexpr unsigned kFull = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int warpBase = i - lane;
    const int n = c.n;
    if (warpBase >= n) return;  // whole warp idle
    const bool valid = i < n;
    const float4 pi = valid ? pred[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const int cx = __float2int_rz(pi.x / c.h), cy = __float2int_rz(pi.y / c.h), cz = __float2int_rz(pi.z / c.h);
    const uint32_t base = valid ? key_base(b, i) : 0u;
    const int C = c.circles, P = c.perCircle;
    if (valid) record_cell(c, i, pi, cx, cy, cz, base);
    const bool pow2 = (c.grid & (c.grid - 1)) == 0;
    const uint32_t gmask = c.grid - 1;
    const int ux = __shfl_up_sync(kFull, cx, 1), uy = __shfl_up_sync(kFull, cy, 1), uz = __shfl_up_sync(kFull, cz, 1);
    const uint32_t ub = __shfl_up_sync(kFull, base, 1);
    const bool head = valid && (lane == 0 || cx != ux || cy != uy || cz != uz || base != ub);
    uint32_t heads = __ballot_sync(kFull, head);
    const uint32_t validMask = __ballot_sync(kFull, valid);
    const uint32_t ltMask = (1u << lane) - 1u;
    const uint32_t capP = (uint32_t)P * 0x01010101u;
    uint32_t cntLo = 0, cntHi = 0;  // this lane's particle: 8 circles x 8-bit counters
    while (heads) {
        const int h0 = __ffs(heads) - 1;
        heads &= heads - 1;
        const int h1 = heads ? __ffs(heads) - 1 : 32;
        const uint32_t upTo = h1 == 32 ? kFull : ((1u << h1) - 1u);
        const uint32_t runMask = validMask & upTo & ~((1u << h0) - 1u);
        const int rx0 = __shfl_sync(kFull, cx, h0), ry0 = __shfl_sync(kFull, cy, h0), rz0 = __shfl_sync(kFull, cz, h0);
        const uint32_t rbase = __shfl_sync(kFull, base, h0);
        // lane q < 27: neighbour cell q in the scan order (x, then y, then z offsets)
        uint32_t start = 0, count = 0;
        if (lane < 27) {
            const int x = lane / 9 - 1, y = (lane / 3) % 3 - 1, z = lane % 3 - 1;
            const uint32_t m = expand_bits(rx0 + x) | (expand_bits(ry0 + y) << 1) | (expand_bits(rz0 + z) << 2);
            const uint2 range = cells[rbase + (pow2 ? (m & gmask) : (m % c.grid))];
            if (range.x != kEmpty) {
                const uint32_t last = min(range.y, (uint32_t)(n - 1));
                if (range.x > last) atomicOr(err, kErrCellTable);
                else { start = range.x; count = last - range.x + 1u; }
            }
        }
        uint32_t end = count;  // inclusive scan: candidates up to and including cell q
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(kFull, end, d);
            if (lane >= d) end += v;
        }
        const uint32_t total = __shfl_sync(kFull, end, 31);
        for (uint32_t t0 = 0; t0 < total; t0 += 32) {
            const uint32_t t = t0 + (uint32_t)lane;
            const bool tv = t < total;
            int q = 0;  // the first cell with end > t
#pragma unroll
            for (int s = 16; s > 0; s >>= 1) {
                const uint32_t e = __shfl_sync(kFull, end, q + s - 1);
                if (e <= t) q += s;
            }
            const uint32_t qs = __shfl_sync(kFull, start, q), qe = __shfl_sync(kFull, end, q);
            const uint32_t qc = __shfl_sync(kFull, count, q);
            const uint32_t j = qs + (t - (qe - qc));
            const float4 pj = tv ? __ldg(pred + j) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            for (uint32_t rm = runMask; rm; rm &= rm - 1u) {
                const int pl = __ffs(rm) - 1;
                const int ip = warpBase + pl;
                const float px = __shfl_sync(kFull, pi.x, pl), py = __shfl_sync(kFull, pi.y, pl);
                const float pz = __shfl_sync(kFull, pi.z, pl);
                const float rx = px - pj.x, ry = py - pj.y, rz = pz - pj.z;
                const float r2 = dot3(rx, ry, rz, rx, ry, rz);
                const bool acc = tv && (int)j != ip && !(r2 >= c.h2);  // NaN distances are kept, as in the scan
                const uint32_t am = __ballot_sync(kFull, acc);
                if (!am) continue;
                int circ = (r2 >= c.circT[0]) + (r2 >= c.circT[1]) + (r2 >= c.circT[2]) + (r2 >= c.circT[3]);
                if (C > 5) circ += (r2 >= c.circT[4]) + (r2 >= c.circT[5]) + (r2 >= c.circT[6]);
                const uint32_t plo = __shfl_sync(kFull, cntLo, pl), phi = __shfl_sync(kFull, cntHi, pl);
                if (acc) {
                    const uint32_t peers = __match_any_sync(am, circ);
                    const uint32_t have = circ < 4 ? (plo >> (8 * circ)) & 0xFFu : (phi >> (8 * (circ - 4))) & 0xFFu;
                    const uint32_t rank = have + (uint32_t)__popc(peers & ltMask);
                    if ((int)rank < P) list[(size_t)(circ * P + (int)rank) * n + ip] = j;
                }
                const uint32_t incLo = (acc && circ < 4) ? 1u << (8 * circ) : 0u;
                const uint32_t incHi = (acc && circ >= 4) ? 1u << (8 * (circ - 4)) : 0u;
                const uint32_t sLo = __reduce_add_sync(kFull, incLo), sHi = __reduce_add_sync(kFull, incHi);
                if (lane == pl) {  // bytes stay below 256 (<= 64 + 32), then saturate at perCircle
                    cntLo = __vminu4(plo + sLo, capP);
                    cntHi = __vminu4(phi + sHi, capP);
                }
            }
        }
    }
    if (!valid) return;
    const uint64_t cnt = (uint64_t)cntLo | ((uint64_t)cntHi << 32);
    int total = 0;
    uint64_t mt = 0;
    for (int k = 0; k < C; ++k) {
        total += (int)byte_of(cnt, k);
        mt |= (uint64_t)byte_of(cnt, k) << (7 * k);
    }
    mt |= (uint64_t)(c.complete ? C : circles_kept(cnt, C, total, 0.6f)) << 56;
    mt |= (uint64_t)(c.complete ? C : circles_kept(cnt, C, total, 0.5f)) << 60;
    meta[i] = make_uint2((uint32_t)mt, (uint32_t)(mt >> 32));
}

// ------------------------------------------------- balanced thread map --
// The block's particles handed to its threads in decreasing order of their
// friend count, so that the lanes of a warp walk lists of similar length;
// a particle's result does not depend on which thread computes it.  Counting
// sort in shared memory over the kept-circle count (saturated at 255), ties
// in any order.  Every thread of the block must call it (it synchronises);
// returns the particle index, or -1 for threads beyond the block's particles.
__device__ __forceinline__ int balanced_particle(const uint2* __restrict__ meta, int n, bool densityPass, int tile) {
    __shared__ uint32_t bins[256];
    __shared__ int order[kMaxBlock];
    const int t = threadIdx.x;
    const int i = tile * blockDim.x + t;
    for (int k = t; k < 256; k += blockDim.x) bins[k] = 0u;
    __syncthreads();
    int key = -1;
    if (i < n) {
        const uint64_t mt = load_meta(meta, i);
        const int kept = densityPass ? kept_density(mt) : kept_other(mt);
        int tot = 0;
        for (int c = 0; c < kept; ++c) tot += (int)circle_count(mt, c);
        key = 255 - min(tot, 255);
        atomicAdd(&bins[key], 1u);
    }
    __syncthreads();
    if (t < 32) {  // exclusive scan of the 256 bins: 8 per lane
        uint32_t v[8], s = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) { v[k] = bins[8 * t + k]; s += v[k]; }
        uint32_t incl = s;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (t >= d) incl += u;
        }
        uint32_t run = incl - s;
#pragma unroll
        for (int k = 0; k < 8; ++k) { bins[8 * t + k] = run; run += v[k]; }
    }
    __syncthreads();
    if (key >= 0) order[atomicAdd(&bins[key], 1u)] = i;
    __syncthreads();
    const int valid = min(n - tile * (int)blockDim.x, (int)blockDim.x);
    return t < valid ? order[t] : -1;
}

// ---------------------------------------------------- tiles of a launch --
// A launch covers `tiles` tiles of blockDim particles.  With tiles == 0, one
// block per tile (tile = blockIdx.x).  Otherwise a persistent grid of at
// most the resident blocks takes the tiles in order from counter[0], one
// atomic per tile, so busy SMs take fewer tiles; no block waits on another.
// The last block to find the tiles exhausted resets counter[0] and
// counter[1] to 0 for the next launch on the stream.  Every thread of a
// block runs every tile the block takes (the balanced thread map
// synchronises).
template <typename F>
__device__ __forceinline__ void for_tiles(int tiles, int* counter, F body) {
    if (tiles == 0) {
        body((int)blockIdx.x);
        return;
    }
    __shared__ int nextTile;
    while (true) {
        if (threadIdx.x == 0) nextTile = atomicAdd(&counter[0], 1);
        __syncthreads();
        const int t = nextTile;
        __syncthreads();
        if (t >= tiles) break;
        body(t);
    }
    if (threadIdx.x == 0 && atomicAdd(&counter[1], 1) == (int)gridDim.x - 1) {
        counter[0] = 0;
        counter[1] = 0;
    }
}

// -------------------------------------------------------------- scaling --
// Relaxed variants (R = true, relaxedMath): per pair one reciprocal square
// root w = 1/|r| replaces sqrt(r^2) and the divisions by |r|, and sums are
// fused multiply-adds: the reference's kernels as its own
// -cl-fast-relaxed-math -cl-mad-enable build may evaluate them.
// Spiky gradient magnitude over |r|: (h - |r|)^2 / |r| with |r| = r^2 w.
__device__ __forceinline__ float spiky_over_r(const DevConsts& c, float r2, float& w) {
    w = rsqrtf(r2);
    const float hr = fmaf(-r2, w, c.h);
    return hr * hr * w;
}

// compute_scaling.cl:27-112 followed by pack_data.cl (w = lambda).  Q: the
// exact quotients by |r| through one reciprocal (quotient_rn).
template <bool R, bool B, int W, bool Q>
__device__ __forceinline__ void compute_scaling_body(const DevConsts& c, const float4* __restrict__ pred,
                                                     float4* __restrict__ predPacked, float* __restrict__ density,
                                                     const uint32_t* __restrict__ list, const uint2* __restrict__ meta,
                                                     const uint32_t* __restrict__ flatIn, uint32_t* __restrict__ flatOut,
                                                     int i, const float4 pi, uint64_t mt) {
    const int n = c.n;
    // complete neighbour sets count the particle itself first: d = h^2 - 0
    float ds = c.complete ? c.h2 * c.h2 * c.h2 : 0.0f, gsk = 0.0f, gx = 0.0f, gy = 0.0f, gz = 0.0f;
    constexpr int U = 4;  // friends in flight: the passes wait on their neighbour gathers (long scoreboard)
    gather_walk<W, U, true>(list, flatIn, flatOut, n, i, FriendRows(mt, kept_density(mt), c.perCircle),
                      [&](uint32_t j) { return __ldg(pred + checked_index(j, (uint32_t)n, c.err, kErrFriendIndex)); }, [&](const float4 pj) {
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        if (R) {
            const float r2 = fmaf(rz, rz, fmaf(ry, ry, rx * rx));
            if (in_support(c, r2)) {
                float w;
                const float s = c.gradSpiky * spiky_over_r(c, r2, w);
                const float g0 = s * rx, g1 = s * ry, g2 = s * rz;
                const float d = c.h2 - r2;
                ds = fmaf(d * d, d, ds);
                gsk = fmaf(g2, g2, fmaf(g1, g1, fmaf(g0, g0, gsk)));
                gx += g0;
                gy += g1;
                gz += g2;
            }
        } else {
            const float r2 = dot3(rx, ry, rz, rx, ry, rz);
            if (in_support(c, r2)) {
                float rl, y;
                if (Q) sqrt_recip_rn(r2, rl, y);
                else rl = sqrtf(r2);
                const float hr = c.h - rl;
                const float sc = c.gradSpiky * hr * hr;
                float g0, g1, g2;
                if (Q) {
                    g0 = quotient_rn(sc * rx, rl, y);
                    g1 = quotient_rn(sc * ry, rl, y);
                    g2 = quotient_rn(sc * rz, rl, y);
                } else {
                    g0 = (sc * rx) / rl;
                    g1 = (sc * ry) / rl;
                    g2 = (sc * rz) / rl;
                }
                const float d = c.h2 - r2;
                ds = ds + d * d * d;
                gsk = gsk + dot3(g0, g1, g2, g0, g1, g2);
                gx = gx + g0;
                gy = gy + g1;
                gz = gz + g2;
            }
        }
    });
    ds = ds * c.poly6;
    density[i] = ds;
    gsk = gsk + dot3(gx, gy, gz, gx, gy, gz);
    const float constraint = (ds / c.rho0) - 1.0f;
    const float lambda = -1.0f * constraint / (gsk / c.rho0sq + c.eps);
    predPacked[i] = make_float4(pi.x, pi.y, pi.z, lambda);
}

// The exact recording pass is held to 40 registers (three 512-thread blocks
// per SM): 11 % faster than its natural 60, spills and all.
template <bool R, bool B, int W>
__global__ void __launch_bounds__(kMaxBlock, (!R && W == kWalkRecord) ? 3 : 0)
compute_scaling_kernel(DevConsts c, const float4* __restrict__ pred, float4* __restrict__ predPacked,
                       float* __restrict__ density, const uint32_t* __restrict__ list,
                       const uint2* __restrict__ meta, const uint32_t* __restrict__ flatIn,
                       uint32_t* __restrict__ flatOut, int tiles, int* tileCounter) {
    for_tiles(tiles, tileCounter, [&](int tile) {
        const int i = B ? balanced_particle(meta, c.n, true, tile) : tile * (int)blockDim.x + (int)threadIdx.x;
        if (i < 0 || i >= c.n) return;
        const float4 pi = pred[i];
        const uint64_t mt = load_meta(meta, i);
        // a particle that may hold a friend at an irregular position divides the IEEE way
        if (!R && c.quotients && !quotients_tainted(c, i)) compute_scaling_body<R, B, W, true>(c, pred, predPacked, density, list, meta, flatIn, flatOut, i, pi, mt);
        else compute_scaling_body<R, B, W, false>(c, pred, predPacked, density, list, meta, flatIn, flatOut, i, pi, mt);
    });
}

// ---------------------------------------------------------------- delta --
// compute_delta.cl:54-185 (force planes: identity for an all-zero mask) with
// the optional box clamp on `future`, then update_predicted.cl.  After the
// last iteration w carries the density (pack_data.cl with the density source,
// src/Simulation.cpp:591).
template <bool R, bool B, int W, bool Q>
__device__ __forceinline__ void compute_delta_body(const DevConsts& c, const Batch& b, const float4* __restrict__ pp,
                                                   const float4* __restrict__ posPrev, float4* __restrict__ predOut,
                                                   const float* __restrict__ density, const uint32_t* __restrict__ list,
                                                   const uint2* __restrict__ meta, int lastIteration,
                                                   uint8_t* __restrict__ clampMask, const uint32_t* __restrict__ flatIn,
                                                   int i, const float4 pi, uint64_t mt) {
    const int n = c.n;
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    constexpr int U = 4;  // friends in flight: the passes wait on their neighbour gathers (long scoreboard)
    gather_walk<W, U, true>(list, flatIn, nullptr, n, i, FriendRows(mt, kept_other(mt), c.perCircle),
                      [&](uint32_t j) { return __ldg(pp + checked_index(j, (uint32_t)n, c.err, kErrFriendIndex)); }, [&](const float4 pj) {
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        if (R) {
            const float r2 = fmaf(rz, rz, fmaf(ry, ry, rx * rx));
            if (in_support(c, r2)) {
                float w;
                const float k = spiky_over_r(c, r2, w);
                const float d = c.h2 - r2;
                const float rq = d * d * d * c.invPoly6q;
                const float rq2 = rq * rq;
                const float a = fmaf(c.K * rq2, rq2, pi.w + pj.w) * k;
                sx = fmaf(a, rx, sx);
                sy = fmaf(a, ry, sy);
                sz = fmaf(a, rz, sz);
            }
        } else {
            const float r2 = dot3(rx, ry, rz, rx, ry, rz);
            if (in_support(c, r2)) {
                float rl, y;
                if (Q) sqrt_recip_rn(r2, rl, y);
                else rl = sqrtf(r2);
                const float hr = c.h - rl;
                float g0, g1, g2;
                if (Q) {
                    g0 = quotient_rn(rx, rl, y) * hr * hr;
                    g1 = quotient_rn(ry, rl, y) * hr * hr;
                    g2 = quotient_rn(rz, rl, y) * hr * hr;
                } else {
                    g0 = (rx / rl) * hr * hr;
                    g1 = (ry / rl) * hr * hr;
                    g2 = (rz / rl) * hr * hr;
                }
                const float d = c.h2 - r2;
                const float p6 = d * d * d;
                const float rq = c.quotientPoly6q ? quotient_rn(p6, c.poly6q, c.recipPoly6q) : p6 / c.poly6q;
                const float scorr = c.K * rq * rq * rq * rq;
                const float a = pi.w + pj.w + scorr;
                sx = sx + a * g0;
                sy = sy + a * g1;
                sz = sz + a * g2;
            }
        }
    });
    float fx, fy, fz;
    if (R) {
        fx = fmaf(c.dpScale, sx, pi.x);
        fy = fmaf(c.dpScale, sy, pi.y);
        fz = fmaf(c.dpScale, sz, pi.z);
    } else {
        fx = pi.x + (c.negGradSpiky * sx) / c.rho0;
        fy = pi.y + (c.negGradSpiky * sy) / c.rho0;
        fz = pi.z + (c.negGradSpiky * sz) / c.rho0;
    }
    if (c.nquads > 0) {  // force planes, in order (compute_delta.cl:157-182)
        const float4 prev = posPrev[i];
        const float edge = plane_edge_offset(c, fx, fy, fz);
        for (int q = 0; q < c.nquads; ++q) bounce_point_quad(c, c.quads[q], prev.x, prev.y, prev.z, fx, fy, fz, edge);
    }
    if (c.clamp) {
        const float* lo = c.lo;
        const float* hi = c.hi;
        if (b.scenes) {
            const SceneParams& sp = b.scenes[b.sceneOf[i]];
            lo = sp.lo;
            hi = sp.hi;
        }
        // the wave generator's moving wall: xMin + wavePos (pbf_set_wave_position)
        const float lx = c.wave ? lo[0] + *c.wave : lo[0];
        if (clampMask)  // which coordinates the clamp moves: 2 bits per axis, 1 low, 2 high
            clampMask[i] = (uint8_t)((fx < lx ? 1 : (fx > hi[0] ? 2 : 0)) | (fy < lo[1] ? 4 : (fy > hi[1] ? 8 : 0)) |
                                     (fz < lo[2] ? 16 : (fz > hi[2] ? 32 : 0)));
        fx = fx < lx ? lx : (fx > hi[0] ? hi[0] : fx);
        fy = fy < lo[1] ? lo[1] : (fy > hi[1] ? hi[1] : fy);
        fz = fz < lo[2] ? lo[2] : (fz > hi[2] ? hi[2] : fz);
    } else if (clampMask) {
        clampMask[i] = 0;
    }
    const float dx = fx - pi.x, dy = fy - pi.y, dz = fz - pi.z;
    const float4 out = make_float4(pi.x + dx, pi.y + dy, pi.z + dz, lastIteration ? density[i] : pi.w + 0.0f);
    predOut[i] = out;
    if (!R) note_position(c, i, out.x, out.y, out.z);
}

// The exact position pass is held to 40 registers (from 46): 1.3 % faster.
template <bool R, bool B, int W>
__global__ void __launch_bounds__(kMaxBlock, R ? 0 : 3)
compute_delta_kernel(DevConsts c, Batch b, const float4* __restrict__ pp, const float4* __restrict__ posPrev,
                     float4* __restrict__ predOut, const float* __restrict__ density, const uint32_t* __restrict__ list,
                     const uint2* __restrict__ meta, int lastIteration, uint8_t* __restrict__ clampMask,
                     const uint32_t* __restrict__ flatIn, int tiles, int* tileCounter) {
    for_tiles(tiles, tileCounter, [&](int tile) {
        const int i = B ? balanced_particle(meta, c.n, false, tile) : tile * (int)blockDim.x + (int)threadIdx.x;
        if (i < 0 || i >= c.n) return;
        const float4 pi = pp[i];
        const uint64_t mt = load_meta(meta, i);
        // a particle that may hold a friend at an irregular position divides the IEEE way
        if (!R && c.quotients && !quotients_tainted(c, i)) compute_delta_body<R, B, W, true>(c, b, pp, posPrev, predOut, density, list, meta, lastIteration, clampMask, flatIn, i, pi, mt);
        else compute_delta_body<R, B, W, false>(c, b, pp, posPrev, predOut, density, list, meta, lastIteration, clampMask, flatIn, i, pi, mt);
    });
}

// ----------------------------------------------------------- velocities --
// update_velocities.cl:11-14 (the GL texture write is dropped).
// Also moves the sorted particle ids back to their fixed buffer.
__global__ void update_velocities_kernel(DevConsts c, const float4* __restrict__ pred,
                                         const float4* __restrict__ posIn, float4* __restrict__ posOut,
                                         float4* __restrict__ vel, const uint32_t* __restrict__ idsIn,
                                         uint32_t* __restrict__ idsOut) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    if (idsIn) idsOut[i] = idsIn[i];
    const float4 p = pred[i], q = posIn[i];
    float4 v = vel[i];
    v.x = (p.x - q.x) / c.dt;
    v.y = (p.y - q.y) / c.dt;
    v.z = (p.z - q.z) / c.dt;
    vel[i] = v;
    posOut[i] = make_float4(p.x, p.y, p.z, sqrtf(dot3(v.x, v.y, v.z, v.x, v.y, v.z)));
}

// apply_viscosity.cl:12-86, every neighbour read from the pre-pass
// velocities (Jacobi).  omega.w receives |omega| (sqrt of its dot product, as
// apply_vorticity.cl:55 forms it for each neighbour), so that the vorticity
// pass reads it instead of recomputing it per pair.
template <bool R, bool B, int W, bool Q>
__device__ __forceinline__ void apply_viscosity_body(const DevConsts& c, const Batch& b, const float4* __restrict__ pred,
                                                     const float4* __restrict__ velIn, float4* __restrict__ velOut,
                                                     float4* __restrict__ omega, const uint32_t* __restrict__ list,
                                                     const uint2* __restrict__ meta, const uint32_t* __restrict__ flatIn,
                                                     int i, const float4 pi, const float4 vi, uint64_t mt) {
    const int n = c.n;
    float vsx = 0.0f, vsy = 0.0f, vsz = 0.0f, ox = 0.0f, oy = 0.0f, oz = 0.0f;
    constexpr int U = 4;  // friends in flight: the passes wait on their neighbour gathers (long scoreboard)
    gather_walk<W, U>(list, flatIn, nullptr, n, i, FriendRows(mt, kept_other(mt), c.perCircle),
                      [&](uint32_t j) { j = checked_index(j, (uint32_t)n, c.err, kErrFriendIndex); return PairRec{__ldg(pred + j), __ldg(velIn + j)}; }, [&](const PairRec& q) {
        const float4 pj = q.a;
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        const float r2 = rx * rx + ry * ry + rz * rz;
        if (in_support(c, r2) && fabsf(pj.w) > 1e-8f) {
            const float4 vj = q.b;
            const float ux = vj.x - vi.x, uy = vj.y - vi.y, uz = vj.z - vi.z;
            const float d = c.h2 - r2;
            if (R) {
                float w;
                const float k = spiky_over_r(c, r2, w);
                const float g0 = k * rx, g1 = k * ry, g2 = k * rz;
                ox += fmaf(uy, g2, -uz * g1);
                oy += fmaf(uz, g0, -ux * g2);
                oz += fmaf(ux, g1, -uy * g0);
                const float d3 = d * d * d;
                vsx = fmaf(ux, d3, vsx);
                vsy = fmaf(uy, d3, vsy);
                vsz = fmaf(uz, d3, vsz);
            } else {
                float rl, y;
                if (Q) sqrt_recip_rn(r2, rl, y);
                else rl = sqrtf(r2);
                const float hr = c.h - rl;
                float g0, g1, g2;
                if (Q) {
                    g0 = quotient_rn(rx, rl, y) * hr * hr;
                    g1 = quotient_rn(ry, rl, y) * hr * hr;
                    g2 = quotient_rn(rz, rl, y) * hr * hr;
                } else {
                    g0 = (rx / rl) * hr * hr;
                    g1 = (ry / rl) * hr * hr;
                    g2 = (rz / rl) * hr * hr;
                }
                ox = ox + (uy * g2 - uz * g1);
                oy = oy + (uz * g0 - ux * g2);
                oz = oz + (ux * g1 - uy * g0);
                const float d3 = d * d * d;
                vsx = vsx + ux * d3;
                vsy = vsy + uy * d3;
                vsz = vsz + uz * d3;
            }
        }
    });
    vsx = vsx * c.poly6;
    vsy = vsy * c.poly6;
    vsz = vsz * c.poly6;
    const float visc = b.scenes ? b.scenes[b.sceneOf[i]].visc : c.visc;
    velOut[i] = make_float4(vi.x + visc * vsx, vi.y + visc * vsy, vi.z + visc * vsz, vi.w + visc * 0.0f);
    const float wx = ox * c.negGradSpiky, wy = oy * c.negGradSpiky, wz = oz * c.negGradSpiky;
    omega[i] = make_float4(wx, wy, wz, sqrtf(dot3(wx, wy, wz, wx, wy, wz)));
}

template <bool R, bool B, int W>
__global__ void __launch_bounds__(kMaxBlock)
apply_viscosity_kernel(DevConsts c, Batch b, const float4* __restrict__ pred, const float4* __restrict__ velIn,
                       float4* __restrict__ velOut, float4* __restrict__ omega,
                       const uint32_t* __restrict__ list, const uint2* __restrict__ meta,
                       const uint32_t* __restrict__ flatIn, int tiles, int* tileCounter) {
    for_tiles(tiles, tileCounter, [&](int tile) {
        const int i = B ? balanced_particle(meta, c.n, false, tile) : tile * (int)blockDim.x + (int)threadIdx.x;
        if (i < 0 || i >= c.n) return;
        const float4 pi = pred[i], vi = velIn[i];
        const uint64_t mt = load_meta(meta, i);
        // a particle that may hold a friend at an irregular position divides the IEEE way
        if (!R && c.quotients && !quotients_tainted(c, i)) apply_viscosity_body<R, B, W, true>(c, b, pred, velIn, velOut, omega, list, meta, flatIn, i, pi, vi, mt);
        else apply_viscosity_body<R, B, W, false>(c, b, pred, velIn, velOut, omega, list, meta, flatIn, i, pi, vi, mt);
    });
}

// apply_vorticity.cl:12-86; |omega_j| is read from omega.w (apply_viscosity).
template <bool R, bool B, int W, bool Q>
__device__ __forceinline__ void apply_vorticity_body(const DevConsts& c, const float4* __restrict__ pred,
                                                     const float4* __restrict__ omega, const float4* __restrict__ velIn,
                                                     float4* __restrict__ velOut, const uint32_t* __restrict__ list,
                                                     const uint2* __restrict__ meta, const uint32_t* __restrict__ flatIn,
                                                     int i, const float4 pi, uint64_t mt) {
    const int n = c.n;
    float ex = 0.0f, ey = 0.0f, ez = 0.0f;
    constexpr int U = 4;  // friends in flight: the passes wait on their neighbour gathers (long scoreboard)
    gather_walk<W, U>(list, flatIn, nullptr, n, i, FriendRows(mt, kept_other(mt), c.perCircle),
                      [&](uint32_t j) { j = checked_index(j, (uint32_t)n, c.err, kErrFriendIndex); return PairRec{__ldg(pred + j), __ldg(omega + j)}; }, [&](const PairRec& q) {
        const float4 pj = q.a;
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        const float r2 = rx * rx + ry * ry + rz * rz;
        if (in_support(c, r2) && fabsf(pj.w) > 1e-8f) {
            const float4 oj = q.b;
            if (R) {
                float w;
                const float k = spiky_over_r(c, r2, w);
                const float o2 = fmaf(oj.z, oj.z, fmaf(oj.y, oj.y, oj.x * oj.x));
                const float s = o2 > 0.0f ? o2 * rsqrtf(o2) * k : 0.0f;
                ex = fmaf(s, rx, ex);
                ey = fmaf(s, ry, ey);
                ez = fmaf(s, rz, ez);
            } else {
                float rl, y;
                if (Q) sqrt_recip_rn(r2, rl, y);
                else rl = sqrtf(r2);
                const float hr = c.h - rl;
                float g0, g1, g2;
                if (Q) {
                    g0 = quotient_rn(rx, rl, y) * hr * hr;
                    g1 = quotient_rn(ry, rl, y) * hr * hr;
                    g2 = quotient_rn(rz, rl, y) * hr * hr;
                } else {
                    g0 = (rx / rl) * hr * hr;
                    g1 = (ry / rl) * hr * hr;
                    g2 = (rz / rl) * hr * hr;
                }
                const float ol = oj.w;  // sqrt(dot(omega_j, omega_j)), formed once by apply_viscosity
                ex = ex + ol * g0;
                ey = ey + ol * g1;
                ez = ez + ol * g2;
            }
        }
    });
    ex = ex * c.negGradSpiky;
    ey = ey * c.negGradSpiky;
    ez = ez * c.negGradSpiky;
    if (R) {
        const float l2 = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
        if (l2 > 0.0f) {
            const float w = rsqrtf(l2);
            ex *= w;
            ey *= w;
            ez *= w;
        }
    } else {
        const float l = sqrtf(dot3(ex, ey, ez, ex, ey, ez));
        if (l > 0.0f) {
            ex = ex / l;
            ey = ey / l;
            ez = ez / l;
        }
    }
    const float4 oi = omega[i];
    const float fx = c.vort * (ey * oi.z - ez * oi.y);
    const float fy = c.vort * (ez * oi.x - ex * oi.z);
    const float fz = c.vort * (ex * oi.y - ey * oi.x);
    const float4 v = velIn[i];
    velOut[i] = make_float4(v.x + fx * c.dt, v.y + fy * c.dt, v.z + fz * c.dt, v.w + 0.0f);
}

template <bool R, bool B, int W>
__global__ void __launch_bounds__(kMaxBlock)
apply_vorticity_kernel(DevConsts c, const float4* __restrict__ pred, const float4* __restrict__ omega,
                       const float4* __restrict__ velIn, float4* __restrict__ velOut,
                       const uint32_t* __restrict__ list, const uint2* __restrict__ meta,
                       const uint32_t* __restrict__ flatIn, int tiles, int* tileCounter, int tileOffset) {
    for_tiles(tiles, tileCounter, [&](int tile) {
        tile += tileOffset;  // a launch over part of the tiles (one block per tile)
        const int i = B ? balanced_particle(meta, c.n, false, tile) : tile * (int)blockDim.x + (int)threadIdx.x;
        if (i < 0 || i >= c.n) return;
        const float4 pi = pred[i];
        const uint64_t mt = load_meta(meta, i);
        // a particle that may hold a friend at an irregular position divides the IEEE way
        if (!R && c.quotients && !quotients_tainted(c, i)) apply_vorticity_body<R, B, W, true>(c, pred, omega, velIn, velOut, list, meta, flatIn, i, pi, mt);
        else apply_vorticity_body<R, B, W, false>(c, pred, omega, velIn, velOut, list, meta, flatIn, i, pi, mt);
    });
}

}  // namespace

// ------------------------------------------------------------- launchers --
void launch_predict_keys(const DevConsts& c, Batch b, const float4* pos, float4* vel, float4* pred, uint32_t* keys,
                         uint32_t* perm, int paused, cudaStream_t s) {
    predict_keys_kernel<<<blocks_for(c.n), kBlock, 0, s>>>(c, b, pos, vel, pred, keys, perm, paused);
}

void launch_compute_keys(const DevConsts& c, Batch b, const float4* pred, uint32_t* keys, uint32_t* perm,
                         cudaStream_t s) {
    compute_keys_kernel<<<blocks_for(c.n), kBlock, 0, s>>>(c, b, pred, keys, perm);
}

void launch_gather_sorted(int n, const uint32_t* perm, const float4* pos, const float4* pred, const uint32_t* ids,
                          float4* posOut, float4* predOut, uint32_t* idsOut, int* err, cudaStream_t s) {
    gather_sorted_kernel<<<blocks_for(n), kBlock, 0, s>>>(n, perm, pos, pred, ids, posOut, predOut, idsOut, err);
}

void launch_update_cells(int n, const uint32_t* keys, uint32_t* cells, uint32_t keyLimit, int* err, cudaStream_t s,
                         uint32_t* cellStart) {
    update_cells_kernel<<<blocks_for(n), kBlock, 0, s>>>(n, keys, cells, keyLimit, err, cellStart);
}

void launch_reset_cells(int n, const uint32_t* keys, uint32_t* cells, uint32_t keyLimit, int* err, cudaStream_t s) {
    reset_cells_kernel<<<blocks_for(n), kBlock, 0, s>>>(n, keys, reinterpret_cast<uint2*>(cells), keyLimit, err);
}

// Grid of a neighbour pass: one block per tile of `block` particles, or
// (persistent) at most as many blocks as the device keeps resident, which
// then take the tiles from a counter (*tiles receives their count; 0 for one
// block per tile).  A launcher's tileCounter (two words, zero between
// launches) selects the persistent grid; NULL, one block per tile.
template <typename K>
unsigned grid_for_tiles(K kernel, int n, int block, bool persistent, int* tiles) {
    const unsigned all = blocks_for(n, block);
    *tiles = 0;
    if (!persistent) return all;  // no tile counter: one block per tile
    static int sms[64] = {};  // per device, filled on first use
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return all;
    if (!sms[dev]) cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    int resident = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kernel, block, 0) != cudaSuccess || resident < 1 ||
        sms[dev] < 1) {
        cudaGetLastError();
        return all;
    }
    const unsigned cap = (unsigned)resident * (unsigned)sms[dev];
    if (all <= cap) return all;
    *tiles = (int)all;
    return cap;
}

bool launch_build_friends(const DevConsts& c, Batch b, const float4* pred, const uint32_t* cells, uint32_t* list,
                          uint32_t* flat, uint2* meta, int* errorWord, int block, int algorithm, cudaStream_t s) {
    const bool pow2 = (c.grid & (c.grid - 1)) == 0;
    const uint32_t keys = c.grid * (uint32_t)(b.scenes ? b.nscenes : 1);
    const uint2* cellPairs = reinterpret_cast<const uint2*>(cells);
    // narrow counters: at most 5 circles of at most 63 friends
    const bool narrow = c.circles <= 5 && c.perCircle <= 63;
    if (algorithm == 2 && pow2 && c.grid >= 64) {  // one block per 4x4x4-cell brick over all scenes
        auto kb = narrow ? build_friends_brick_kernel<4, true> : build_friends_brick_kernel<4, false>;
        kb<<<keys / 64u, BrickShape<4>::threads, 0, s>>>(c, pred, cellPairs, list, meta, errorWord);
        return false;
    }
    if (algorithm == 1) {
        build_friends_warp_kernel<<<blocks_for(c.n, block), block, 0, s>>>(c, b, pred, cellPairs, list, meta, errorWord);
        return false;
    }
    // one block per tile: the tile loop of a persistent grid costs this kernel
    // spilled registers in its candidate loop, and the grid gains nothing
    auto k = narrow ? build_friends_kernel<2, true> : build_friends_kernel<2, false>;
    k<<<blocks_for(c.n, block), block, 0, s>>>(c, b, pred, cellPairs, list, meta, errorWord);
    return false;
}

namespace {
// The kept circles' friends as flat rows, in order, from the circle rows,
// when no density pass records them (zero solver iterations).
__global__ void flatten_friends_kernel(int n, int perCircle, const uint32_t* __restrict__ list,
                                       const uint2* __restrict__ meta, uint32_t* __restrict__ flat) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t mt = load_meta(meta, i);
    FriendRows fr(mt, kept_density(mt), perCircle);
    for (int t = 0; t < fr.total; ++t) flat[(size_t)t * n + i] = list[(size_t)fr.row(t) * n + i];
}
}  // namespace

void launch_flatten_friends(const DevConsts& c, const uint32_t* list, const uint2* meta, uint32_t* flat, cudaStream_t s) {
    flatten_friends_kernel<<<blocks_for(c.n), kBlock, 0, s>>>(c.n, c.perCircle, list, meta, flat);
}

// The first density pass of a substep records the flat rows from the circle
// rows (flatOut); the other passes walk the flat rows (flatIn).
void launch_compute_scaling(const DevConsts& c, const float4* pred, float4* predPacked, float* density,
                            const uint32_t* list, const uint2* meta, const uint32_t* flatIn, uint32_t* flatOut,
                            int block, int balance, int* tileCounter, cudaStream_t s) {
    const bool record = flatOut != nullptr;
    auto pick = [record](auto rec, auto flat) { return record ? rec : flat; };
    auto k = c.relaxed ? (balance ? pick(compute_scaling_kernel<true, true, kWalkRecord>, compute_scaling_kernel<true, true, kWalkFlat>)
                                  : pick(compute_scaling_kernel<true, false, kWalkRecord>, compute_scaling_kernel<true, false, kWalkFlat>))
                       : (balance ? pick(compute_scaling_kernel<false, true, kWalkRecord>, compute_scaling_kernel<false, true, kWalkFlat>)
                                  : pick(compute_scaling_kernel<false, false, kWalkRecord>, compute_scaling_kernel<false, false, kWalkFlat>));
    int tiles = 0;
    const unsigned grid = grid_for_tiles(k, c.n, block, tileCounter != nullptr, &tiles);
    k<<<grid, block, 0, s>>>(c, pred, predPacked, density, list, meta, flatIn, flatOut, tiles, tileCounter);
}

void launch_compute_delta(const DevConsts& c, Batch b, const float4* predPacked, const float4* posPrev,
                          float4* predOut, const float* density, const uint32_t* list, const uint2* meta,
                          int lastIteration, uint8_t* clampMask, const uint32_t* flatIn, int block, int balance,
                          int* tileCounter, cudaStream_t s) {
    auto k = c.relaxed ? (balance ? compute_delta_kernel<true, true, kWalkFlat> : compute_delta_kernel<true, false, kWalkFlat>)
                       : (balance ? compute_delta_kernel<false, true, kWalkFlat> : compute_delta_kernel<false, false, kWalkFlat>);
    int tiles = 0;
    const unsigned grid = grid_for_tiles(k, c.n, block, tileCounter != nullptr, &tiles);
    k<<<grid, block, 0, s>>>(c, b, predPacked, posPrev, predOut, density, list, meta, lastIteration, clampMask, flatIn,
                             tiles, tileCounter);
}

void launch_update_velocities(const DevConsts& c, const float4* pred, const float4* posIn, float4* posOut,
                              float4* vel, const uint32_t* idsIn, uint32_t* idsOut, cudaStream_t s) {
    update_velocities_kernel<<<blocks_for(c.n), kBlock, 0, s>>>(c, pred, posIn, posOut, vel, idsIn, idsOut);
}

void launch_apply_viscosity(const DevConsts& c, Batch b, const float4* pred, const float4* velIn, float4* velOut,
                            float4* omega, const uint32_t* list, const uint2* meta, const uint32_t* flatIn, int block,
                            int balance, int* tileCounter, cudaStream_t s) {
    auto k = c.relaxed ? (balance ? apply_viscosity_kernel<true, true, kWalkFlat> : apply_viscosity_kernel<true, false, kWalkFlat>)
                       : (balance ? apply_viscosity_kernel<false, true, kWalkFlat> : apply_viscosity_kernel<false, false, kWalkFlat>);
    int tiles = 0;
    const unsigned grid = grid_for_tiles(k, c.n, block, tileCounter != nullptr, &tiles);
    k<<<grid, block, 0, s>>>(c, b, pred, velIn, velOut, omega, list, meta, flatIn, tiles, tileCounter);
}

void launch_apply_vorticity(const DevConsts& c, const float4* pred, const float4* omega, const float4* velIn,
                            float4* velOut, const uint32_t* list, const uint2* meta, const uint32_t* flatIn, int block,
                            int balance, int* tileCounter, cudaStream_t s, int firstTile, int tileCount) {
    auto k = c.relaxed ? (balance ? apply_vorticity_kernel<true, true, kWalkFlat> : apply_vorticity_kernel<true, false, kWalkFlat>)
                       : (balance ? apply_vorticity_kernel<false, true, kWalkFlat> : apply_vorticity_kernel<false, false, kWalkFlat>);
    if (tileCount > 0) {  // tiles [firstTile, firstTile + tileCount), one block each
        k<<<(unsigned)tileCount, block, 0, s>>>(c, pred, omega, velIn, velOut, list, meta, flatIn, 0, nullptr, firstTile);
        return;
    }
    int tiles = 0;
    const unsigned grid = grid_for_tiles(k, c.n, block, tileCounter != nullptr, &tiles);
    k<<<grid, block, 0, s>>>(c, pred, omega, velIn, velOut, list, meta, flatIn, tiles, tileCounter, 0);
}

}  // namespace pbf
