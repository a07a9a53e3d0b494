// pbf_adjoint.cu — reverse accumulation through one substep, over a fixed
// neighbour structure (the substep's sort permutation, friend lists and box
// clamp decisions are constants of the derivative).
//
// With r = p_i - p_j, k(r) = (h - |r|)^2 r/|r| and W(r) = (h^2 - |r|^2)^3, the
// forward of a substep is (compute_scaling.cl, compute_delta.cl,
// update_velocities.cl, apply_viscosity.cl, apply_vorticity.cl):
//   lambda_i = -(rho_i/rho0 - 1) / (D_i/rho0^2 + eps),
//     rho_i = POLY6 sum W,  D_i = sum |G k|^2 + |sum G k|^2
//   p'_i = clamp(p_i - (G/rho0) sum (lambda_i + lambda_j + K (W/Wq)^4) k)
//   v2 = (p^I - x)/dt,  v3 = v2 + c POLY6 sum (v2_j - v2_i) W,
//   omega_i = -G sum (v2_j - v2_i) x k,  eta_i = -G sum |omega_j| k,
//   v4 = v3 + dt eps_v (eta/|eta|) x omega_i.
// Each kernel below walks the same friends as its forward kernel (the flat
// rows the substep recorded: friend t of particle i at list[t * N + i]) and
// scatters neighbour terms with atomics, so the sums are not ordered: these
// are FP32 gradients, not bit-reproducible ones.  The derivation is the same
// as the FP64 adjoint the tests compare against.

#include <cuda_runtime.h>
#include <cstdint>

#include "pbf_device.cuh"
#include "pbf_internal.h"

namespace pbf {
namespace {

constexpr int kAdjBlock = 128;

struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3(const float4& a) { return {a.x, a.y, a.z}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator*(float s, F3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 cross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ float len(F3 a) { return sqrtf(dot(a, a)); }

__device__ __forceinline__ void add3(float4* a, F3 v) { atomicAdd(a, make_float4(v.x, v.y, v.z, 0.0f)); }

// A friend's records as the walks below load them, four friends in flight
// (gather_flat): its index and one or two float4 records.
struct Friend1 {
    uint32_t j;
    float4 a;
};
struct Friend2 {
    uint32_t j;
    float4 a, b;
};
constexpr int kAdjU = 4;

// k(r) and the adjoint of its argument: d/dr [k . kb] = f kb + f'(|r|)(kb.r) r/|r|
// with f = (h-|r|)^2/|r|, f' = -(h-|r|)(h+|r|)/|r|^2.  y is 1/|r| within an
// ulp (sqrt_recip_rn): the adjoint is an FP32 gradient, not a bit-exact one.
__device__ __forceinline__ F3 kvec(F3 r, float rl, float y, float h) {
    const float hr = h - rl;
    return (hr * hr * y) * r;
}
__device__ __forceinline__ F3 kvec_adj(F3 r, float rl, float y, float h, F3 kb) {
    const float hr = h - rl;
    const float f = hr * hr * y;
    const float fp = -hr * (h + rl) * y * y;
    return f * kb + (fp * dot(kb, r) * y) * r;
}
// |r| and 1/|r| of a pair.
__device__ __forceinline__ float pair_length(float r2, float& y) {
    float rl;
    sqrt_recip_rn(r2, rl, y);
    return rl;
}

__device__ __forceinline__ bool xsph_pair(const DevConsts& c, float r2, float rhoj) {
    return in_support(c, r2) && fabsf(rhoj) > 1e-8f;
}

template <typename T> __device__ __forceinline__ T block_sum(T v) {
    __shared__ T part[kAdjBlock / 32];
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, d);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
    __syncthreads();
    T s = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kAdjBlock / 32; ++w) s += part[w];
    return s;
}

// v4 = v3 + dt*vort*(N x omega_i): adjoints of omega (omb) and of p^I (pb).
__global__ void __launch_bounds__(kAdjBlock)
adj_vorticity_kernel(DevConsts c, const float4* __restrict__ pI, const float4* __restrict__ omega,
                     const uint32_t* __restrict__ list, const uint2* __restrict__ meta,
                     const float4* __restrict__ vb, float4* __restrict__ omb, float4* __restrict__ pb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = c.n;
    if (i >= n) return;
    const uint64_t mt = load_meta(meta, i);
    const F3 pi = f3(pI[i]);
    const float G = c.gradSpiky;
    F3 eta = {0.0f, 0.0f, 0.0f};
    FlatFriends f1(mt, kept_other(mt));
    auto loadPO = [&](uint32_t j) {
        j = checked_index(j, (uint32_t)n, c.err, kErrFriendIndex);
        return Friend2{j, pI[j], omega[j]};
    };
    gather_flat<kAdjU>(list, n, i, f1.total, loadPO, [&](const Friend2& f) {
        const F3 r = pi - f3(f.a);
        const float r2 = dot(r, r);
        if (!xsph_pair(c, r2, f.a.w)) return;
        float y;
        const float rl = pair_length(r2, y);
        eta = eta + len(f3(f.b)) * kvec(r, rl, y, c.h);
    });
    eta = -G * eta;
    const float l = len(eta);
    if (!(l > 0.0f)) return;
    const F3 N = (1.0f / l) * eta;
    const F3 ub = (c.vort * c.dt) * f3(vb[i]);
    const F3 oi = f3(omega[i]);
    const F3 Nb = cross(oi, ub);
    add3(&omb[i], cross(ub, N));
    const F3 etab = (1.0f / l) * (Nb - dot(N, Nb) * N);
    FlatFriends f2(mt, kept_other(mt));
    F3 pbi = {0.0f, 0.0f, 0.0f};  // particle i's own terms, added once
    gather_flat<kAdjU>(list, n, i, f2.total, loadPO, [&](const Friend2& f) {
        const F3 r = pi - f3(f.a);
        const float r2 = dot(r, r);
        if (!xsph_pair(c, r2, f.a.w)) return;
        float y;
        const float rl = pair_length(r2, y);
        const F3 k = kvec(r, rl, y, c.h);
        const F3 oj = f3(f.b);
        const float ol = len(oj);
        if (ol > 0.0f) add3(&omb[f.j], (-G * dot(etab, k) / ol) * oj);
        const F3 rb = kvec_adj(r, rl, y, c.h, (-G * ol) * etab);
        pbi = pbi + rb;
        add3(&pb[f.j], -1.0f * rb);
    });
    add3(&pb[i], pbi);
}

// v3 = v2 + c POLY6 sum (v2_j - v2_i) W and omega = -G sum (v2_j - v2_i) x k:
// adjoints of v2 (v2b), p^I (pb) and of the XSPH factor (cbar).
__global__ void __launch_bounds__(kAdjBlock)
adj_viscosity_kernel(DevConsts c, const float4* __restrict__ pI, const float4* __restrict__ v2,
                     const float4* __restrict__ omb, const float4* __restrict__ vb, const uint32_t* __restrict__ list,
                     const uint2* __restrict__ meta, float4* __restrict__ v2b, float4* __restrict__ pb,
                     float* __restrict__ cbar) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = c.n;
    float cacc = 0.0f;
    if (i < n) {
        const uint64_t mt = load_meta(meta, i);
        const F3 pi = f3(pI[i]), v3b = f3(vb[i]), ob = f3(omb[i]), vi = f3(v2[i]);
        const float G = c.gradSpiky;
        F3 v2bi = v3b, pbi = {0.0f, 0.0f, 0.0f};  // particle i's own terms, added once
        FlatFriends fr(mt, kept_other(mt));
        auto loadPV = [&](uint32_t j) {
            j = checked_index(j, (uint32_t)n, c.err, kErrFriendIndex);
            return Friend2{j, pI[j], v2[j]};
        };
        gather_flat<kAdjU>(list, n, i, fr.total, loadPV, [&](const Friend2& f) {
            const uint32_t j = f.j;
            const F3 r = pi - f3(f.a);
            const float r2 = dot(r, r);
            if (!xsph_pair(c, r2, f.a.w)) return;
            float y;
            const float rl = pair_length(r2, y);
            const F3 u = f3(f.b) - vi;
            const float d = c.h2 - r2;
            const float w = c.poly6 * d * d * d;
            const F3 k = kvec(r, rl, y, c.h);
            cacc += w * dot(v3b, u);
            const F3 ub = (c.visc * w) * v3b + (-G) * cross(k, ob);
            add3(&v2b[j], ub);
            v2bi = v2bi - ub;
            const float Wb = c.visc * c.poly6 * dot(v3b, u);
            const F3 rb = (Wb * -6.0f * d * d) * r + kvec_adj(r, rl, y, c.h, (-G) * cross(ob, u));
            pbi = pbi + rb;
            add3(&pb[j], -1.0f * rb);
        });
        add3(&v2b[i], v2bi);
        add3(&pb[i], pbi);
    }
    const float s = block_sum(cacc);
    if (threadIdx.x == 0 && s != 0.0f) atomicAdd(cbar, s);
}

// v2 = (p^I - x)/dt and x' = p^I.
__global__ void adj_velocity_kernel(DevConsts c, const float4* __restrict__ xb, const float4* __restrict__ v2b,
                                    float4* __restrict__ pb, float4* __restrict__ xsb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const F3 v = f3(v2b[i]);
    const F3 p = f3(pb[i]) + f3(xb[i]) + (1.0f / c.dt) * v;
    pb[i] = make_float4(p.x, p.y, p.z, 0.0f);
    xsb[i] = make_float4(-v.x / c.dt, -v.y / c.dt, -v.z / c.dt, 0.0f);
}

// p^{t+1} = clamp(p^t + delta(p^t, lambda^t)): adjoints of p^t (pbt) and
// lambda^t (lb) from that of p^{t+1} (pbn).  q = (p^t, lambda^t).
__global__ void __launch_bounds__(kAdjBlock)
adj_delta_kernel(DevConsts c, const float4* __restrict__ q, const uint8_t* __restrict__ mask,
                 const float4* __restrict__ pbn, const uint32_t* __restrict__ list, const uint2* __restrict__ meta,
                 float4* __restrict__ pbt, float* __restrict__ lb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = c.n;
    if (i >= n) return;
    F3 fb = f3(pbn[i]);
    if (mask) {
        const uint8_t m = mask[i];
        if (m & 3) fb.x = 0.0f;
        if (m & 12) fb.y = 0.0f;
        if (m & 48) fb.z = 0.0f;
    }
    F3 pbi = fb;  // particle i's own terms, added once
    float lbi = 0.0f;
    const float4 qi = q[i];
    const F3 pi = f3(qi);
    const float a0 = -c.gradSpiky / c.rho0;
    const uint64_t mt = load_meta(meta, i);
    FlatFriends fr(mt, kept_other(mt));
    auto loadQ = [&](uint32_t j) {
        j = checked_index(j, (uint32_t)n, c.err, kErrFriendIndex);
        return Friend1{j, q[j]};
    };
    gather_flat<kAdjU>(list, n, i, fr.total, loadQ, [&](const Friend1& f) {
        const uint32_t j = f.j;
        const float4 qj = f.a;
        const F3 r = pi - f3(qj);
        const float r2 = dot(r, r);
        if (!in_support(c, r2)) return;
        float y;
        const float rl = pair_length(r2, y);
        const float d = c.h2 - r2;
        const float rq = d * d * d / c.poly6q;
        const float a = qi.w + qj.w + c.K * rq * rq * rq * rq;
        const F3 k = kvec(r, rl, y, c.h);
        const float ab = a0 * dot(fb, k);
        lbi += ab;
        atomicAdd(&lb[j], ab);
        const float sW = ab * 4.0f * c.K * rq * rq * rq / c.poly6q;
        const F3 rb = (sW * -6.0f * d * d) * r + kvec_adj(r, rl, y, c.h, (a0 * a) * fb);
        pbi = pbi + rb;
        add3(&pbt[j], -1.0f * rb);
    });
    atomicAdd(&lb[i], lbi);
    add3(&pbt[i], pbi);
}

// lambda^t from p^t: adjoint of p^t (pbt) from that of lambda^t (lb).
__global__ void __launch_bounds__(kAdjBlock)
adj_scaling_kernel(DevConsts c, const float4* __restrict__ q, const float* __restrict__ lb,
                   const uint32_t* __restrict__ list, const uint2* __restrict__ meta, float4* __restrict__ pbt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = c.n;
    if (i >= n) return;
    const float lbar = lb[i];
    if (lbar == 0.0f) return;
    const F3 pi = f3(q[i]);
    const float G = c.gradSpiky;
    const uint64_t mt = load_meta(meta, i);
    float ds = 0.0f, gsk = 0.0f;
    F3 S = {0.0f, 0.0f, 0.0f};
    FlatFriends f1(mt, kept_density(mt));
    auto loadQ = [&](uint32_t j) {
        j = checked_index(j, (uint32_t)n, c.err, kErrFriendIndex);
        return Friend1{j, q[j]};
    };
    gather_flat<kAdjU>(list, n, i, f1.total, loadQ, [&](const Friend1& f) {
        const F3 r = pi - f3(f.a);
        const float r2 = dot(r, r);
        if (!in_support(c, r2)) return;
        float y;
        const float rl = pair_length(r2, y);
        const F3 g = G * kvec(r, rl, y, c.h);
        const float d = c.h2 - r2;
        ds += d * d * d;
        gsk += dot(g, g);
        S = S + g;
    });
    const float rho = ds * c.poly6, D = gsk + dot(S, S);
    const float den = D / c.rho0sq + c.eps, Cc = rho / c.rho0 - 1.0f;
    const float rhob = (-lbar / den) / c.rho0;
    const float Db = lbar * Cc / (den * den) / c.rho0sq;
    FlatFriends f2(mt, kept_density(mt));
    F3 pbi = {0.0f, 0.0f, 0.0f};  // particle i's own terms, added once
    gather_flat<kAdjU>(list, n, i, f2.total, loadQ, [&](const Friend1& f) {
        const uint32_t j = f.j;
        const F3 r = pi - f3(f.a);
        const float r2 = dot(r, r);
        if (!in_support(c, r2)) return;
        float y;
        const float rl = pair_length(r2, y);
        const float d = c.h2 - r2;
        const F3 g = G * kvec(r, rl, y, c.h);
        const F3 rb = (rhob * c.poly6 * -6.0f * d * d) * r + kvec_adj(r, rl, y, c.h, (G * 2.0f * Db) * (g + S));
        pbi = pbi + rb;
        add3(&pbt[j], -1.0f * rb);
    });
    add3(&pbt[i], pbi);
}

// Undo the sort and the prediction p0 = x + dt (v + dt g): adjoints of the
// substep's inputs x, v (previous order) and of g.
__global__ void __launch_bounds__(kAdjBlock)
adj_unsort_predict_kernel(DevConsts c, const uint32_t* __restrict__ perm, const float4* __restrict__ xsb,
                          const float4* __restrict__ pb0, float4* __restrict__ xo, float4* __restrict__ vo,
                          float* __restrict__ gbar) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    F3 g = {0.0f, 0.0f, 0.0f};
    if (k < c.n) {
        const uint32_t i = perm[k];
        const F3 p = f3(pb0[k]);
        const F3 x = f3(xsb[k]) + p;
        xo[i] = make_float4(x.x, x.y, x.z, 0.0f);
        vo[i] = make_float4(c.dt * p.x, c.dt * p.y, c.dt * p.z, 0.0f);
        g = (c.dt * c.dt) * p;
    }
    const float gx = block_sum(g.x);
    __syncthreads();
    const float gy = block_sum(g.y);
    __syncthreads();
    const float gz = block_sum(g.z);
    if (threadIdx.x == 0) {
        atomicAdd(&gbar[0], gx);
        atomicAdd(&gbar[1], gy);
        atomicAdd(&gbar[2], gz);
    }
}

// xb[k] = src[ids[k]] (to the current order) or dst[ids[k]] = xb[k] (back).
__global__ void scatter_by_id_kernel(int n, const uint32_t* __restrict__ ids, const float4* __restrict__ byId,
                                     float4* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = byId[ids[k]];
}
__global__ void gather_to_id_kernel(int n, const uint32_t* __restrict__ ids, const float4* __restrict__ in,
                                    float4* __restrict__ byId) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) byId[ids[k]] = in[k];
}

inline unsigned grid_for(int n) { return (unsigned)((n + kAdjBlock - 1) / kAdjBlock); }

}  // namespace

void adjoint_substep(const DevConsts& c, const AdjointTape& tp, AdjointBuffers& ab, cudaStream_t s) {
    const int n = c.n;
    const size_t v4 = 16 * (size_t)n;
    cudaMemsetAsync(ab.omb, 0, v4, s);
    cudaMemsetAsync(ab.pb, 0, v4, s);
    cudaMemsetAsync(ab.v2b, 0, v4, s);
    adj_vorticity_kernel<<<grid_for(n), kAdjBlock, 0, s>>>(c, tp.pI, tp.omega, tp.list, tp.meta, ab.vb, ab.omb, ab.pb);
    adj_viscosity_kernel<<<grid_for(n), kAdjBlock, 0, s>>>(c, tp.pI, tp.v2, ab.omb, ab.vb, tp.list, tp.meta, ab.v2b,
                                                           ab.pb, ab.scalars);
    adj_velocity_kernel<<<grid_for(n), kAdjBlock, 0, s>>>(c, ab.xb, ab.v2b, ab.pb, ab.xsb);
    for (int t = tp.iterations - 1; t >= 0; --t) {
        cudaMemsetAsync(ab.pbt, 0, v4, s);
        cudaMemsetAsync(ab.lb, 0, 4 * (size_t)n, s);
        adj_delta_kernel<<<grid_for(n), kAdjBlock, 0, s>>>(c, tp.q[t], tp.mask ? tp.mask + (size_t)t * n : nullptr,
                                                           ab.pb, tp.list, tp.meta, ab.pbt, ab.lb);
        adj_scaling_kernel<<<grid_for(n), kAdjBlock, 0, s>>>(c, tp.q[t], ab.lb, tp.list, tp.meta, ab.pbt);
        float4* tmp = ab.pb;
        ab.pb = ab.pbt;
        ab.pbt = tmp;
    }
    adj_unsort_predict_kernel<<<grid_for(n), kAdjBlock, 0, s>>>(c, tp.perm, ab.xsb, ab.pb, ab.xo, ab.vo,
                                                                ab.scalars + 1);
    float4* t1 = ab.xb;
    ab.xb = ab.xo;
    ab.xo = t1;
    float4* t2 = ab.vb;
    ab.vb = ab.vo;
    ab.vo = t2;
}

int adjoint_launches(int iterations) { return 4 + 2 * iterations; }

void scatter_by_id(int n, const uint32_t* ids, const float4* byId, float4* out, cudaStream_t s) {
    scatter_by_id_kernel<<<grid_for(n), kAdjBlock, 0, s>>>(n, ids, byId, out);
}

void gather_to_id(int n, const uint32_t* ids, const float4* in, float4* byId, cudaStream_t s) {
    gather_to_id_kernel<<<grid_for(n), kAdjBlock, 0, s>>>(n, ids, in, byId);
}

}  // namespace pbf
