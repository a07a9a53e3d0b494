// Test kernels: quotient_rn (the exact passes' division through one
// reciprocal) against IEEE division, on seeded random operands in the range
// the passes use it for, and sqrt_recip_rn (their square root and reciprocal)
// against sqrtf and __frcp_rn on every non-negative float.  Built by
// tests/test_gpu_quotients.py with nvcc and loaded through ctypes; not part
// of the library.
#include <cstdint>

#include "pbf_device.cuh"

namespace {

__device__ __forceinline__ uint32_t mix(uint64_t x) {  // SplitMix64 finaliser, upper half
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return (uint32_t)((x ^ (x >> 31)) >> 32);
}

// A float with a random 23-bit mantissa, a random sign (when `sign`) and an
// exponent drawn uniformly from [elo, ehi].
__device__ __forceinline__ float draw(uint64_t k, int elo, int ehi, bool sign) {
    const uint32_t m = mix(2 * k) & 0x7FFFFFu;
    const uint32_t r = mix(2 * k + 1);
    const int e = elo + (int)(r % (uint32_t)(ehi - elo + 1));
    const uint32_t bits = ((uint32_t)(e + 127) << 23) | m | (sign && (r & 0x80000000u) ? 0x80000000u : 0u);
    return __uint_as_float(bits);
}

// mode 0: b = |r| in [2^-60, 2^10], a in [2^-100, 2^40] with either sign,
//         y = RN(1/b); mode 1: a = (h^2 - r^2)^3 in [2^-99, 2^1], b = the
//         constant poly6q passed in, y = its reciprocal passed in.
__global__ void check_kernel(uint64_t seed, uint64_t count, int mode, float b0, float y0,
                             unsigned long long* mismatches, float* first) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < count; t += stride) {
        const uint64_t k = seed * 0x100000000ull + t;
        float a, b, y;
        if (mode == 0) {
            b = draw(3 * k, -60, 10, false);
            a = draw(3 * k + 1, -100, 40, true);
            y = __frcp_rn(b);
        } else {
            b = b0;
            y = y0;
            a = draw(3 * k + 2, -99, 1, false);
        }
        const float want = a / b;
        const float got = pbf::quotient_rn(a, b, y);
        if (__float_as_uint(want) != __float_as_uint(got)) {
            if (atomicAdd(mismatches, 1ull) == 0ull) {
                first[0] = a;
                first[1] = b;
            }
        }
    }
}

// Every float whose bit pattern lies in [lo, hi): sqrt_recip_rn's |r|
// against sqrtf (mismatches[0]); the r2 whose y differs from
// __frcp_rn(sqrtf(r2)) are counted (mismatches[1]) and listed.
__global__ void sqrt_recip_kernel(uint32_t lo, uint32_t hi, unsigned long long* mismatches, uint32_t* list,
                                  uint32_t cap, float* first) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t b = lo + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; b < hi; b += stride) {
        const float r2 = __uint_as_float((uint32_t)b);
        const float wantRl = sqrtf(r2);
        float rl, y;
        pbf::sqrt_recip_rn(r2, rl, y);
        if (__float_as_uint(rl) != __float_as_uint(wantRl) && atomicAdd(&mismatches[0], 1ull) == 0ull) first[0] = r2;
        if (__float_as_uint(y) != __float_as_uint(__frcp_rn(wantRl))) {
            const unsigned long long k = atomicAdd(&mismatches[1], 1ull);
            if (k < cap) list[k] = (uint32_t)b;
        }
    }
}

// For each listed r2 and every numerator significand a in [1, 2):
// quotient_rn(a, |r|, y) against a / |r| (mismatches[2]).  Quotients scale
// exactly with the numerator's exponent and sign, so this covers every
// numerator in quotient_rn's range.
__global__ void listed_quotient_kernel(const uint32_t* list, uint32_t count, unsigned long long* mismatches,
                                       float* first) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x, total = (uint64_t)count << 23;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total; t += stride) {
        const float r2 = __uint_as_float(list[t >> 23]);
        float rl, y;
        pbf::sqrt_recip_rn(r2, rl, y);
        const float a = __uint_as_float(0x3F800000u | (uint32_t)(t & 0x7FFFFFu));
        if (__float_as_uint(pbf::quotient_rn(a, rl, y)) != __float_as_uint(a / rl) &&
            atomicAdd(&mismatches[2], 1ull) == 0ull)
            first[1] = r2;
    }
}

__global__ void sqrt_recip_at_kernel(float r2, float a, float* out) {
    float rl, y;
    pbf::sqrt_recip_rn(r2, rl, y);
    out[0] = rl;
    out[1] = y;
    out[2] = pbf::quotient_rn(a, rl, y);  // what the passes form from them
    const float want = sqrtf(r2);
    out[3] = a / want;                    // the IEEE quotient
}

}  // namespace

// sqrt_recip_rn at one r2, with the quotient a / |r| formed from it and by
// IEEE division: out = {|r|, y, quotient_rn(a, |r|, y), a / sqrtf(r2)}.
extern "C" int sqrt_recip_at(float r2, float a, float* out) {
    float* d = nullptr;
    if (cudaMalloc(&d, 4 * sizeof(float)) != cudaSuccess) return 1;
    sqrt_recip_at_kernel<<<1, 1>>>(r2, a, d);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaMemcpy(out, d, 4 * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? 0 : 2;
}

// mismatches = {|r| != sqrtf(r2), y != __frcp_rn(|r|), quotients != IEEE
// division over the r2 of the second kind}; first = {first r2 of the first
// kind, first r2 of the third}.  Returns 3 when more than 2^16 r2 have a
// different y (the quotient check would be incomplete).
extern "C" int sqrt_recip_check(uint32_t lo, uint32_t hi, unsigned long long* mismatches, float* first) {
    constexpr uint32_t kCap = 1u << 16;
    unsigned long long* dm = nullptr;
    float* df = nullptr;
    uint32_t* dl = nullptr;
    if (cudaMalloc(&dm, 3 * sizeof(unsigned long long)) != cudaSuccess) return 1;
    if (cudaMalloc(&df, 2 * sizeof(float)) != cudaSuccess) { cudaFree(dm); return 1; }
    if (cudaMalloc(&dl, kCap * sizeof(uint32_t)) != cudaSuccess) { cudaFree(dm); cudaFree(df); return 1; }
    cudaMemset(dm, 0, 3 * sizeof(unsigned long long));
    cudaMemset(df, 0, 2 * sizeof(float));
    sqrt_recip_kernel<<<152 * 8, 256>>>(lo, hi, dm, dl, kCap, df);
    cudaError_t e = cudaDeviceSynchronize();
    unsigned long long listed = 0;
    cudaMemcpy(&listed, dm + 1, sizeof(listed), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && listed <= kCap && listed > 0) {
        listed_quotient_kernel<<<152 * 8, 256>>>(dl, (uint32_t)listed, dm, df);
        e = cudaDeviceSynchronize();
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaMemcpy(mismatches, dm, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    cudaMemcpy(first, df, 2 * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(dm);
    cudaFree(df);
    cudaFree(dl);
    if (e != cudaSuccess) return 2;
    return listed > kCap ? 3 : 0;
}

extern "C" int quotient_check(uint64_t seed, uint64_t count, int mode, float b0, float y0,
                              unsigned long long* mismatches, float* first) {
    unsigned long long* dm = nullptr;
    float* df = nullptr;
    if (cudaMalloc(&dm, sizeof(unsigned long long)) != cudaSuccess) return 1;
    if (cudaMalloc(&df, 2 * sizeof(float)) != cudaSuccess) { cudaFree(dm); return 1; }
    cudaMemset(dm, 0, sizeof(unsigned long long));
    cudaMemset(df, 0, 2 * sizeof(float));
    check_kernel<<<152 * 8, 256>>>(seed, count, mode, b0, y0, dm, df);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaMemcpy(mismatches, dm, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    cudaMemcpy(first, df, 2 * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(dm);
    cudaFree(df);
    return e == cudaSuccess ? 0 : 2;
}
