// Test kernel: quotient_rn (the exact passes' division through one
// reciprocal) against IEEE division, on seeded random operands in the range
// the passes use it for.  Built by tests/test_gpu_quotients.py with nvcc and
// loaded through ctypes; not part of the library.
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

}  // namespace

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
