// pbf_render.cu — the reference's particle renderer as CUDA kernels into
// device images (no graphics API).
//
// The passes follow src/visual/visual.cpp:340-440 (CVisual::renderParticles,
// smooth mode) and its shaders:
//   splat     particles.vs + particles_color.fs: each particle is a sphere
//             impostor of gl_PointSize = widthOfNearPlane * pointSize / w
//             pixels; a fragment's depth is that of the sphere surface; the
//             LEQUAL depth test (visual.cpp:101) keeps the nearest fragment,
//             the last drawn of equal ones.  Here: one 64-bit atomicMin per
//             fragment on (depth bits, ~index), then a resolve pass.
//   visible   vis_scan.cms: every pixel marks the particle its colour names.
//   grid      grid_chain_reset.cms + grid_build.cms: visible particles hashed
//             into 2048 x 2048 buckets.  The shader chains them with atomic
//             exchanges (order left to the hardware); here the chain of a
//             bucket is its particles in decreasing index order, from a
//             stable radix sort by bucket.
//   smooth    fluid_depth_smoothing.fs: two Newton steps of the pixel's point
//             along the camera ray towards the density shell sum (h^2 - r^2)^3
//             = 1; colour = (window depth, normalized gradient).
//   final     fluid_final_render.fs: diffuse + specular lighting with the
//             smoothed gradient as normal.
// Every step is one IEEE FP32 operation in the shaders' order (this file is
// compiled with --fmad=false); the oracle restates the same arithmetic.
// Pixel (i, j) has its centre at (i + 0.5, j + 0.5), row 0 at the bottom.

#include <cuda_runtime.h>
#include <cstdint>

#include "pbf_internal.h"

namespace pbf {
namespace {

constexpr uint32_t kGridBuckets = 2048u * 2048u;  // grid_build.cms: GRID_BUF_SIZE
constexpr uint64_t kEmptyKey = ~0ull;

struct V4 {
    float x, y, z, w;
};

// column-major 4x4 times (x, y, z, w), summed left to right
__device__ __forceinline__ V4 mat_mul(const float* m, float x, float y, float z, float w) {
    V4 r;
    r.x = ((m[0] * x + m[4] * y) + m[8] * z) + m[12] * w;
    r.y = ((m[1] * x + m[5] * y) + m[9] * z) + m[13] * w;
    r.z = ((m[2] * x + m[6] * y) + m[10] * z) + m[14] * w;
    r.w = ((m[3] * x + m[7] * y) + m[11] * z) + m[15] * w;
    return r;
}

__device__ __forceinline__ float dot3f(float ax, float ay, float az, float bx, float by, float bz) {
    return (ax * bx + ay * by) + az * bz;
}

// GLSL max / min / clamp: max(x, y) = x < y ? y : x
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gclamp(float x, float a, float b) { return gmin(gmax(x, a), b); }

// GLSL int(float): truncation; NaN gives 0 and out-of-range values saturate
__device__ __forceinline__ int to_int(float v) { return __float2int_rz(v); }

__device__ __forceinline__ uint32_t expand_bits_i(int xi) {
    uint32_t x = (uint32_t)xi;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

// grid_build.cms calcGridHash: mortonNumber(gridPos) % (2048 * 2048)
__device__ __forceinline__ uint32_t render_hash(int x, int y, int z) {
    const int m = (int)(expand_bits_i(x) | (expand_bits_i(y) << 1) | (expand_bits_i(z) << 2));
    return (uint32_t)(m % (int)kGridBuckets);
}

// One fragment of particle `p` (eye-space centre e, clip w, window centre
// xw, yw, sprite size s) at pixel (i, j): the sphere normal and the window
// depth, or false where particles_color.fs discards it.
struct Frag {
    float nx, ny, nz, depth;
};
__device__ __forceinline__ bool fragment(const PbfCamera& cam, float ex, float ey, float ez, float xw, float yw, float s,
                                         int i, int j, Frag& f) {
    const float pcx = 0.5f + (((float)i + 0.5f) - xw) / s;        // gl_PointCoord.s
    const float pcy = 0.5f - (((float)j + 0.5f) - yw) / s;        // gl_PointCoord.t (upper-left origin)
    f.nx = pcx * 2.0f + -1.0f;
    f.ny = pcy * 2.0f + -1.0f;
    const float mag = f.nx * f.nx + f.ny * f.ny;
    if (mag > 1.0f) return false;
    f.nz = sqrtf(1.0f - mag);
    const V4 c = mat_mul(cam.projection, ex + f.nx * cam.pointSize, ey + f.ny * cam.pointSize,
                         ez + f.nz * cam.pointSize, 1.0f);
    const float ndc = c.z / c.w;
    if (ndc < -1.0f) return false;
    f.depth = ((1.0f * ndc + 0.0f) + 1.0f) / 2.0f;
    return f.depth <= 1.0f;  // LEQUAL against the cleared depth 1.0
}

// particles.vs for particle p: eye position, clip w, window centre and
// sprite size; false when the point is clipped.
__device__ __forceinline__ bool sprite(const PbfCamera& cam, float4 p, float& ex, float& ey, float& ez, float& xw,
                                       float& yw, float& s) {
    const V4 e = mat_mul(cam.modelView, p.x, p.y, p.z, 1.0f);
    const V4 c = mat_mul(cam.projection, e.x, e.y, e.z, e.w);
    if (!(c.w > 0.0f)) return false;
    const float nx = c.x / c.w, ny = c.y / c.w, nz = c.z / c.w;
    if (!(fabsf(nx) <= 1.0f && fabsf(ny) <= 1.0f && fabsf(nz) <= 1.0f)) return false;
    s = cam.widthOfNearPlane * cam.pointSize / c.w;
    s = fminf(fmaxf(s, 1.0f), 1024.0f);
    const float hw = 0.5f * (float)cam.width, hh = 0.5f * (float)cam.height;
    xw = nx * hw + hw;
    yw = ny * hh + hh;
    ex = e.x;
    ey = e.y;
    ez = e.z;
    return true;
}

__global__ void splat_kernel(PbfCamera cam, int n, const float4* __restrict__ pos, unsigned long long* __restrict__ dkey) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float ex, ey, ez, xw, yw, s;
    if (!sprite(cam, pos[p], ex, ey, ez, xw, yw, s)) return;
    const int i0 = max(0, (int)ceilf(xw - s * 0.5f - 0.5f)), i1 = min(cam.width - 1, (int)ceilf(xw + s * 0.5f - 0.5f) - 1);
    const int j0 = max(0, (int)ceilf(yw - s * 0.5f - 0.5f)), j1 = min(cam.height - 1, (int)ceilf(yw + s * 0.5f - 0.5f) - 1);
    for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
            Frag f;
            if (!fragment(cam, ex, ey, ez, xw, yw, s, i, j, f)) continue;
            const unsigned long long key = ((unsigned long long)__float_as_uint(f.depth) << 32) | (0xFFFFFFFFu - (uint32_t)p);
            atomicMin(dkey + (size_t)j * cam.width + i, key);
        }
}

// hsv2rgb of particles_color.fs, mix(a, b, t) = a (1 - t) + b t
__device__ __forceinline__ float hsv_channel(float h, float k, float s, float v) {
    const float x = h + k;
    const float fr = x - floorf(x);
    const float p = fabsf(fr * 6.0f - 3.0f);
    const float q = gclamp(p - 1.0f, 0.0f, 1.0f);
    return v * (1.0f * (1.0f - s) + q * s);
}

__global__ void resolve_kernel(PbfCamera cam, int n, int mode, const float4* __restrict__ pos,
                               const unsigned long long* __restrict__ dkey, float4* __restrict__ splat) {
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= cam.width * cam.height) return;
    const unsigned long long key = dkey[pix];
    if (key == kEmptyKey) {
        splat[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const uint32_t p = 0xFFFFFFFFu - (uint32_t)(key & 0xFFFFFFFFu);
    const float depth = __uint_as_float((uint32_t)(key >> 32));
    if (mode == 0) {
        splat[pix] = make_float4(depth, (float)(int)p, 0.0f, 1.0f);
        return;
    }
    const int i = pix % cam.width, j = pix / cam.width;
    const float4 q = pos[p];
    float ex, ey, ez, xw, yw, s;
    Frag f{};
    sprite(cam, q, ex, ey, ez, xw, yw, s);
    fragment(cam, ex, ey, ez, xw, yw, s, i, j, f);
    const float cosA = gclamp(dot3f(f.nx, f.ny, f.nz, 1.0f, 1.0f, 1.0f), 0.0f, 1.0f);
    float r, g, b;
    if (mode == 1) {
        const float v = q.w / 20.0f;
        r = v;
        g = v;
        b = 1.0f;
    } else {
        const float hue = (float)(int)p / (float)n * 0.7f;
        r = hsv_channel(hue, 1.0f, 0.9f, 0.9f);
        g = hsv_channel(hue, 2.0f / 3.0f, 0.9f, 0.9f);
        b = hsv_channel(hue, 1.0f / 3.0f, 0.9f, 0.9f);
    }
    splat[pix] = make_float4(r * cosA, g * cosA, b * cosA, 1.0f * cosA);
}

__global__ void visible_kernel(int pixels, int n, const float4* __restrict__ splat, uint8_t* __restrict__ vis) {
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= pixels) return;
    const uint32_t x = (uint32_t)(splat[pix].y + 0.5f);
    if (x < (uint32_t)n) vis[x] = 1;
}

__global__ void grid_keys_kernel(int n, float h, const float4* __restrict__ pos, const uint8_t* __restrict__ vis,
                                 uint32_t* __restrict__ keys, uint32_t* __restrict__ perm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    keys[i] = vis[i] ? render_hash(to_int(p.x / h), to_int(p.y / h), to_int(p.z / h)) : kGridBuckets;
    perm[i] = (uint32_t)i;
}

// first / last sorted index of every bucket (0xFFFFFFFF where empty)
__global__ void grid_cells_kernel(int n, const uint32_t* __restrict__ keys, uint32_t* __restrict__ cells) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t key = keys[k];
    if (key >= kGridBuckets) return;
    if (k == 0 || keys[k - 1] != key) cells[2 * (size_t)key] = (uint32_t)k;
    if (k == n - 1 || keys[k + 1] != key) cells[2 * (size_t)key + 1] = (uint32_t)k;
}

// fluid_depth_smoothing.fs SampleDensityAndGradient
__device__ void sample_density(float h, const float4* __restrict__ pos, const uint32_t* __restrict__ perm,
                               const uint32_t* __restrict__ cells, float wx, float wy, float wz, float& density,
                               float& gx, float& gy, float& gz) {
    const float h2 = h * h;
    density = 0.0f;
    gx = gy = gz = 0.0f;
    const int cx = to_int(wx / h), cy = to_int(wy / h), cz = to_int(wz / h);
    for (int iz = -1; iz <= 1; ++iz)
        for (int iy = -1; iy <= 1; ++iy)
            for (int ix = -1; ix <= 1; ++ix) {
                const uint32_t b = render_hash(cx + ix, cy + iy, cz + iz);
                const uint32_t first = cells[2 * (size_t)b];
                if (first == 0xFFFFFFFFu) continue;
                for (int k = (int)cells[2 * (size_t)b + 1]; k >= (int)first; --k) {
                    const float4 pp = pos[perm[k]];
                    const float dx = pp.x - wx, dy = pp.y - wy, dz = pp.z - wz;
                    const float r2 = dot3f(dx, dy, dz, dx, dy, dz);
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
    gx = gx * -6.0f;
    gy = gy * -6.0f;
    gz = gz * -6.0f;
}

// uvToWorld / uvToViewSpace: the point of pixel (i, j) at buffer depth z
__device__ __forceinline__ V4 pixel_world(const PbfCamera& cam, int i, int j, float z) {
    const float nearv = cam.depthRange[0], farv = cam.depthRange[1];
    const float lz = nearv / (farv - z * (farv - nearv)) * farv;
    const float u = (((float)i + 0.5f) / (float)cam.width * 2.0f - 1.0f) * cam.invFocalLen[0];
    const float v = (((float)j + 0.5f) / (float)cam.height * 2.0f - 1.0f) * cam.invFocalLen[1];
    return mat_mul(cam.invModelView, u * lz, v * lz, -lz, 1.0f);
}

__device__ __forceinline__ void normalize3(float& x, float& y, float& z) {
    const float l = sqrtf(dot3f(x, y, z, x, y, z));
    x = x / l;
    y = y / l;
    z = z / l;
}

__global__ void smooth_kernel(PbfCamera cam, float h, const float4* __restrict__ pos, const uint32_t* __restrict__ perm,
                              const uint32_t* __restrict__ cells, const float4* __restrict__ splat,
                              float4* __restrict__ out) {
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= cam.width * cam.height) return;
    const int i = pix % cam.width, j = pix / cam.width;
    const float z = splat[pix].x;
    out[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (z == 1.0f) return;  // the far plane: discard
    const V4 m = pixel_world(cam, i, j, z);
    const float camx = cam.invModelView[12], camy = cam.invModelView[13], camz = cam.invModelView[14];
    float nx = camx - m.x, ny = camy - m.y, nz = camz - m.z;
    normalize3(nx, ny, nz);
    float tp = 0.0f, sx = m.x, sy = m.y, sz = m.z;
    float density, gx = 0.0f, gy = 0.0f, gz = 0.0f;
    for (int it = 0; it < 2; ++it) {
        sample_density(h, pos, perm, cells, sx, sy, sz, density, gx, gy, gz);
        const float dd = density - 1.0f;
        const float ga = dot3f(nx, ny, nz, gx, gy, gz);
        tp += dd / ga;
        sx = m.x + tp * nx;
        sy = m.y + tp * ny;
        sz = m.z + tp * nz;
    }
    const V4 vs = mat_mul(cam.modelView, sx, sy, sz, 1.0f);
    const V4 c = mat_mul(cam.projection, vs.x, vs.y, vs.z, 1.0f);
    const float ndc = c.z / c.w;
    if (ndc < -1.0f) return;
    const float zb = ((1.0f * ndc + 0.0f) + 1.0f) / 2.0f;
    normalize3(gx, gy, gz);
    out[pix] = make_float4(zb, gx, gy, gz);
}

// pow(x, 50) by binary powers (x^32 x^16 x^2); negative and NaN give NaN
__device__ __forceinline__ float pow50(float x) {
    if (!(x >= 0.0f)) return __int_as_float(0x7FC00000);
    const float x2 = x * x, x4 = x2 * x2, x8 = x4 * x4, x16 = x8 * x8, x32 = x16 * x16;
    return (x32 * x16) * x2;
}

__global__ void final_kernel(PbfCamera cam, const float4* __restrict__ smooth, float4* __restrict__ out) {
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= cam.width * cam.height) return;
    const int i = pix % cam.width, j = pix / cam.width;
    out[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    // uvToEye of the pixel and its four neighbours: any at the far plane discards
    const int di[5] = {0, 1, -1, 0, 0}, dj[5] = {0, 0, 0, 1, -1};
    for (int k = 0; k < 5; ++k) {
        const int a = i + di[k], b = j + dj[k];
        const float z = (a >= 0 && a < cam.width && b >= 0 && b < cam.height) ? smooth[(size_t)b * cam.width + a].x : 0.0f;
        if (z == 1.0f) return;
    }
    const float4 s = smooth[pix];
    const float nx = s.y, ny = s.z, nz = s.w;
    const V4 w = pixel_world(cam, i, j, s.x);
    float ex = cam.invModelView[12] - w.x, ey = cam.invModelView[13] - w.y, ez = cam.invModelView[14] - w.z;
    normalize3(ex, ey, ez);
    const float lx = 0.0f, ly = 1.0f, lz = 0.0f;  // normalize(vec3(0, 1, 0))
    float hx = lx + ex, hy = ly + ey, hz = lz + ez;
    normalize3(hx, hy, hz);
    const float diff = gclamp(dot3f(lx, ly, lz, nx, ny, nz), 0.0f, 1.0f);
    const float spec = gmax(0.0f, pow50(dot3f(nx, ny, nz, hx, hy, hz)));
    out[pix] = make_float4(0.0f * diff + 1.0f * spec, 0.0f * diff + 1.0f * spec, 0.5f * diff + 1.0f * spec, 1.0f);
}

inline unsigned blocks(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

int render_launches(int mode, const SortPlan& plan) {
    return mode == 0 ? 6 + radix_sort_launches(plan) : 2;
}

void render_frame(const PbfCamera& cam, int mode, int n, float h, const float4* pos, RenderBuffers& rb,
                  cudaStream_t s) {
    const size_t pixels = (size_t)cam.width * cam.height;
    cudaMemsetAsync(rb.dkey, 0xFF, 8 * pixels, s);
    splat_kernel<<<blocks(n, 128), 128, 0, s>>>(cam, n, pos, rb.dkey);
    resolve_kernel<<<blocks(pixels, 256), 256, 0, s>>>(cam, n, mode, pos, rb.dkey, rb.splat);
    if (mode != 0) {
        cudaMemcpyAsync(rb.out, rb.splat, 16 * pixels, cudaMemcpyDeviceToDevice, s);
        return;
    }
    cudaMemsetAsync(rb.vis, 0, (size_t)n, s);
    visible_kernel<<<blocks(pixels, 256), 256, 0, s>>>((int)pixels, n, rb.splat, rb.vis);
    grid_keys_kernel<<<blocks(n, 256), 256, 0, s>>>(n, h, pos, rb.vis, rb.keys[0], rb.perm[0]);
    const int cur = launch_radix_sort(rb.plan, rb.keys, rb.perm, rb.hist, nullptr, nullptr, nullptr, nullptr, s);
    cudaMemsetAsync(rb.cells, 0xFF, 8 * (size_t)kGridBuckets, s);
    grid_cells_kernel<<<blocks(n, 256), 256, 0, s>>>(n, rb.keys[cur], rb.cells);
    smooth_kernel<<<blocks(pixels, 128), 128, 0, s>>>(cam, h, pos, rb.perm[cur], rb.cells, rb.splat, rb.smooth);
    final_kernel<<<blocks(pixels, 256), 256, 0, s>>>(cam, rb.smooth, rb.out);
}

size_t render_grid_words() { return 2 * (size_t)kGridBuckets; }

}  // namespace pbf
