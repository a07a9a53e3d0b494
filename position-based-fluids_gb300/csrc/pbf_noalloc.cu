// pbf_noalloc.cu — the key / sort / cell-table stage for callers that may
// not allocate device memory.
//
// Some hosts reserve all of their device memory when they start and forbid
// any allocation afterwards: a real-time frame loop in which a cudaMalloc
// could stall or fragment the heap, or an engine that owns the GPU's memory
// budget and hands plug-ins only the buffers it allocated itself.  Such a
// caller can still run the sort stage through pbf_sort_state_noalloc, which
// takes device buffers for its inputs and outputs and keeps its working
// memory in the file-scope array below instead of allocating it.
//
// The array is a fixed-size `__device__` object: every GPU that loads this
// library holds it (PBF_NOALLOC_SCRATCH_BYTES) until the process exits, and
// every call on that GPU shares it.  Host code cannot use the array's name
// as a device address, so the first call on each device looks the address up
// with cudaGetSymbolAddress while that device is current and keeps it.

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "pbf_capi.h"
#include "pbf_internal.h"

namespace {

constexpr size_t kMaxKeys = PBF_NOALLOC_MAX_KEYS;
constexpr size_t kTileKeys = 2048;  // keys per radix-sort tile from 2^18 to 2^21 keys; the 1024-key tiles of
                                    // smaller sorts (pbf_sort.cu) need fewer histograms (2^18 / 1024 = 256)
constexpr size_t kHistWords = 256 * (kMaxKeys / kTileKeys) + 256;  // a 256-bin histogram per tile + digit totals
constexpr size_t kScratchWords = 2 * kMaxKeys + kHistWords;   // keys + permutation ping-pong, histograms
static_assert(kScratchWords * 4 == PBF_NOALLOC_SCRATCH_BYTES, "scratch size stated in pbf_capi.h");

// Working memory of every pbf_sort_state_noalloc call on a device:
//   [0, kMaxKeys)            keys of the odd sort passes
//   [kMaxKeys, 2*kMaxKeys)   permutation of the odd sort passes
//   [2*kMaxKeys, ...)        per-tile digit histograms
// Every word a call reads is written by that call before the read, so the
// contents left by an earlier call never need clearing.
static __device__ __align__(256) uint32_t g_sortScratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_lock;
uint32_t* g_scratch[kMaxDevices] = {};

// Device address of g_sortScratch on the current device, looked up once.
int scratch_on_current_device(uint32_t** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return pbf::fail(nullptr, PBF_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return pbf::fail(nullptr, PBF_ERR_INVALID, "device ordinal beyond 63");
    std::lock_guard<std::mutex> guard(g_lock);
    if (!g_scratch[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_sortScratch);
        if (e != cudaSuccess || !p)
            return pbf::fail(nullptr, PBF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratch[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch[dev];
    return PBF_OK;
}

// PBF_OK when `ptr` is device (or managed) memory of device `dev`; a caller's
// host pointer or a buffer of another GPU is refused here instead of faulting
// the kernels.  `what` names the argument in the message.
int check_device_pointer(const void* ptr, int dev, const char* what) {
    cudaPointerAttributes a{};
    const cudaError_t e = cudaPointerGetAttributes(&a, ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();  // an unregistered address reports an error on some runtimes; it is this call's
        return pbf::fail(nullptr, PBF_ERR_INVALID, std::string("pbf_sort_state_noalloc: ") + what +
                                                       " is not a device address (" + cudaGetErrorString(e) + ")");
    }
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)
        return pbf::fail(nullptr, PBF_ERR_INVALID,
                         std::string("pbf_sort_state_noalloc: ") + what + " is not device memory");
    if (a.type == cudaMemoryTypeDevice && a.device != dev)
        return pbf::fail(nullptr, PBF_ERR_INVALID, std::string("pbf_sort_state_noalloc: ") + what + " is on device " +
                                                       std::to_string(a.device) + ", not the current device " +
                                                       std::to_string(dev));
    return PBF_OK;
}

}  // namespace

extern "C" int pbf_sort_state_noalloc(const PbfParameters* params, const float* d_pred, uint32_t* d_keys,
                                      uint32_t* d_perm, uint32_t* d_cells, void* stream) {
    if (!params || !d_pred || !d_keys || !d_perm)
        return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_sort_state_noalloc: NULL argument");
    const uint32_t n = params->particleCount;
    if (n < 1 || n > kMaxKeys)
        return pbf::fail(nullptr, PBF_ERR_INVALID,
                         "pbf_sort_state_noalloc: particleCount " + std::to_string(n) +
                             " is outside [1, " + std::to_string(kMaxKeys) + "], the size of its fixed scratch array");
    if (params->gridBufSize < 1 || params->gridBufSize > (1u << 30))
        return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_sort_state_noalloc: gridBufSize must be in [1, 2^30]");
    if (!(params->h > 0.0f)) return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_sort_state_noalloc: SmoothLen must be positive");
    // d_pred is read as float4 records, the others as 32-bit words
    if (reinterpret_cast<uintptr_t>(d_pred) % 16 != 0)
        return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_sort_state_noalloc: d_pred is not 16-byte aligned");
    if (reinterpret_cast<uintptr_t>(d_keys) % 4 != 0 || reinterpret_cast<uintptr_t>(d_perm) % 4 != 0 ||
        reinterpret_cast<uintptr_t>(d_cells) % 4 != 0)
        return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_sort_state_noalloc: d_keys, d_perm and d_cells must be 4-byte aligned");
    // An error left pending by the caller's earlier work would be read back
    // below as this call's own; it is reported as the caller's and left set.
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess)
        return pbf::fail(nullptr, PBF_ERR_CUDA, std::string("pbf_sort_state_noalloc: a CUDA error was pending before "
                                                            "the call (nothing enqueued): ") + cudaGetErrorString(e));
    uint32_t* scratch = nullptr;
    int rc = scratch_on_current_device(&scratch);
    if (rc) return rc;
    int dev = -1;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess)
        return pbf::fail(nullptr, PBF_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if ((rc = check_device_pointer(d_pred, dev, "d_pred")) || (rc = check_device_pointer(d_keys, dev, "d_keys")) ||
        (rc = check_device_pointer(d_perm, dev, "d_perm")) || (d_cells && (rc = check_device_pointer(d_cells, dev, "d_cells"))))
        return rc;
    if (stream) {  // a stream of another device would run the kernels there, against this device's scratch address
        int sdev = -1;
        if ((e = cudaStreamGetDevice(static_cast<cudaStream_t>(stream), &sdev)) != cudaSuccess) {
            cudaGetLastError();
            return pbf::fail(nullptr, PBF_ERR_INVALID, std::string("pbf_sort_state_noalloc: stream: ") + cudaGetErrorString(e));
        }
        if (sdev != dev)
            return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_sort_state_noalloc: stream belongs to device " +
                                                           std::to_string(sdev) + ", not the current device " +
                                                           std::to_string(dev));
    }

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const pbf::DevConsts c = pbf::make_consts(*params, (int)n);
    const pbf::SortPlan plan = pbf::make_sort_plan((int)n, params->gridBufSize);
    if (plan.histWords > kHistWords)
        return pbf::fail(nullptr, PBF_ERR_INVALID, "pbf_sort_state_noalloc: histogram exceeds its scratch region");
    uint32_t* keys[2] = {d_keys, scratch};
    uint32_t* perm[2] = {d_perm, scratch + kMaxKeys};
    uint32_t* hist = scratch + 2 * kMaxKeys;

    pbf::launch_compute_keys(c, pbf::Batch{nullptr, nullptr}, reinterpret_cast<const float4*>(d_pred), keys[0], perm[0], s);
    const int r = pbf::launch_radix_sort(plan, keys, perm, hist, nullptr, nullptr, nullptr, nullptr, s);
    if (r == 1) {  // an odd number of passes left the result in the scratch half
        if ((e = cudaMemcpyAsync(d_keys, keys[1], 4 * (size_t)n, cudaMemcpyDeviceToDevice, s)) == cudaSuccess)
            e = cudaMemcpyAsync(d_perm, perm[1], 4 * (size_t)n, cudaMemcpyDeviceToDevice, s);
    }
    if (e == cudaSuccess && d_cells) {
        e = cudaMemsetAsync(d_cells, 0xFF, 8 * (size_t)params->gridBufSize, s);
        if (e == cudaSuccess) pbf::launch_update_cells((int)n, d_keys, d_cells, params->gridBufSize, nullptr, s);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return pbf::fail(nullptr, PBF_ERR_CUDA, std::string("pbf_sort_state_noalloc: ") + cudaGetErrorString(e));
    return PBF_OK;
}
