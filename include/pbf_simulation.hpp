// pbf_simulation.hpp — C++ facade with the reference's host interface.
//
// Mirrors src/Simulation.hpp:28-151 and src/ParamUtils.hpp: a global
// `Parameters Params`, `LoadParameters(std::string)`, and a class
// `Simulation` whose InitBuffers / InitCells / LoadForceMasks / InitKernels /
// Step keep their names, order and meaning.  Differences a caller sees:
//   - the constructor takes a CUDA device ordinal instead of an OpenCL
//     context and device (Simulation.cpp:56-63);
//   - positions live in device memory owned by the library, not in GL
//     buffers: DevicePositions() gives their address, ReadState() copies them
//     out (the reference's mSharedPingBufferID / mSharedPongBufferID);
//   - errors are thrown as std::runtime_error carrying the library's message
//     (the reference throws cl::Error / std::runtime_error), and InitKernels
//     returns false on a parameter set the kernels cannot run, as the
//     reference returns false on a build failure (Simulation.cpp:186-188).
// Header-only over include/pbf_capi.h; link with libpbf_gb300.so.
#pragma once

#include <deque>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "pbf_capi.h"

typedef PbfParameters Parameters;

// src/ParamUtils.cpp:19-22: the global parameter set, zero-initialised.
inline Parameters Params = {};
inline bool ParametersChanged = false;

// src/ParamUtils.cpp:24-100
inline void LoadParameters(std::string fileContents) {
    if (pbf_load_parameters(fileContents.c_str(), &Params, nullptr) != PBF_OK)
        throw std::runtime_error(pbf_last_error(nullptr));
    ParametersChanged = true;
}

// src/OCLPerfMon.h: one performance tracker (without the cl::Event), and the
// monitor whose Trackers vector the reference's UI reads
// (src/UIManager.cpp:185-215, 336-345).
typedef struct {
    std::string eventName;
    uint64_t time_start;  // [nano sec]
    uint64_t time_end;    // [nano sec]
    double total_time;    // [millisec]
    double last_time;     // [millisec]
    int Tag;
} PM_PERFORMANCE_TRACKER;

class OCLPerfMon {
public:
    std::vector<PM_PERFORMANCE_TRACKER*> Trackers;

    // OCLPerfMon::UpdateTimings: here the library keeps the smoothed times;
    // this copies them in (pbf_perf_trackers).
    void UpdateTimings(pbf_ctx* ctx) {
        int count = 0;
        if (pbf_perf_trackers(ctx, nullptr, 0, &count) != PBF_OK) return;
        std::vector<PbfPerfTracker> t((size_t)count);
        if (count && pbf_perf_trackers(ctx, t.data(), count, &count) != PBF_OK) return;
        while (mStore.size() < t.size()) {
            mStore.push_back(PM_PERFORMANCE_TRACKER{});
            Trackers.push_back(&mStore.back());
        }
        for (size_t i = 0; i < t.size(); ++i) {
            PM_PERFORMANCE_TRACKER& p = mStore[i];
            p.eventName = t[i].eventName;
            p.time_start = t[i].time_start;
            p.time_end = t[i].time_end;
            p.total_time = t[i].total_time;
            p.last_time = t[i].last_time;
        }
    }

private:
    std::deque<PM_PERFORMANCE_TRACKER> mStore;  // stable addresses for Trackers
};

class Simulation {
public:
    explicit Simulation(int device = 0) : mDevice(device) {}
    ~Simulation() { pbf_destroy(mCtx); }
    Simulation(const Simulation&) = delete;
    Simulation& operator=(const Simulation&) = delete;

    // Simulation::InitBuffers (src/Simulation.cpp:206-244): buffers for
    // Params.particleCount particles, initial positions from `pos` (float4 per
    // particle) or the reference's CreateParticles lattice, velocities from
    // `vel` or zero.
    void InitBuffers(const float* pos = nullptr, const float* vel = nullptr) {
        pbf_destroy(mCtx);
        mCtx = nullptr;
        check(pbf_create(&Params, mDevice, &mCtx), nullptr);
        check(pbf_init_buffers(mCtx, pos, vel));
    }

    // Simulation::InitCells (src/Simulation.cpp:246-255)
    void InitCells() {
        syncParams(false);
        check(pbf_init_cells(mCtx));
    }

    // Simulation::LoadForceMasks (src/Simulation.cpp:257-281): the empty mask,
    // or `mask` (width x height texels, R channel) where the reference reads
    // Scene_fp_mask.png.
    void LoadForceMasks(const uint32_t* mask = nullptr, int width = 0, int height = 0) {
        check(pbf_load_force_masks(mCtx, mask, width, height));
    }

    // The force planes the reference hard-codes in computeDelta
    // (compute_delta.cl:169-182), as data.
    void SetForceQuads(const PbfForceQuad* quads, int count) { check(pbf_set_force_quads(mCtx, quads, count)); }

    // Simulation::InitKernels (src/Simulation.cpp:129-204)
    bool InitKernels() {
        if (!mCtx) return false;
        if (pbf_set_params(mCtx, &Params) != PBF_OK) return false;
        return pbf_init_kernels(mCtx) == PBF_OK;
    }

    // Simulation::Step (src/Simulation.cpp:554-621): one substep, synchronous.
    // fWavePos moves the box clamp's low x wall (the reference passes it to
    // computeDelta, which ignores it); bDumpParticlesData saves the state
    // after the step to DumpPath (the reference's dump is unfinished,
    // src/Simulation.cpp:605-611).
    void Step() {
        check(pbf_set_pause(mCtx, bPauseSim ? 1 : 0));
        if (fWavePos != mWaveSent) {
            check(pbf_set_wave_position(mCtx, fWavePos));
            mWaveSent = fWavePos;
        }
        if (mTrack) check(pbf_enable_stage_timing(mCtx, 1));
        check(pbf_step(mCtx, 1));
        if (mTrack) PerfData.UpdateTimings(mCtx);
        if (bDumpParticlesData) {
            bDumpParticlesData = false;
            SaveState(DumpPath);
        }
    }

    // Binary particle state (pbf_save_state / pbf_load_state).
    void SaveState(const std::string& path) { check(pbf_save_state(mCtx, path.c_str())); }
    void LoadState(const std::string& path) { check(pbf_load_state(mCtx, path.c_str())); }

    // Simulation::KernelFileList (src/Simulation.cpp:103-127): the sources
    // the device code is built from.
    const std::string* KernelFileList() {
        static const std::string files[] = {"pbf_kernels.cu", "pbf_sort.cu", "pbf_adjoint.cu", "pbf_capi.cu",
                                            "pbf_noalloc.cu", ""};
        return files;
    }

    // ---- state access replacing the GL-shared buffers ----
    void* DevicePositions() {
        void* p = nullptr;
        check(pbf_device_positions(mCtx, &p));
        return p;
    }
    void ReadState(float* pos, float* vel, float* pred = nullptr) { check(pbf_read_state(mCtx, pos, vel, pred)); }
    void WriteState(const float* pos, const float* vel) { check(pbf_write_state(mCtx, pos, vel)); }

    // Turns the per-stage trackers on (each Step then times its stages).
    void TrackPerformance(bool on) {
        mTrack = on;
        check(pbf_enable_stage_timing(mCtx, on ? 1 : 0));
    }

    pbf_ctx* handle() const { return mCtx; }

    bool bPauseSim = false;
    float fWavePos = 0.0f;            // src/Simulation.hpp:150
    bool bDumpParticlesData = false;  // src/Simulation.hpp:149
    std::string DumpPath = "particles.pbfstate";
    OCLPerfMon PerfData;

private:
    void check(int rc, pbf_ctx* ctx) const {
        if (rc != PBF_OK) throw std::runtime_error(pbf_last_error(ctx));
    }
    void check(int rc) const { check(rc, mCtx); }

    void syncParams(bool strict) {
        if (!mCtx) throw std::runtime_error("InitBuffers must run first");
        int rc = pbf_set_params(mCtx, &Params);
        if (strict) check(rc);
    }

    int mDevice = 0;
    float mWaveSent = 0.0f;
    pbf_ctx* mCtx = nullptr;
    bool mTrack = false;
};
