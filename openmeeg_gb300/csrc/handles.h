// Handle types of the C ABI, shared by the translation units that implement
// entry points (api.cpp, noalloc.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <vector>

#include "omg_internal.h"

using omg::DevGeom;
using omg::Error;
using omg::HostGeometry;

struct omg_context_s {
    int device = 0;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    int* d_err = nullptr;          // [0] status, [1..2] pad
    int64_t* d_errcol = nullptr;
    double* d_scalar = nullptr;
    int64_t launches_at_create = 0;
    int refs = 1;              // the caller's handle + one per live geometry / solver
    // second stream and the events of the factorization's look-ahead (created on first use)
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr, ev_c = nullptr, ev_d = nullptr, ev_e = nullptr;
    // highest-priority stream of the latency-bound solve chains (their CTAs go first onto SMs that free up
    // while other work runs on the second stream; created on first use)
    cudaStream_t hi = nullptr;
};

inline void release_aux(omg_context_s* c) {
    if (c->hi) cudaStreamDestroy(c->hi);
    c->hi = nullptr;
    if (c->aux) cudaStreamDestroy(c->aux);
    for (cudaEvent_t e : {c->ev_a, c->ev_b, c->ev_c, c->ev_d, c->ev_e})
        if (e) cudaEventDestroy(e);
    c->aux = nullptr;
    c->ev_a = c->ev_b = c->ev_c = c->ev_d = c->ev_e = nullptr;
}

// Live bytes of all device buffers of the library and their high-water mark
// (reset by the calls that report a peak footprint).
extern std::atomic<int64_t> g_dev_live, g_dev_peak;
inline void note_alloc(int64_t bytes) {
    const int64_t now = g_dev_live.fetch_add(bytes) + bytes;
    int64_t pk = g_dev_peak.load();
    while (now > pk && !g_dev_peak.compare_exchange_weak(pk, now)) {
    }
}

// Device buffer.  Temporaries of one call are stream-ordered
// (cudaMallocAsync/cudaFreeAsync on the call's stream); buffers that outlive
// the call (geometry, solver) are plain allocations, so freeing them never
// depends on a stream that may be gone by then.
struct DevBuf {
    void* p = nullptr;
    cudaStream_t s = nullptr;
    bool persistent = false;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(size_t nbytes, cudaStream_t st, bool keep = false) : s(st), persistent(keep) {
        if (!nbytes) return;
        cudaError_t e = persistent ? cudaMalloc(&p, nbytes) : cudaMallocAsync(&p, nbytes, st);
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (e == cudaErrorMemoryAllocation && cudaStreamIsCapturing(st, &cs) == cudaSuccess &&
            cs == cudaStreamCaptureStatusNone) {
            // memory freed into the stream-ordered pool stays with the pool, in blocks that may not take
            // this request: wait for the pending frees, hand the pool's unused memory back, try once more
            cudaGetLastError();
            cudaDeviceSynchronize();
            int dev = 0;
            cudaMemPool_t pool;
            if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
                cudaMemPoolTrimTo(pool, 0);
            e = persistent ? cudaMalloc(&p, nbytes) : cudaMallocAsync(&p, nbytes, st);
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            size_t fr = 0, tot = 0;
            cudaMemGetInfo(&fr, &tot);
            throw ::omg::Error(e == cudaErrorMemoryAllocation ? OMG_ERR_NOMEM : OMG_ERR_CUDA,
                               "device allocation of " + std::to_string(nbytes >> 20) + " MiB (" +
                                   std::to_string(fr >> 20) + " MiB free): " + cudaGetErrorString(e));
        }
        bytes = nbytes;
        note_alloc((int64_t)bytes);
    }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), s(o.s), persistent(o.persistent), bytes(o.bytes) {
        o.p = nullptr;
        o.bytes = 0;
    }
    DevBuf& operator=(DevBuf&& o) noexcept {
        release();
        p = o.p;
        s = o.s;
        persistent = o.persistent;
        bytes = o.bytes;
        o.p = nullptr;
        o.bytes = 0;
        return *this;
    }
    ~DevBuf() { release(); }
    void release() {
        if (p) {
            if (persistent) {
                cudaStreamSynchronize(s);
                cudaFree(p);
            } else {
                cudaFreeAsync(p, s);
            }
            g_dev_live.fetch_sub((int64_t)bytes);
        }
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

template <typename T>
inline T* upload(std::vector<DevBuf>& keep, const std::vector<T>& v, cudaStream_t s) {
    keep.emplace_back(std::max<size_t>(1, v.size()) * sizeof(T), s, true);
    if (!v.empty()) OMG_CUDA(cudaMemcpyAsync(keep.back().p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return keep.back().as<T>();
}

struct omg_geometry_s {
    omg_context ctx = nullptr;
    int refs = 1;              // the caller's handle + one per live solver
    HostGeometry h;
    DevGeom d;                  // assembly: every mesh with its own vertex copies
    DevGeom dg;                 // the reference's unknowns (distinct vertices); == d unless meshes share vertices
    int64_t* gbeg = nullptr;    // distinct vertex u -> its copies gcopy[gbeg[u] .. gbeg[u + 1])
    int64_t* gcopy = nullptr;
    int* bgrp = nullptr;        // per domain boundary entry: index of its interface within the domain
    std::vector<DevBuf> bufs;
    // mesh-level device tables
    int32_t* tmesh = nullptr;
    int64_t* tidx_ref = nullptr;
    int* barrier = nullptr;
    int* orient = nullptr;      // per domain boundary entry (ndom x maxb): the mesh's orientation in its interface
    int64_t* tbeg = nullptr;
    double* jump = nullptr;
    int32_t* eeg_cand = nullptr;
    int64_t n_eeg_cand = 0;
    int64_t* eeg_seg = nullptr;   // candidate offsets of each interface touching a zero-conductivity domain
    int n_eeg_seg = 0;
    // domain tables
    int ndom = 0, maxb = 1;
    int* dnb = nullptr;
    int* bmesh = nullptr;
    int* binside = nullptr;
    double* dsigma = nullptr;
    int prepared_order = -1;
    float* grec = nullptr;      // FP32 far-field records (mixed precision), built on first use
    uint64_t version = 0;       // bumped when the conductivities change (captured graphs go stale)
};


// Thread-local message behind omg_last_error().
void set_last_error(const char* msg);
