// Head2MEGMat without any device allocation.
//
// Who needs this: programs that must not allocate device memory once they
// are running.  Examples are an acquisition or neurofeedback loop that
// recomputes MEG sensor matrices as the head moves and cannot stall on the
// allocator, a host that reserves (nearly) all of the GPU's memory for itself
// at start-up, or a plugin host whose memory policy forbids device
// allocations from plugins.  The regular entry point allocates an
// n_squids x n_triangles scratch array for the Ferguson pass on every call;
// this variant uses one fixed array that lives in the library's device image.
//
// Contract
//  - The scratch array below is OMG_NOALLOC_SCRATCH_DOUBLES doubles (32 MiB);
//    every GPU on which this entry point runs holds it until the process exits.
//    Requests with n_squids x n_triangles above that size are rejected with
//    OMG_ERR_INVALID and nothing is launched.
//  - The first call on a device does the set-up: it resolves the array's
//    device address with cudaGetSymbolAddress (which also loads this part of
//    the library onto that device).  Make that first call during
//    initialisation, before any stream capture and before the phase in which
//    the program may not allocate.
//  - All calls share the one array.  Calls whose work overlaps on the GPU --
//    on different streams or different host threads -- race on it and give
//    wrong results; serialise them (one stream, or one call at a time).
//  - Nothing in the array needs to start at zero: the Ferguson pass writes
//    every entry it later reads.  The output matrix is cleared by the call.
//  - The call waits for its work on the context's stream to finish before it
//    returns, as omg_head2megmat_dev does.
//  - No cudaMalloc, cudaMallocAsync, cudaFree or allocating library routine
//    is called.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "pipeline.h"

namespace omg {
void launch_h2mm(const DevGeom& g, const double* sq, int64_t np, const int32_t* tmesh, const double* jump, int perm,
                 double* out, int64_t rs, int64_t cs, int64_t col0, double* F, cudaStream_t s,
                 double mag = kMagFactor);
}

static __device__ __align__(256) double g_h2mm_scratch[OMG_NOALLOC_SCRATCH_DOUBLES];

namespace {
constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;

// Device address of the scratch array on `device` (the current device).
double* scratch_address(int device) {
    if (device < 0 || device >= kMaxDevices) throw Error(OMG_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        const cudaError_t rc = cudaGetSymbolAddress(&p, g_h2mm_scratch);
        if (rc != cudaSuccess || p == nullptr)
            throw Error(OMG_ERR_CUDA, std::string("cudaGetSymbolAddress of the scratch array failed: ") +
                                          cudaGetErrorString(rc));
        g_scratch_addr[device] = static_cast<double*>(p);
    }
    return g_scratch_addr[device];
}
}  // namespace

extern "C" int omg_head2megmat_noalloc_dev(omg_context ctx, omg_geometry geo, const double* squids, int64_t n_squids,
                                           double* h2mm) {
    return guarded([&] {
        OMG_REQUIRE(ctx && geo, "null argument");
        OMG_REQUIRE(n_squids >= 0, "negative sensor count");
        OMG_REQUIRE(n_squids == 0 || (squids && h2mm), "null sensors or output");
        if (geo->h.shared)   // the per-distinct-vertex sum needs a buffer of the vertex copies
            throw Error(OMG_ERR_UNSUPPORTED, "geometries whose meshes share vertices need omg_head2megmat_dev");
        set_device(ctx);
        double* scratch = scratch_address(ctx->device);
        if (n_squids == 0) return;
        const int64_t need = n_squids * geo->h.nt;
        if (need > (int64_t)OMG_NOALLOC_SCRATCH_DOUBLES)
            throw Error(OMG_ERR_INVALID, "n_squids x n_triangles = " + std::to_string(need) +
                                             " exceeds the fixed scratch of " +
                                             std::to_string((long long)OMG_NOALLOC_SCRATCH_DOUBLES) + " doubles");
        cudaStream_t s = ctx->stream;
        OMG_CUDA(cudaMemsetAsync(h2mm, 0, (size_t)n_squids * geo->h.N * sizeof(double), s));
        omg::launch_h2mm(geo->d, squids, n_squids, geo->tmesh, geo->jump, 0, h2mm, n_squids, 1, 0, scratch, s);
        OMG_CUDA(cudaStreamSynchronize(s));
        OMG_CUDA(cudaGetLastError());
    });
}
