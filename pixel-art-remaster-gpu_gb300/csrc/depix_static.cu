// depix_static.cu -- heuristic crossing resolution in place, with its graph
// snapshot held in a fixed device array instead of allocated memory.
//
// The heuristics read a snapshot of the graph while they rewrite it (the
// reference copies graph to graph_aux before ambiguous_cross_Kernel,
// kernel.cu:415-423). depix_resolve_heuristics takes that snapshot from the
// caller; depix_resolve_heuristics_static keeps it in g_static_snapshot
// below, so a caller that cannot allocate device memory still gets the
// in-place stage. The array exists once per device that loads the library
// and stays until the process exits.
#include <mutex>
#include <string>
#include <vector>

#include "depix_internal.h"

namespace {

constexpr size_t kStaticSnapshotBytes = (size_t)DEPIX_STATIC_MAX_PIXELS; // one byte per node

static __device__ __align__(256) uint8_t g_static_snapshot[kStaticSnapshotBytes];

std::mutex g_static_mu;
struct StaticAddr {
    uint8_t* p = nullptr; // device address of g_static_snapshot
    CUcontext ctx = nullptr; // the context it was looked up in
};
std::vector<StaticAddr> g_static_addr; // per device

// The calling thread's current context (driver entry point reached through
// the runtime; nullptr when unavailable).
CUcontext current_context()
{
    using GetCurrent = CUresult (*)(CUcontext*);
    static GetCurrent fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<GetCurrent>(p);
    }();
    CUcontext c = nullptr;
    if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
    return c;
}

// Looks up the array's device address once per device and context, with
// that device current. The host-side name g_static_snapshot is not a device
// address. A saved address is reused only in the context it was looked up
// in: after cudaDeviceReset the device's primary context is a new one, and
// the array's address is looked up again.
depix_status static_snapshot(uint8_t** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        depix::set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
        return DEPIX_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_static_mu);
    CUcontext ctx = current_context();
    if (dev < (int)g_static_addr.size() && g_static_addr[dev].p && ctx && g_static_addr[dev].ctx == ctx) {
        *out = g_static_addr[dev].p;
        return DEPIX_OK;
    }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_snapshot);
    if (e != cudaSuccess || !p) {
        depix::set_last_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return DEPIX_ERR_CUDA;
    }
    if (dev >= (int)g_static_addr.size()) g_static_addr.resize(dev + 1);
    // the first call in a context made that context current (cudaGetDevice
    // and the lookup above), so ctx is set from then on
    g_static_addr[dev] = StaticAddr{static_cast<uint8_t*>(p), ctx ? ctx : current_context()};
    *out = g_static_addr[dev].p;
    return DEPIX_OK;
}

}  // namespace

extern "C" {

depix_status depix_resolve_heuristics_static(uint8_t* d_graph, int w, int h, depix_stream s)
{
    if (!d_graph || w < 1 || h < 1) {
        depix::set_last_error("graph pointer is NULL or a size is below 1");
        return DEPIX_ERR_INVALID_ARG;
    }
    const size_t n = (size_t)w * (size_t)h;
    if (n > kStaticSnapshotBytes) {
        depix::set_last_error("frame of " + std::to_string(n) + " pixels is larger than the fixed snapshot of " +
                              std::to_string(kStaticSnapshotBytes) + " pixels");
        return DEPIX_ERR_TOO_LARGE;
    }
    uint8_t* snap = nullptr;
    depix_status st = static_snapshot(&snap);
    if (st != DEPIX_OK) return st;
    cudaStream_t cs = reinterpret_cast<cudaStream_t>(s);
    // the copy overwrites every snapshot byte the kernel reads: nothing has
    // to start at zero, whatever an earlier call left in the array
    cudaError_t e = cudaMemcpyAsync(snap, d_graph, n, cudaMemcpyDeviceToDevice, cs);
    if (e == cudaSuccess) e = depix::launch_heuristics(depix::GraphBatch{snap, d_graph, 0, w, h}, 1, cs);
    if (e != cudaSuccess) {
        depix::set_last_error(std::string("snapshot copy or launch: ") + cudaGetErrorString(e));
        return DEPIX_ERR_CUDA;
    }
    return DEPIX_OK;
}

}  // extern "C"
