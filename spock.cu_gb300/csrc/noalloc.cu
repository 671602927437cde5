// spock_project_dynamics_noalloc: the dynamics-projection sweep with its workspaces in a
// static device buffer, for callers that must not allocate device memory while they solve.
//
// The sweep normally keeps its two workspaces (the backward-sweep q of every node and the
// d of every nonleaf node) in memory the solver allocates.  Some callers cannot let a call
// allocate: a control loop that re-solves every sample under a hard deadline, where a
// cudaMalloc's latency or failure is not acceptable, or a host application whose framework
// owns the device memory pool and forbids allocations outside it.  For them the workspaces
// live in g_spockDynScratch below, a file-scope device array of kScratchBytes (8 MiB) that
// every GPU loading this library holds until the process exits.
#include <cuda_runtime.h>

#include <mutex>
#include <stdexcept>
#include <string>

#include "capi_internal.hpp"

namespace {

constexpr size_t kScratchBytes = size_t(8) << 20;
static __device__ __align__(256) unsigned char g_spockDynScratch[kScratchBytes];

constexpr int kMaxDevices = 64;
void *g_scratchAddr[kMaxDevices] = {};
std::mutex g_scratchMutex;

// Device address of the buffer on the current device, looked up once per device.  In host
// code g_spockDynScratch names a host-side stand-in, never the device memory itself.  The
// cached address stays valid while the device's primary context lives; a process that resets
// the device (cudaDeviceReset) must not call this entry point afterwards.
void *scratchOnCurrentDevice() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) throw std::runtime_error(std::string("[noalloc] cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) throw std::runtime_error("[noalloc] device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_scratchMutex);
    if (!g_scratchAddr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_spockDynScratch);
        if (e != cudaSuccess || !p)
            throw std::runtime_error(std::string("[noalloc] cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratchAddr[dev] = p;
    }
    return g_scratchAddr[dev];
}

// Makes `device` current for the call and gives the caller back its own current device after.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int device) {
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) throw std::runtime_error(std::string("[noalloc] cudaGetDevice: ") + cudaGetErrorString(e));
        if (prev != device) {
            e = cudaSetDevice(device);
            if (e != cudaSuccess)
                throw std::runtime_error(std::string("[noalloc] cudaSetDevice: ") + cudaGetErrorString(e));
        }
    }
    ~DeviceGuard() {
        int cur = -1;
        if (cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace

extern "C" int spock_project_dynamics_noalloc(spock_solver s, const void *x0, void *prim_ux, void *stream) {
    return spock::guardedCall([&] {
        spock::EngineBase *eng = spock::engineOf(s);
        if (!x0 || !prim_ux) throw std::invalid_argument("[noalloc] null device pointer");
        DeviceGuard guard(eng->device());
        void *scratch = scratchOnCurrentDevice();
        // nothing in the buffer needs to start at zero: the sweep writes every workspace entry
        // before it reads it
        eng->projectDynamicsOn(x0, prim_ux, scratch, kScratchBytes, static_cast<cudaStream_t>(stream));
    });
}
