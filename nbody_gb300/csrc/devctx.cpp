// devctx.cpp -- identity of the CUDA context current on the calling thread.
//
// Several per-device caches in this library hold values that belong to one
// CUDA context: the drop-in entry point's workspace, the planner's occupancy
// table together with the shared-memory attributes it set on the kernels,
// and the device address of the fixed scratch array.  A host that calls
// cudaDeviceReset destroys the device's primary context (the reference's
// teardown does, src/nbody.cu:497-507); the runtime creates a new context at
// the next call, and every cached pointer and attribute of the old one is
// gone.  The caches therefore remember the id of the context they were
// filled under and start again when it changes.  The id is the driver's
// cuCtxGetId (unique within the process, never reused), reached through the
// runtime's entry-point query so the library has no link-time dependency on
// libcuda.
#include <cuda.h>
#include <cuda_runtime.h>

#include "nbgb_internal.h"
#include "nbody_gb300.h"

namespace nbgb {
namespace {

typedef CUresult (*PfnCtxGetCurrent)(CUcontext *);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long *);

struct DriverFns {
    PfnCtxGetCurrent get_current = nullptr;
    PfnCtxGetId get_id = nullptr;
};

const DriverFns &driver_fns() {
    static const DriverFns fns = [] {
        DriverFns f;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f.get_current = (PfnCtxGetCurrent)p;
        p = nullptr;
        q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f.get_id = (PfnCtxGetId)p;
        return f;
    }();
    return fns;
}

}  // namespace

int current_context(int *device, unsigned long long *ctx_id) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return NBGB_ERR_CUDA;
    const DriverFns &f = driver_fns();
    if (!f.get_current || !f.get_id)
        return NBGB_ERR_CUDA;
    CUcontext c = nullptr;
    if (f.get_current(&c) != CUDA_SUCCESS)
        return NBGB_ERR_CUDA;
    if (!c) {
        // No context current on this thread yet: make the device's primary
        // context current, as the runtime's next call would.
        if (cudaSetDevice(dev) != cudaSuccess || f.get_current(&c) != CUDA_SUCCESS || !c)
            return NBGB_ERR_CUDA;
    }
    unsigned long long id = 0;
    if (f.get_id(c, &id) != CUDA_SUCCESS)
        return NBGB_ERR_CUDA;
    *device = dev;
    *ctx_id = id;
    return NBGB_OK;
}

}  // namespace nbgb
