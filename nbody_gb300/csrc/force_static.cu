// force_static.cu -- the force evaluation for callers that cannot allocate
// device memory.
//
// nbgb_force and the drop-in entry point need scratch space (the paired
// j-stream, and split partials plus counters for large j-splits).  nbgb_force
// takes it from the caller, the drop-in allocates and caches it.  Some callers
// can do neither: hosts that own all device memory through their own pool or a
// budget fixed at start-up (a cudaMalloc behind their back breaks their
// accounting and can fail mid-run), and latency-critical step loops, where
// cudaMalloc/cudaFree may synchronise the device and take driver-wide locks.
// nbgb_force_static serves them: its scratch is this file's fixed device array,
// so a call allocates nothing.
//
// Costs and rules of that choice:
//  * the array (kStaticScratchBytes = 32 MiB) is part of the library's device
//    image: every GPU that loads the library holds it until the process exits;
//  * N is limited to what a plan inside 32 MiB can handle: the j-stream alone
//    needs 16 B per body, so at most 2,097,152 bodies; larger N is rejected
//    with NBGB_ERR_TOO_LARGE before anything is launched;
//  * every call on a device shares the one array and it keeps the previous
//    call's contents; the split counters that must start at zero are cleared by
//    the call's own first kernel, so calls in sequence are independent, but
//    calls that overlap on the GPU (different streams, or host threads) race;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress, once per device and context, with that device
//    current); make that first call before capturing any stream.  After a
//    cudaDeviceReset the next call looks the address up again in the new
//    context.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "nbgb_internal.h"
#include "nbody_gb300.h"

namespace nbgb {
namespace {

constexpr size_t kStaticScratchBytes = (size_t)32 << 20;

// Device scratch shared by every nbgb_force_static call on a device.  In host
// code this name is only a stand-in for the symbol; its device address comes
// from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {nullptr};
unsigned long long g_scratch_ctx[kMaxDevices] = {0};

// Device address of g_static_scratch on the current device, looked up once
// per device and context (a reset context loads the module again, possibly
// at another address).
int scratch_address(void **out) {
    int dev = 0;
    unsigned long long ctx = 0;
    if (current_context(&dev, &ctx) != NBGB_OK || dev < 0 || dev >= kMaxDevices)
        return NBGB_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev] || g_scratch_ctx[dev] != ctx) {
        void *p = nullptr;
        g_scratch_addr[dev] = nullptr;
        if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p)
            return NBGB_ERR_CUDA;
        g_scratch_addr[dev] = p;
        g_scratch_ctx[dev] = ctx;
    }
    *out = g_scratch_addr[dev];
    return NBGB_OK;
}

}  // namespace
}  // namespace nbgb

extern "C" {

NBGB_API size_t nbgb_force_static_capacity_bytes(void) { return nbgb::kStaticScratchBytes; }

NBGB_API int nbgb_force_static(float *force, const float *posMass, float softeningSquared,
                               size_t N, void *stream) {
    if (N == 0)
        return NBGB_OK;
    if (!force || !posMass)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (((uintptr_t)force | (uintptr_t)posMass) & 15u)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (N > nbgb::kStaticScratchBytes / 16)
        return NBGB_ERR_TOO_LARGE;
    nbgb::ForcePlan pl;
    int rc = nbgb::plan_force_within(N, nbgb::kStaticScratchBytes, pl);
    if (rc != NBGB_OK)
        return rc;
    void *ws = nullptr;
    if ((rc = nbgb::scratch_address(&ws)) != NBGB_OK)
        return rc;
    cudaStream_t st = (cudaStream_t)stream;
    // The pack launch also zeroes the split counters the force launch uses.
    if ((rc = nbgb::launch_pack(pl, (const float4 *)posMass, ws, st)) != NBGB_OK)
        return rc;
    return nbgb::launch_force(pl, (float4 *)force, (const float4 *)posMass, nullptr,
                              softeningSquared, ws, st);
}

}  // extern "C"
