// nbgb_internal.h -- declarations shared between the library's translation
// units (not part of the public C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace nbgb {

// Largest N any entry point accepts (indices are 32-bit inside the kernels).
constexpr size_t kMaxBodies = (size_t)1 << 30;

// The current device and the id of the CUDA context current on this thread
// (unique within the process; a context re-created after cudaDeviceReset has
// a new id).  Per-device caches compare it to detect a reset.  NBGB_OK or
// NBGB_ERR_CUDA.
int current_context(int *device, unsigned long long *ctx_id);

// One force evaluation's decomposition and workspace layout.
struct ForcePlan {
    int config = 0;       // index into the kernel configuration table
    int nsplit = 1;       // j-slices of each split i-block
    int nfull = 0;        // leading i-blocks evaluated whole (one unit each); the
                          // rest are split nsplit ways (nsplit = 1: nfull = nblocks)
    size_t n = 0;         // bodies (sources; also the targets unless nt says otherwise)
    size_t nt = 0;        // target bodies (rows) when they are a slice: 0 = n
    int block_bodies = 0; // targets per CTA (BI)
    int tile_bodies = 0;  // sources per shared-memory tile (JT)
    int nblocks = 0;      // i-blocks
    int ntiles = 0;       // j-tiles (the j-stream holds ntiles*JT bodies)
    int js_vpb = 1;       // float4s per body in the j-stream (1 pairs, 2 duplicated)
    int js_log = 0;       // 1: pairs q % 4 == 0 hold log2 masses (mode 6)
    size_t ni_pad = 0;    // nblocks * BI
    size_t off_js = 0, off_hi = 0, off_lo = 0, off_cnt = 0;
    size_t workspace_bytes = 0;
};

int plan_force(size_t n, int force_config, int force_nsplit, ForcePlan &pl);
// As plan_force(n, -1, -1), among configurations without log-domain pairs
// (for masses < 0, which have no logarithm).
int plan_force_rsqrt(size_t n, ForcePlan &pl);
int plan_force_within(size_t n, size_t max_bytes, ForcePlan &pl);
// Plan for `rows` target bodies (a contiguous slice of the n bodies) against
// all n sources; launch_force then takes the slice's first body as posMass.
int plan_force_rows(size_t n, size_t rows, ForcePlan &pl);
inline size_t plan_targets(const ForcePlan &pl) { return pl.nt ? pl.nt : pl.n; }
// i-blocks whose j-range is split (each has a partial-sum slot per slice and
// a completion counter), and the work units of one launch
inline int split_blocks(const ForcePlan &pl) { return pl.nsplit > 1 ? pl.nblocks - pl.nfull : 0; }
inline long long plan_units(const ForcePlan &pl) {
    return (long long)pl.nblocks + (long long)split_blocks(pl) * (pl.nsplit - 1);
}
// js_out == nullptr: the j-stream inside the workspace (and the split
// counters are zeroed); else only that j-stream buffer is written.
int launch_pack(const ForcePlan &pl, const float4 *posMass, void *workspace, cudaStream_t stream,
                float4 *js_out = nullptr);
// The reference integrator fused into the force launch's epilogue: pm is the
// posMass the launch reads its targets from (updated in place), js the
// j-stream buffer for the next step (not the one being read).  js_vpb and
// js_log are taken from the plan.
struct FusedIntegrate {
    float4 *pm = nullptr;
    float4 *vel = nullptr;
    float4 *js = nullptr;
    float dt = 0.f, damping = 1.f;
    int fused_drift = 0;
    int js_vpb = 1, js_log = 0;
};
// jstream == nullptr: use the j-stream inside the workspace.  fi != nullptr
// (full systems only, not row slices): integrate every target after its force.
int launch_force(const ForcePlan &pl, float4 *force, const float4 *posMass, const float4 *jstream,
                 float eps2, void *workspace, cudaStream_t stream,
                 const FusedIntegrate *fi = nullptr);
int read_and_clear_status(unsigned *bits);
int read_status_ensemble(unsigned *bits);
int read_status_integrate(unsigned *bits);
// js_vpb, js_log: j-stream layout of the plan the j-stream is written for.
// fused_drift: x = fma(v, dt, x), as the reference's own build computes it.
int launch_integrate_reference(float4 *pm, float4 *vel, const float4 *force, float dt,
                               float damping, size_t n, int fused_drift, float4 *js, int js_vpb,
                               int js_log, int npad, unsigned *counters, int ncounters,
                               cudaStream_t st);
// FP64 SoA state x64 = [x, y, z, vx, vy, vz], each component ld doubles
// (ld even, >= n).
int launch_kick_drift(double *x64, size_t ld, const float *mass, const float4 *accel,
                      double kick_dt, double drift_dt, size_t n, float4 *pm, float4 *js,
                      int js_vpb, int js_log, int npad, unsigned *counters, int ncounters,
                      cudaStream_t st);
int launch_half_kick(double *x64, size_t ld, const float4 *accel, double kick_dt, size_t n,
                     cudaStream_t st);
size_t diag_scratch_bytes();
int launch_diagnostics(int n, const double *x64, size_t ld, const float *mass, const float4 *pm,
                       const float4 *vel, const float4 *phi, double *scratch, double *out8,
                       cudaStream_t st);
// Newton-3 evaluation of many systems in one launch (the ensemble): one
// entry per system, ordered, pair_begin = block pairs of the entries before.
// js: paired j-stream padded with zero masses to nblocks * sym_block_bodies()
// bodies (no log2 masses); acc: [3][npad] FP64 sums, zero on entry, left
// zero on exit; out: FP32 accelerations.
struct SymSystem {
    const float4 *pm;
    const float4 *js;
    double *acc;
    float4 *out;
    int n, npad, nblocks;
    float eps2;
    long long pair_begin;
};
int launch_sym_systems(const SymSystem *d_tab, const SymSystem *h_tab, int nsys,
                       cudaStream_t st);
int sym_block_bodies();

// force-kernel configuration that also returns the potential (in w)
constexpr int kPotentialConfig = 23;
const char *config_name(int c);
int num_configs();

}  // namespace nbgb
