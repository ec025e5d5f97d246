// force.cu -- all-pairs softened gravity on GB300 (sm_103a).
//
// Computes, for every target body i,
//     F_i = sum_j m_j (p_j - p_i) / (|p_j - p_i|^2 + eps2)^(3/2)
// exactly the sum of src/bodybodyInteraction.cuh:40-65 over all j (self term
// included; it is 0 because eps2 > 0), as the reference's
// ComputeGravitation_* algorithms do (e.g. src/nbody_GPU_Shared.cu:42-81).
//
// Structure (one launch per force evaluation, after a tiny pack launch):
//
//   pack_jstream   float4 AOS {x,y,z,m} -> "j-stream": bodies in pairs laid
//                  out {x0,x1,y0,y1,z0,z1,m0,m1} (32 B per pair), padded with
//                  zero-mass bodies to a whole number of j-tiles.  The same
//                  launch zeroes the split counters.
//   force_kernel   one CTA per work unit (i-block, j-split).  The i-block is
//                  W warps x 32 lanes x K target bodies held in registers.  The
//                  j-split's tiles of JT bodies are streamed into shared memory
//                  by 1-D bulk copies (cp.async.bulk, TMA) into a STAGES-deep
//                  ring completing on mbarriers, read back with broadcast
//                  128-bit shared loads, and evaluated two interactions per
//                  instruction with the f32x2 FP32 instructions (rsqrt on the
//                  MUFU pipe; mode 6 takes every fourth source pair's
//                  m r^-3 in the log domain, 2^(log2 m - 1.5 log2 r^2), to
//                  move work from the FMA pipe to the MUFU pipe, whose ex2
//                  runs at twice the rsqrt rate on sm_103).  Every 256
//                  sources the FP32 partial sum is
//                  folded into a per-body compensated (TwoSum) running sum.
//                  When the i-blocks do not fill the GPU's CTA slots in whole
//                  waves, the j-range of the last ones (or of all, for small
//                  N) is cut into nsplit slices, so the tail of the launch is
//                  made of shorter units that finish together: units
//                  0..nfull-1 are whole i-blocks (launched first), the rest
//                  are (i-block, slice) units.  Each slice writes its (hi, lo)
//                  partials; the last slice of an i-block to finish (atomic
//                  counter) adds the partials of slices 0..nsplit-1 in fixed
//                  order, so the result does not depend on which finishes
//                  last.  Splitting only the tail keeps the partials (32 B per
//                  body and slice) small enough to stay in L2.
//
// The drop-in entry point ComputeGravitation_GPU_GB300 has the reference's
// pfnComputeGravitation_AOS_t signature (src/nbody.h:68) and its conventions
// (device pointers, legacy stream, event-timed milliseconds returned, 0 on
// error, synchronised before return: src/nbody_GPU_Shared.cu:83-103).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "nbgb_device.cuh"
#include "nbgb_internal.h"
#include "nbody_gb300.h"

namespace nbgb {

struct ForceParams {
    const float4 *__restrict__ ipos;     // targets, AOS {x,y,z,m}
    const float4 *__restrict__ jstream;  // sources, paired layout, ntiles*JT bodies
    float4 *__restrict__ force;          // output {fx,fy,fz,0}
    float4 *__restrict__ part_hi;        // [nsplit][ni_split] (split i-blocks only)
    float4 *__restrict__ part_lo;        // [nsplit][ni_split]
    unsigned *__restrict__ counters;     // [split i-blocks]
    int n;
    int ntiles;
    int nsplit;
    int nfull;     // i-blocks 0..nfull-1 are whole units; the rest are split
    int ni_split;  // (nblocks - nfull) * BI
    float eps2;
    FusedIntegrate fi;  // fi.vel == nullptr: forces only
};

// ---------------------------------------------------------------------------
// pack: AOS -> paired j-stream, zero-mass padding, counter reset.
// ---------------------------------------------------------------------------
// One body per thread (coalesced loads; the pairs are assembled with a lane
// swap, store_jstream_body), vpb 1 paired or 2 duplicated layout.  logm != 0
// (log-domain plans): pairs q with q % 4 == 0 carry log2 of their masses
// (jstream_log_mass) instead of the masses.
__global__ void pack_jstream_kernel(const float4 *__restrict__ pm, float4 *__restrict__ js, int n,
                                    int npad, unsigned *__restrict__ counters, int ncounters,
                                    int vpb, int logm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // body
    if (i < ncounters)
        counters[i] = 0u;
    const float4 b = (i < n) ? pm[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    store_jstream_body(js, vpb, logm, i, b, i < npad);
}

// The reference integrator (integrateOne, src/nbody.cu:158-182) applied to
// target i by the unit that produced its final force F: v += (F invMass) dt;
// v *= damping; x += v dt, each operation rounded separately or, fused drift,
// x = fma(v, dt, x) -- the same arithmetic as integrate_reference_kernel, so
// the results are identical.  Writes posMass (mass kept), velInvMass and body
// i's entry of the next step's j-stream (fi.js, the other buffer: the current
// one is still being read by other units).  Only the last unit of an
// i-block writes its targets, after every unit of that i-block has loaded
// them, so no unit reads a target this launch has moved.
__device__ __forceinline__ void fused_integrate(const FusedIntegrate &fi, int i, float x, float y,
                                                float z, float m, float fx, float fy, float fz) {
    float4 v = fi.vel[i];
    const float im = v.w, dt = fi.dt;
    v.x = __fmul_rn(__fadd_rn(v.x, __fmul_rn(__fmul_rn(fx, im), dt)), fi.damping);
    v.y = __fmul_rn(__fadd_rn(v.y, __fmul_rn(__fmul_rn(fy, im), dt)), fi.damping);
    v.z = __fmul_rn(__fadd_rn(v.z, __fmul_rn(__fmul_rn(fz, im), dt)), fi.damping);
    if (fi.fused_drift) {
        x = __fmaf_rn(v.x, dt, x);
        y = __fmaf_rn(v.y, dt, y);
        z = __fmaf_rn(v.z, dt, z);
    } else {
        x = __fadd_rn(x, __fmul_rn(v.x, dt));
        y = __fadd_rn(y, __fmul_rn(v.y, dt));
        z = __fadd_rn(z, __fmul_rn(v.z, dt));
    }
    fi.pm[i] = make_float4(x, y, z, m);
    fi.vel[i] = v;
    const int q = i >> 1, h = i & 1;
    float w = m;
    if (fi.js_log && jstream_log_slot(q))
        w = jstream_log_mass(w);
    if (fi.js_vpb == 2) {
        fi.js[2 * i] = make_float4(x, x, y, y);
        fi.js[2 * i + 1] = make_float4(z, z, w, w);
    } else {
        float *a = reinterpret_cast<float *>(fi.js + 2 * q);
        a[h] = x;
        a[2 + h] = y;
        a[4 + h] = z;
        a[6 + h] = w;
    }
}

// ---------------------------------------------------------------------------
// force kernel
// ---------------------------------------------------------------------------
template <int W, int K, int JT, int STAGES, int MODE, int UNROLL, int MINB>
__global__ void __launch_bounds__(W * 32, MINB) force_kernel(ForceParams p) {
    constexpr int NT = W * 32;
    constexpr int BI = NT * K;
    // float4s per source body in the j-stream: 1 (pairs of sources) or 2
    // (MODE 4: each source duplicated, targets paired in registers)
    constexpr int VPB = (MODE == 4) ? 2 : 1;
    constexpr uint32_t TILE_BYTES = JT * 16u * VPB;
    static_assert(JT % 2 == 0, "tiles hold whole pairs");
    static_assert(MODE != 4 || K % 2 == 0, "targets are paired");
    // Sources summed in plain FP32 before each fold into the compensated
    // (TwoSum) sum: at most 256 (128 per f32x2 half), whatever the tile size.
    constexpr int FLUSH = JT < 256 ? JT : 256;
    static_assert(JT % FLUSH == 0, "tiles hold whole flush chunks");
    static_assert((MODE != 6 && MODE != 7) || (FLUSH % 8 == 0 && (UNROLL < 4 || UNROLL % 4 == 0)),
                  "mode 6 steps through whole groups of 4 source pairs");

    extern __shared__ __align__(128) unsigned char smem_raw[];
    float4 *ring = reinterpret_cast<float4 *>(smem_raw);
    __shared__ __align__(8) uint64_t full[STAGES];
    __shared__ unsigned released[STAGES];  // warps that finished each stage, cumulative
    __shared__ int stage_tile[STAGES];     // tile most recently issued into each stage
    __shared__ int abort_flag;
    __shared__ int s_last;

    const int tid = threadIdx.x;
    const int unit = blockIdx.x;
    // units 0..nfull-1: whole i-blocks; then (i-block, slice) units
    int ib, r, ns;
    if (unit < p.nfull) {
        ib = unit;
        r = 0;
        ns = 1;
    } else {
        const int u = unit - p.nfull;
        ns = p.nsplit;
        ib = p.nfull + u / ns;
        r = u - (ib - p.nfull) * ns;
    }
    const int t_begin = (int)(((long long)r * p.ntiles) / ns);
    const int t_end = (int)(((long long)(r + 1) * p.ntiles) / ns);
    const int nt = t_end - t_begin;

    const int lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full[s], 1);
            released[s] = 0u;
            stage_tile[s] = -1;
        }
        abort_flag = 0;
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < STAGES && s < nt; s++) {
            mbar_expect_tx(&full[s], TILE_BYTES);
            bulk_g2s(ring + s * JT * VPB, p.jstream + (size_t)(t_begin + s) * JT * VPB,
                     TILE_BYTES, &full[s]);
            stage_tile[s] = s;
        }
    }

    // Targets: thread tid owns bodies ib*BI + k*NT + tid (coalesced loads).
    // MODE 5 also accumulates the potential sum_j m_j / r_ij (returned in w)
    constexpr bool POT = (MODE == 5);
    f2 nx[K], ny[K], nz[K];     // packed mode: (-x,-x) etc.
    float px[K], py[K], pz[K];  // scalar mode
    float pm_self[K];           // MODE 5: the target's own mass
    float hx[K], hy[K], hz[K], lx[K], ly[K], lz[K], hp[K], lp[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int i = ib * BI + k * NT + tid;
        float4 b = (i < p.n) ? p.ipos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        px[k] = b.x;
        py[k] = b.y;
        pz[k] = b.z;
        pm_self[k] = b.w;
        hp[k] = lp[k] = 0.f;
        nx[k] = f2_pack(-b.x, -b.x);
        ny[k] = f2_pack(-b.y, -b.y);
        nz[k] = f2_pack(-b.z, -b.z);
        hx[k] = hy[k] = hz[k] = lx[k] = ly[k] = lz[k] = 0.f;
    }
    if constexpr (MODE == 4) {  // pair targets 2c and 2c+1 in one register pair
#pragma unroll
        for (int c = 0; c < K / 2; c++) {
            nx[c] = f2_pack(-px[2 * c], -px[2 * c + 1]);
            ny[c] = f2_pack(-py[2 * c], -py[2 * c + 1]);
            nz[c] = f2_pack(-pz[2 * c], -pz[2 * c + 1]);
        }
    }
    const f2 eps2p = f2_pack(p.eps2, p.eps2);
    const f2 zero2 = f2_pack(0.f, 0.f);
    const f2 one2 = f2_pack(1.f, 1.f);
    const f2 m15 = f2_pack(-1.5f, -1.5f);

    // Ring protocol without CTA-wide barriers: every warp waits for a stage's
    // copy on its mbarrier, reads it, then releases it with an acq_rel add;
    // the warp whose release completes the count for this round issues the
    // copy of tile t + STAGES into the stage.  Waits are bounded; a warp
    // whose wait runs out raises abort_flag and the others follow.
    bool failed = false;
    for (int t = 0; t < nt; t++) {
        const int s = t % STAGES;
        const uint32_t parity = (uint32_t)((t / STAGES) & 1);
        if (__any_sync(0xffffffffu, *(volatile int *)&abort_flag != 0)) {
            failed = true;
            break;
        }
        const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&full[s], parity));
        if (!ok) {
            if (lane == 0)
                *(volatile int *)&abort_flag = 1;
            failed = true;
            break;
        }
        {
            const ulonglong2 *tp = reinterpret_cast<const ulonglong2 *>(ring + s * JT * VPB);
            if constexpr (MODE == 4) {  // targets paired, sources duplicated
                constexpr int KP = K / 2 > 0 ? K / 2 : 1;
                f2 ax[KP], ay[KP], az[KP];
#pragma unroll
                for (int j0 = 0; j0 < JT; j0 += FLUSH) {
#pragma unroll
                for (int c = 0; c < K / 2; c++)
                    ax[c] = ay[c] = az[c] = zero2;
#pragma unroll UNROLL
                for (int j = j0; j < j0 + FLUSH; j++) {
                    const ulonglong2 a = tp[2 * j];      // (x,x) (y,y)
                    const ulonglong2 b = tp[2 * j + 1];  // (z,z) (m,m)
#pragma unroll
                    for (int c = 0; c < K / 2; c++)
                        pair_interact2(a.x, a.y, b.x, b.y, nx[c], ny[c], nz[c], eps2p, ax[c],
                                       ay[c], az[c]);
                }
#pragma unroll
                for (int c = 0; c < K / 2; c++) {
                    float l, h;
                    f2_unpack(ax[c], l, h);
                    comp_add(hx[2 * c], lx[2 * c], l);
                    comp_add(hx[2 * c + 1], lx[2 * c + 1], h);
                    f2_unpack(ay[c], l, h);
                    comp_add(hy[2 * c], ly[2 * c], l);
                    comp_add(hy[2 * c + 1], ly[2 * c + 1], h);
                    f2_unpack(az[c], l, h);
                    comp_add(hz[2 * c], lz[2 * c], l);
                    comp_add(hz[2 * c + 1], lz[2 * c + 1], h);
                }
                }
            } else if constexpr (POT) {  // packed f32x2 with the potential
                f2 ax[K], ay[K], az[K], ap[K];
                for (int q0 = 0; q0 < JT / 2; q0 += FLUSH / 2) {
#pragma unroll
                for (int k = 0; k < K; k++)
                    ax[k] = ay[k] = az[k] = ap[k] = zero2;
#pragma unroll UNROLL
                for (int q = q0; q < q0 + FLUSH / 2; q++) {
                    const ulonglong2 a = tp[2 * q];
                    const ulonglong2 b = tp[2 * q + 1];
#pragma unroll
                    for (int k = 0; k < K; k++)
                        pair_interact2_pot(a.x, a.y, b.x, b.y, nx[k], ny[k], nz[k], eps2p, ax[k],
                                           ay[k], az[k], ap[k]);
                }
#pragma unroll
                for (int k = 0; k < K; k++) {
                    float l, h;
                    f2_unpack(ax[k], l, h);
                    comp_add(hx[k], lx[k], l + h);
                    f2_unpack(ay[k], l, h);
                    comp_add(hy[k], ly[k], l + h);
                    f2_unpack(az[k], l, h);
                    comp_add(hz[k], lz[k], l + h);
                    f2_unpack(ap[k], l, h);
                    comp_add(hp[k], lp[k], l + h);
                }
                }
            } else if constexpr (MODE == 6) {  // f32x2, pair q % 4 == 0 in the log domain
                f2 ax[K], ay[K], az[K];
                constexpr int GROUPS = UNROLL >= 4 ? UNROLL / 4 : 1;
                for (int q0 = 0; q0 < JT / 2; q0 += FLUSH / 2) {
#pragma unroll
                for (int k = 0; k < K; k++)
                    ax[k] = ay[k] = az[k] = zero2;
#pragma unroll GROUPS
                for (int q = q0; q < q0 + FLUSH / 2; q += 4) {
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const ulonglong2 a = tp[2 * (q + u)];
                        const ulonglong2 b = tp[2 * (q + u) + 1];
#pragma unroll
                        for (int k = 0; k < K; k++) {
                            if (u == 0)
                                pair_interact2_log(a.x, a.y, b.x, b.y, nx[k], ny[k], nz[k], eps2p,
                                                   m15, ax[k], ay[k], az[k]);
                            else
                                pair_interact2(a.x, a.y, b.x, b.y, nx[k], ny[k], nz[k], eps2p,
                                               ax[k], ay[k], az[k]);
                        }
                    }
                }
#pragma unroll
                for (int k = 0; k < K; k++) {
                    float l, h;
                    f2_unpack(ax[k], l, h);
                    comp_add(hx[k], lx[k], l + h);
                    f2_unpack(ay[k], l, h);
                    comp_add(hy[k], ly[k], l + h);
                    f2_unpack(az[k], l, h);
                    comp_add(hz[k], lz[k], l + h);
                }
                }
            } else if constexpr (MODE == 7) {  // as 6, next source pair loaded one ahead
                // The operands of pair q + 1 are read from shared memory while
                // pair q is evaluated, across group and flush boundaries, so a
                // group never starts by waiting on its first loads.  The last
                // pair of the tile re-reads itself instead of reaching past it.
                f2 ax[K], ay[K], az[K];
                ulonglong2 a = tp[0], b = tp[1];
                for (int q0 = 0; q0 < JT / 2; q0 += FLUSH / 2) {
#pragma unroll
                for (int k = 0; k < K; k++)
                    ax[k] = ay[k] = az[k] = zero2;
                for (int q = q0; q < q0 + FLUSH / 2; q += 4) {
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int qn = min(q + u + 1, JT / 2 - 1);
                        const ulonglong2 an = tp[2 * qn];
                        const ulonglong2 bn = tp[2 * qn + 1];
#pragma unroll
                        for (int k = 0; k < K; k++) {
                            if (u == 0)
                                pair_interact2_log(a.x, a.y, b.x, b.y, nx[k], ny[k], nz[k], eps2p,
                                                   m15, ax[k], ay[k], az[k]);
                            else
                                pair_interact2(a.x, a.y, b.x, b.y, nx[k], ny[k], nz[k], eps2p,
                                               ax[k], ay[k], az[k]);
                        }
                        a = an;
                        b = bn;
                    }
                }
#pragma unroll
                for (int k = 0; k < K; k++) {
                    float l, h;
                    f2_unpack(ax[k], l, h);
                    comp_add(hx[k], lx[k], l + h);
                    f2_unpack(ay[k], l, h);
                    comp_add(hy[k], ly[k], l + h);
                    f2_unpack(az[k], l, h);
                    comp_add(hz[k], lz[k], l + h);
                }
                }
            } else if constexpr (MODE != 0) {  // packed f32x2 (MODE 2: all ops as FMAs)
                f2 ax[K], ay[K], az[K];
                for (int q0 = 0; q0 < JT / 2; q0 += FLUSH / 2) {
#pragma unroll
                for (int k = 0; k < K; k++)
                    ax[k] = ay[k] = az[k] = zero2;
#pragma unroll UNROLL
                for (int q = q0; q < q0 + FLUSH / 2; q++) {
                    const ulonglong2 a = tp[2 * q];
                    const ulonglong2 b = tp[2 * q + 1];
#pragma unroll
                    for (int k = 0; k < K; k++) {
                        if (MODE == 2)
                            pair_interact2_fma(a.x, a.y, b.x, b.y, nx[k], ny[k], nz[k], eps2p,
                                               one2, zero2, ax[k], ay[k], az[k]);
                        else
                            pair_interact2(a.x, a.y, b.x, b.y, nx[k], ny[k], nz[k], eps2p, ax[k],
                                           ay[k], az[k]);
                    }
                }
#pragma unroll
                for (int k = 0; k < K; k++) {
                    float l, h;
                    f2_unpack(ax[k], l, h);
                    comp_add(hx[k], lx[k], l + h);
                    f2_unpack(ay[k], l, h);
                    comp_add(hy[k], ly[k], l + h);
                    f2_unpack(az[k], l, h);
                    comp_add(hz[k], lz[k], l + h);
                }
                }
            } else {
                float ax[K], ay[K], az[K];
                const float4 *tf = reinterpret_cast<const float4 *>(tp);
                for (int q0 = 0; q0 < JT / 2; q0 += FLUSH / 2) {
#pragma unroll
                for (int k = 0; k < K; k++)
                    ax[k] = ay[k] = az[k] = 0.f;
#pragma unroll UNROLL
                for (int q = q0; q < q0 + FLUSH / 2; q++) {
                    const float4 a = tf[2 * q];      // x0 x1 y0 y1
                    const float4 b = tf[2 * q + 1];  // z0 z1 m0 m1
#pragma unroll
                    for (int k = 0; k < K; k++) {
                        pair_interact1(a.x, a.z, b.x, b.z, px[k], py[k], pz[k], p.eps2, ax[k],
                                       ay[k], az[k]);
                        pair_interact1(a.y, a.w, b.y, b.w, px[k], py[k], pz[k], p.eps2, ax[k],
                                       ay[k], az[k]);
                    }
                }
#pragma unroll
                for (int k = 0; k < K; k++) {
                    comp_add(hx[k], lx[k], ax[k]);
                    comp_add(hy[k], ly[k], ay[k]);
                    comp_add(hz[k], lz[k], az[k]);
                }
                }
            }
        }
        __syncwarp();
        if (lane == 0) {
            const unsigned round = (unsigned)(t / STAGES) + 1u;
            const unsigned prev = atom_add_acqrel_shared(&released[s], 1u);
            if (prev == round * W - 1u && t + STAGES < nt) {
                fence_proxy_async_shared();
                mbar_expect_tx(&full[s], TILE_BYTES);
                bulk_g2s(ring + s * JT * VPB,
                         p.jstream + (size_t)(t_begin + t + STAGES) * JT * VPB, TILE_BYTES,
                         &full[s]);
                stage_tile[s] = t + STAGES;
            }
        }
    }
    // Every warp reaches this barrier (all waits are bounded).  After a
    // timeout no warp issues copies any more; the last copy issued into each
    // stage is waited for (bounded again) so no copy is still landing in
    // shared memory when the CTA exits, and nothing is written.
    if (__syncthreads_or(failed)) {
        if (tid == 0)
            for (int s = 0; s < STAGES; s++)
                if (stage_tile[s] >= 0)
                    (void)mbar_wait_bounded(&full[s], (uint32_t)((stage_tile[s] / STAGES) & 1),
                                            100000000ull);
        return;
    }

    // MODE 5: w = -(sum_{j != i} m_j / r_ij); the self term the loop added is
    // m_i * rsqrt(eps2), evaluated exactly as in the loop.
    float self[K];
#pragma unroll
    for (int k = 0; k < K; k++)
        self[k] = POT ? pm_self[k] * rsqrt_mufu(p.eps2) : 0.f;

    if (ns == 1) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int i = ib * BI + k * NT + tid;
            if (i < p.n) {
                const float fx = hx[k] + lx[k], fy = hy[k] + ly[k], fz = hz[k] + lz[k];
                p.force[i] = make_float4(fx, fy, fz, POT ? -((hp[k] - self[k]) + lp[k]) : 0.f);
                if (!POT && p.fi.vel)
                    fused_integrate(p.fi, i, px[k], py[k], pz[k], pm_self[k], fx, fy, fz);
            }
        }
        return;
    }

    // Split j-range: publish partials, the last unit of the i-block combines.
    const int sb = ib - p.nfull;  // index among the split i-blocks
#pragma unroll
    for (int k = 0; k < K; k++) {
        const size_t o = (size_t)r * p.ni_split + (size_t)(sb * BI + k * NT + tid);
        p.part_hi[o] = make_float4(hx[k], hy[k], hz[k], hp[k]);
        p.part_lo[o] = make_float4(lx[k], ly[k], lz[k], lp[k]);
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        const unsigned prev = atomicAdd(&p.counters[sb], 1u);
        s_last = (prev == (unsigned)(ns - 1));
        if (s_last)
            p.counters[sb] = 0u;  // ready for the next launch
    }
    __syncthreads();
    if (!s_last)
        return;
    __threadfence();
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int i = ib * BI + k * NT + tid;
        if (i >= p.n)
            continue;
        float Hx = 0.f, Hy = 0.f, Hz = 0.f, Lx = 0.f, Ly = 0.f, Lz = 0.f, Hp = 0.f, Lp = 0.f;
        for (int rr = 0; rr < ns; rr++) {
            float4 h, l;
            if (rr == r) {
                h = make_float4(hx[k], hy[k], hz[k], hp[k]);
                l = make_float4(lx[k], ly[k], lz[k], lp[k]);
            } else {
                const size_t o = (size_t)rr * p.ni_split + (size_t)(sb * BI + k * NT + tid);
                h = __ldcg(p.part_hi + o);
                l = __ldcg(p.part_lo + o);
            }
            comp_add(Hx, Lx, h.x);
            comp_add(Hy, Ly, h.y);
            comp_add(Hz, Lz, h.z);
            Lx += l.x;
            Ly += l.y;
            Lz += l.z;
            if (POT) {
                comp_add(Hp, Lp, h.w);
                Lp += l.w;
            }
        }
        const float fx = Hx + Lx, fy = Hy + Ly, fz = Hz + Lz;
        p.force[i] = make_float4(fx, fy, fz, POT ? -((Hp - self[k]) + Lp) : 0.f);
        if (!POT && p.fi.vel)
            fused_integrate(p.fi, i, px[k], py[k], pz[k], pm_self[k], fx, fy, fz);
    }
}

// ---------------------------------------------------------------------------
// Configurations.  The planner picks one per N (or a caller forces one).
// ---------------------------------------------------------------------------
struct ForceConfig {
    int warps, k, jt, stages;
    int mode;  // 0 scalar FP32, 1 packed f32x2 (source pairs), 2 as 1 with every
               // op as an FMA, 4 packed f32x2 (target pairs, duplicated sources),
               // 5 as 1 plus the potential in w, 6 as 1 with every fourth source
               // pair in the log domain (j-stream with log2 masses there), 7 as
               // 6 with each source pair read one pair ahead
    const void *fn;
    const char *name;
};

// W warps, K targets per thread, JT sources per tile, ST ring stages, mode
// (0 scalar, 1 f32x2, 2 f32x2 all-FMA, 4 f32x2 target pairs, 5 f32x2 with
// potential, 6 f32x2 with log-domain pairs), inner unroll, minimum resident
// CTAs (register cap).
#define NBGB_CFG(W, K, JT, ST, PK, UN, MB, PIPE)                                           \
    {W, K, JT, ST, PK, (const void *)force_kernel<W, K, JT, ST, PK, UN, MB>,               \
     "w" #W "_k" #K "_jt" #JT "_s" #ST "_" PIPE}

static const ForceConfig kConfigs[] = {
    NBGB_CFG(8, 4, 512, 3, 1, 4, 2, "f32x2"),  // 0: BI 1024
    NBGB_CFG(4, 4, 512, 3, 1, 4, 4, "f32x2"),  // 1: BI 512
    NBGB_CFG(8, 2, 256, 4, 1, 8, 2, "f32x2"),  // 2: BI 512
    NBGB_CFG(4, 2, 256, 4, 1, 8, 4, "f32x2"),  // 3: BI 256
    NBGB_CFG(8, 4, 512, 3, 0, 4, 2, "f32"),   // 4: scalar FP32 pipe, BI 1024
    NBGB_CFG(4, 8, 512, 3, 1, 2, 2, "f32x2"),  // 5: BI 1024, 8 targets per thread
    NBGB_CFG(8, 2, 256, 4, 1, 8, 3, "f32x2"),  // 6: as 2, 3 CTAs/SM (<= 85 regs)
    NBGB_CFG(8, 4, 512, 3, 1, 2, 2, "f32x2"),  // 7: as 0, unroll 2
    NBGB_CFG(4, 4, 512, 3, 1, 8, 3, "f32x2"),  // 8: as 1, unroll 8
    NBGB_CFG(16, 2, 256, 4, 1, 8, 1, "f32x2"), // 9: 512 threads
    NBGB_CFG(8, 2, 256, 4, 1, 4, 2, "f32x2"),  // 10: as 2, unroll 4
    NBGB_CFG(8, 2, 256, 4, 1, 16, 2, "f32x2"), // 11: as 2, unroll 16
    NBGB_CFG(8, 2, 256, 4, 0, 8, 3, "f32"),   // 12: scalar, K 2
    NBGB_CFG(8, 1, 256, 4, 1, 16, 3, "f32x2"), // 13: K 1, 3 CTAs/SM
    NBGB_CFG(8, 2, 256, 4, 2, 4, 2, "fma2"),   // 14: as 10, all-FMA
    NBGB_CFG(4, 8, 512, 3, 2, 2, 2, "fma2"),   // 15: as 5, all-FMA
    NBGB_CFG(8, 2, 256, 4, 2, 8, 2, "fma2"),   // 16: as 2, all-FMA
    NBGB_CFG(16, 2, 256, 4, 2, 4, 1, "fma2"),  // 17: as 9, all-FMA, unroll 4
    NBGB_CFG(8, 4, 256, 4, 4, 4, 2, "tpair"),  // 18: target pairs, K 4
    NBGB_CFG(8, 2, 256, 4, 4, 8, 3, "tpair"),  // 19: target pairs, K 2, 3 CTAs/SM
    NBGB_CFG(8, 4, 256, 4, 4, 8, 2, "tpair"),  // 20: target pairs, K 4, unroll 8
    NBGB_CFG(8, 6, 256, 4, 4, 4, 2, "tpair"),  // 21: target pairs, K 6
    NBGB_CFG(4, 4, 256, 4, 4, 4, 4, "tpair"),  // 22: target pairs, K 4, 128 threads
    NBGB_CFG(8, 2, 256, 4, 5, 4, 2, "pot"),    // 23: force + potential (diagnostics)
    NBGB_CFG(8, 2, 512, 3, 1, 4, 2, "f32x2"),  // 24: as 10, 512-body tiles
    NBGB_CFG(8, 2, 1024, 2, 1, 4, 2, "f32x2"), // 25: as 10, 1024-body tiles
    NBGB_CFG(8, 2, 128, 6, 1, 4, 2, "f32x2"),  // 26: as 10, 128-body tiles
    NBGB_CFG(8, 2, 1024, 2, 6, 4, 2, "log4"),  // 27: as 25, log-domain pairs
    NBGB_CFG(8, 2, 512, 3, 6, 4, 2, "log4"),   // 28: as 24, log-domain pairs
    NBGB_CFG(8, 2, 256, 4, 6, 4, 2, "log4"),   // 29: as 10, log-domain pairs
    NBGB_CFG(8, 2, 1024, 2, 6, 8, 2, "log4"),  // 30: as 27, unroll 8
    NBGB_CFG(8, 4, 512, 3, 6, 4, 2, "log4"),   // 31: as 0, log-domain pairs
    NBGB_CFG(4, 2, 256, 4, 6, 8, 4, "log4"),   // 32: as 3, log-domain pairs
    NBGB_CFG(8, 3, 1024, 2, 6, 4, 2, "log4"),  // 33: as 27, 3 targets per thread
    NBGB_CFG(8, 3, 512, 3, 6, 4, 2, "log4"),   // 34: as 28, 3 targets per thread
    NBGB_CFG(8, 2, 2048, 2, 6, 4, 2, "log4"),  // 35: as 27, 2048-body tiles
    NBGB_CFG(6, 2, 1024, 2, 6, 4, 3, "log4"),  // 36: as 27, 6 warps x 3 CTAs/SM (18 warps)
    NBGB_CFG(9, 2, 1024, 2, 6, 4, 2, "log4"),  // 37: as 27, 9 warps x 2 CTAs/SM (18 warps)
    NBGB_CFG(5, 2, 1024, 2, 6, 4, 4, "log4"),  // 38: as 27, 5 warps x 4 CTAs/SM (20 warps)
    NBGB_CFG(6, 2, 2048, 2, 6, 4, 3, "log4"),  // 39: as 36, 2048-body tiles
    NBGB_CFG(6, 3, 1024, 2, 6, 4, 2, "log4"),  // 40: 3 targets per thread, 12 warps
    NBGB_CFG(7, 2, 1024, 2, 6, 4, 3, "log4"),  // 41: as 27, 7 warps x 3 CTAs/SM (21 warps)
    NBGB_CFG(10, 2, 1024, 2, 6, 4, 2, "log4"), // 42: as 27, 10 warps x 2 CTAs/SM (20 warps)
    NBGB_CFG(4, 2, 1024, 2, 6, 4, 5, "log4"),  // 43: as 27, 4 warps x 5 CTAs/SM (20 warps)
    NBGB_CFG(8, 4, 1024, 2, 6, 4, 2, "log4"),  // 44: as 27, 4 targets per thread
    NBGB_CFG(8, 2, 1024, 3, 6, 4, 2, "log4"),  // 45: as 27, 3 ring stages
    NBGB_CFG(8, 2, 1024, 2, 7, 4, 2, "pf_log4"),  // 46: as 27, sources loaded a pair ahead
    NBGB_CFG(8, 2, 2048, 2, 7, 4, 2, "pf_log4"),  // 47: as 46, 2048-body tiles
};
static const int kNumConfigs = (int)(sizeof(kConfigs) / sizeof(kConfigs[0]));
// Relative throughput of each configuration (interactions/s per resident
// CTA slot, normalised to configuration 25), measured on a GB300 at
// N = 1,048,576 Plummer; the planner divides its wave cost by it.  An
// autotuner can replace the values at run time (nbgb_force_set_speed).
static double g_speed[] = {
    0.943, 0.934, 0.981, 0.970, 0.902, 0.981, 0.955, 0.954, 0.962, 0.973,  // 0-9
    0.990, 0.966, 0.873, 0.936, 0.987, 0.981, 0.981, 0.982, 0.981, 0.928,  // 10-19
    0.987, 0.951, 0.974, 0.900, 0.997, 1.000, 0.977, 1.057, 1.030, 1.026,  // 20-29
    1.034, 1.009, 1.016, 0.997, 1.020, 1.057, 1.000, 1.000, 1.000, 1.000,  // 30-39
    1.000, 1.000, 1.000, 1.000, 1.000, 1.060, 1.000, 1.000,                // 40-47
};
static_assert(sizeof(g_speed) / sizeof(g_speed[0]) == sizeof(kConfigs) / sizeof(kConfigs[0]),
              "one speed per configuration");
static const int kDefaultCandidates[] = {45, 27, 28, 29, 30, 31, 32, 25, 24, 10, 20, 2, 3, 5};
// Candidates without log-domain pairs, for masses that have no logarithm
// (negative masses).
static const int kRsqrtCandidates[] = {25, 24, 10, 20, 2, 3, 5};

static inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

constexpr int kMaxConfigs = 64;
static_assert(sizeof(kConfigs) / sizeof(kConfigs[0]) <= (size_t)kMaxConfigs,
              "DeviceInfo::occ must hold every configuration");

// Per device: SM count and resident CTAs per SM of every configuration.
// Filling it also sets the kernels' dynamic shared-memory attributes, which
// belong to the context, so the entry is refilled when the context changes
// (cudaDeviceReset).
struct DeviceInfo {
    int sms = 0;
    int occ[kMaxConfigs] = {0};
    bool ok = false;
    unsigned long long ctx = 0;
};

static std::mutex g_dev_mu;
static DeviceInfo g_dev[64];

static const DeviceInfo *device_info() {
    int dev = 0;
    unsigned long long ctx = 0;
    if (current_context(&dev, &ctx) != NBGB_OK || dev < 0 || dev >= 64)
        return nullptr;
    std::lock_guard<std::mutex> lk(g_dev_mu);
    DeviceInfo &d = g_dev[dev];
    if (d.ok && d.ctx == ctx)
        return &d;
    d.ok = false;
    d.ctx = ctx;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
        return nullptr;
    d.sms = prop.multiProcessorCount;
    for (int c = 0; c < kNumConfigs; c++) {
        const ForceConfig &cf = kConfigs[c];
        const size_t smem = (size_t)cf.stages * cf.jt * 16 * (cf.mode == 4 ? 2 : 1);
        if (cudaFuncSetAttribute(cf.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return nullptr;
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, cf.fn, cf.warps * 32, smem) !=
            cudaSuccess)
            return nullptr;
        d.occ[c] = occ;
    }
    d.ok = true;
    return &d;
}

// n sources; nt targets (0: the same n bodies).
static void fill_layout(ForcePlan &pl, size_t n, size_t nt = 0) {
    const ForceConfig &cf = kConfigs[pl.config];
    const size_t bi = (size_t)cf.warps * 32 * cf.k;
    pl.n = n;
    pl.nt = nt;
    pl.block_bodies = (int)bi;
    pl.tile_bodies = cf.jt;
    pl.js_vpb = cf.mode == 4 ? 2 : 1;
    pl.js_log = (cf.mode == 6 || cf.mode == 7) ? 1 : 0;
    pl.nblocks = (int)(((nt ? nt : n) + bi - 1) / bi);
    pl.ntiles = (int)((n + cf.jt - 1) / cf.jt);
    pl.ni_pad = (size_t)pl.nblocks * bi;
    if (pl.nsplit == 1 || pl.nfull > pl.nblocks)
        pl.nfull = pl.nblocks;
    pl.off_js = 0;
    size_t o = align_up((size_t)pl.ntiles * cf.jt * 16 * pl.js_vpb, 256);
    const size_t sbk = (size_t)split_blocks(pl);
    if (sbk) {
        pl.off_hi = o;
        o = align_up(o + (size_t)pl.nsplit * sbk * bi * 16, 256);
        pl.off_lo = o;
        o = align_up(o + (size_t)pl.nsplit * sbk * bi * 16, 256);
        pl.off_cnt = o;
        o = align_up(o + sbk * 4, 256);
    } else {
        pl.off_hi = pl.off_lo = pl.off_cnt = 0;
    }
    pl.workspace_bytes = o;
}

// Cost model, fitted to graph-timed sweeps of the log-domain configurations
// x slice counts at N = 1,000-2^20 on GB300 (its plan is within 4 % of the
// fastest measured one at every size; the earlier wave-count model was up to
// 48 % off below N = 131,072).  Time is counted in interactions one SM
// evaluates at full occupancy, scaled by the configuration's measured
// relative speed.  Units are dealt to the SMs in rounds of `occ` co-resident
// CTAs and a round lasts as long as its busiest SM: a full round runs occ
// units at the SM's full throughput, a last partial round k units at the
// throughput k resident CTAs reach, share(k) = (1 - e^{-kW/tau}) /
// (1 - e^{-occ W/tau}) with W warps per CTA and tau = 1.8 warps (eight warps
// nearly saturate the pipes, four do not).  Every round also pays a fixed
// latency (the first j-tile's copy, the epilogue), every unit a small
// overhead, and a split i-block's combining unit reads one partial per
// slice.  SMs do not run at exactly the same speed, and the launch ends with
// the slowest: a tenth of one final-round unit's time is added, so the last
// units are kept short (at N = 2^20, the 224 leftover i-blocks split 19 ways
// rather than 4: 0.6 % faster).  For each configuration and slice count
// s > 1 two decompositions are costed: every i-block split s ways, and only
// the i-blocks left over after whole rounds of whole i-blocks split
// (nfull = whole rounds x slots).  Of the plans within 0.2 % of the
// cheapest, the one with the smallest workspace wins.
constexpr double kUnitOverhead = 9.0;      // sources per unit and target
constexpr double kCombinePerSlice = 37.0;  // sources per slice and target, combining unit
constexpr double kRoundLatency = 29800.0;  // about 1.5 us of one SM's interactions
constexpr double kWarpTau = 1.8;
constexpr double kLastUnitShare = 0.1;     // of one final-round unit's time

static double sm_share(int k, int warps, int occ) {
    return (1.0 - std::exp(-(double)k * warps / kWarpTau)) /
           (1.0 - std::exp(-(double)occ * warps / kWarpTau));
}

// `units` equal units of `sources` sources x bi targets; *k_last: resident
// units per SM in the last round; *unit_time: one unit's time in a full
// round.
static double rounds_time(long long units, double sources, double bi, int sms, int occ,
                          int warps, double speed, int *k_last, double *unit_time) {
    const long long slots = (long long)sms * occ;
    const double w = bi * (sources + kUnitOverhead) / speed;
    const long long full = units / slots, r = units % slots;
    double t = (double)full * (occ * w + kRoundLatency);
    *k_last = occ;
    *unit_time = occ * w;
    if (r) {
        const int k = (int)((r + sms - 1) / sms);
        t += k * w / sm_share(k, warps, occ) + kRoundLatency;
        *k_last = k;
    }
    return t;
}

// nfull whole i-blocks, then the remaining nb - nfull i-blocks split s ways.
static double plan_cost(const ForceConfig &cf, int occ, int sms, long long nb, long long ntl,
                        int s, long long nfull, double speed) {
    const double bi = (double)cf.warps * 32 * cf.k;
    double t = 0.0, last_unit = 0.0;
    int k_last = occ;
    if (nfull > 0)
        t += rounds_time(nfull, (double)ntl * cf.jt, bi, sms, occ, cf.warps, speed, &k_last,
                         &last_unit);
    if (nb > nfull) {
        if (s == 1) {
            t += rounds_time(nb - nfull, (double)ntl * cf.jt, bi, sms, occ, cf.warps, speed,
                             &k_last, &last_unit);
        } else {
            t += rounds_time((nb - nfull) * s, std::ceil((double)ntl / s) * cf.jt, bi, sms, occ,
                             cf.warps, speed, &k_last, &last_unit);
            t += s * kCombinePerSlice * bi / (speed * sm_share(k_last, cf.warps, occ));
        }
    }
    return t + kLastUnitShare * last_unit;
}

// Enumerates the candidate decompositions of n sources / nt targets over
// cands; keep(plan) may reject one (e.g. a workspace limit).  Among the
// candidates within kPlanTie of the cheapest, the one with the smallest
// workspace (fewest partial sums) is written to pl.
constexpr double kPlanTie = 2e-3;

// d: the device's SM count and resident CTAs per configuration (the current
// device's when null).
template <typename Keep>
static int plan_enumerate(size_t n, size_t nt, const int *cands, int ncands, int force_nsplit,
                          ForcePlan &pl, Keep keep, const DeviceInfo *d = nullptr) {
    if (!d)
        d = device_info();
    if (!d)
        return NBGB_ERR_CUDA;
    std::vector<std::pair<double, ForcePlan>> kept;
    double best = 1e300;
    for (int ci = 0; ci < ncands; ci++) {
        const int c = cands[ci];
        const ForceConfig &cf = kConfigs[c];
        const int occ = d->occ[c];
        if (occ <= 0)
            continue;
        const long long slots = (long long)d->sms * occ;
        const long long bi = (long long)cf.warps * 32 * cf.k;
        const long long nb = ((long long)(nt ? nt : n) + bi - 1) / bi;
        const long long ntl = ((long long)n + cf.jt - 1) / cf.jt;
        // force_nsplit > 0: every i-block split that many ways; <= -2: whole
        // i-blocks for the whole rounds they fill, the rest split -force_nsplit
        // ways (every i-block split when they fill no whole round)
        const bool tail_only = force_nsplit <= -2;
        int s_lo = 1, s_hi = (int)std::min<long long>(ntl, 256);
        if (force_nsplit > 0 || tail_only)
            s_lo = s_hi = (int)std::min<long long>(tail_only ? -(long long)force_nsplit
                                                             : (long long)force_nsplit,
                                                   ntl);
        for (int s = s_lo; s <= s_hi; s++) {
            // candidates (whole i-blocks, cost); s == 1: every block whole
            long long opt_full[2];
            double opt_t[2];
            int nopt = 0;
            if (s == 1) {
                opt_full[nopt] = nb;
                opt_t[nopt++] = plan_cost(cf, occ, d->sms, nb, ntl, 1, nb, g_speed[c]);
            } else {
                const long long whole = force_nsplit > 0 ? 0 : (nb / slots) * slots;
                const bool has_tail = whole > 0 && whole < nb;
                if (has_tail) {  // tail-only split first: wins ties
                    opt_full[nopt] = whole;
                    opt_t[nopt++] = plan_cost(cf, occ, d->sms, nb, ntl, s, whole, g_speed[c]);
                }
                if (!(tail_only && has_tail)) {
                    opt_full[nopt] = 0;
                    opt_t[nopt++] = plan_cost(cf, occ, d->sms, nb, ntl, s, 0, g_speed[c]);
                }
            }
            for (int k = 0; k < nopt; k++) {
                const long long units = opt_full[k] + (nb - opt_full[k]) * s;
                if (units > (1ll << 31) - 1 || !(opt_t[k] < best * (1.0 + kPlanTie)))
                    continue;
                ForcePlan cand;
                cand.config = c;
                cand.nsplit = s;
                cand.nfull = (int)opt_full[k];
                fill_layout(cand, n, nt);
                if (!keep(cand))
                    continue;
                best = std::min(best, opt_t[k]);
                kept.emplace_back(opt_t[k], cand);
            }
        }
    }
    // enumeration order decides among equal workspaces (first wins)
    bool found = false;
    for (const auto &e : kept)
        if (e.first <= best * (1.0 + kPlanTie) &&
            (!found || e.second.workspace_bytes < pl.workspace_bytes)) {
            pl = e.second;
            found = true;
        }
    return found ? NBGB_OK : NBGB_ERR_UNSUPPORTED;
}

static int plan_force_among(size_t n, const std::vector<int> &cands, int force_nsplit,
                            ForcePlan &pl, size_t nt = 0, const DeviceInfo *d = nullptr) {
    return plan_enumerate(
        n, nt, cands.data(), (int)cands.size(), force_nsplit, pl,
        [](const ForcePlan &) { return true; }, d);
}

static int plan_force_on(size_t n, int force_config, int force_nsplit, ForcePlan &pl,
                         const DeviceInfo *d) {
    if (n == 0 || n > kMaxBodies)
        return NBGB_ERR_INVALID_ARGUMENT;
    std::vector<int> cands;
    if (force_config >= 0) {
        if (force_config >= kNumConfigs)
            return NBGB_ERR_INVALID_ARGUMENT;
        cands.push_back(force_config);
    } else {
        cands.assign(std::begin(kDefaultCandidates), std::end(kDefaultCandidates));
    }
    return plan_force_among(n, cands, force_nsplit, pl, 0, d);
}

int plan_force(size_t n, int force_config, int force_nsplit, ForcePlan &pl) {
    return plan_force_on(n, force_config, force_nsplit, pl, nullptr);
}

int plan_force_rows(size_t n, size_t rows, ForcePlan &pl) {
    if (n == 0 || n > kMaxBodies || rows == 0 || rows > n)
        return NBGB_ERR_INVALID_ARGUMENT;
    return plan_force_among(n,
                            std::vector<int>(std::begin(kDefaultCandidates),
                                             std::end(kDefaultCandidates)),
                            -1, pl, rows);
}

int plan_force_rsqrt(size_t n, ForcePlan &pl) {
    if (n == 0 || n > kMaxBodies)
        return NBGB_ERR_INVALID_ARGUMENT;
    return plan_force_among(n, std::vector<int>(std::begin(kRsqrtCandidates),
                                                std::end(kRsqrtCandidates)),
                            -1, pl);
}

// The best plan (same cost model as plan_force) whose workspace fits in
// max_bytes; NBGB_ERR_TOO_LARGE when none does.  Used by the fixed-scratch
// entry point.
int plan_force_within(size_t n, size_t max_bytes, ForcePlan &pl) {
    if (n == 0 || n > kMaxBodies)
        return NBGB_ERR_INVALID_ARGUMENT;
    const int rc = plan_enumerate(
        n, 0, kDefaultCandidates, (int)(sizeof(kDefaultCandidates) / sizeof(int)), -1, pl,
        [max_bytes](const ForcePlan &c) { return c.workspace_bytes <= max_bytes; });
    return rc == NBGB_ERR_UNSUPPORTED ? NBGB_ERR_TOO_LARGE : rc;
}

int launch_force(const ForcePlan &pl, float4 *force, const float4 *posMass, const float4 *jstream,
                 float eps2, void *workspace, cudaStream_t stream, const FusedIntegrate *fi) {
    const ForceConfig &cf = kConfigs[pl.config];
    char *ws = (char *)workspace;
    ForceParams p;
    p.ipos = posMass;
    p.jstream = jstream ? jstream : (const float4 *)(ws + pl.off_js);
    p.force = force;
    const bool split = split_blocks(pl) > 0;
    p.part_hi = split ? (float4 *)(ws + pl.off_hi) : nullptr;
    p.part_lo = split ? (float4 *)(ws + pl.off_lo) : nullptr;
    p.counters = split ? (unsigned *)(ws + pl.off_cnt) : nullptr;
    p.n = (int)plan_targets(pl);
    p.ntiles = pl.ntiles;
    p.nsplit = pl.nsplit;
    p.nfull = pl.nfull;
    p.ni_split = split_blocks(pl) * pl.block_bodies;
    p.eps2 = eps2;
    if (fi) {
        if (!fi->vel || !fi->pm || !fi->js || pl.nt || cf.mode == 5)
            return NBGB_ERR_INVALID_ARGUMENT;
        p.fi = *fi;
        p.fi.js_vpb = pl.js_vpb;
        p.fi.js_log = pl.js_log;
    } else {
        p.fi = FusedIntegrate{};
    }
    const size_t smem = (size_t)cf.stages * cf.jt * 16 * pl.js_vpb;
    void *args[] = {&p};
    const unsigned grid = (unsigned)plan_units(pl);
    cudaError_t e = cudaLaunchKernel(cf.fn, dim3(grid), dim3(cf.warps * 32), args, smem, stream);
    return e == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

int launch_pack(const ForcePlan &pl, const float4 *posMass, void *workspace, cudaStream_t stream,
                float4 *js_out) {
    char *ws = (char *)workspace;
    float4 *js = js_out ? js_out : (float4 *)(ws + pl.off_js);
    unsigned *cnt = (!js_out && split_blocks(pl)) ? (unsigned *)(ws + pl.off_cnt) : nullptr;
    const int npad = pl.ntiles * pl.tile_bodies;
    const int ncnt = cnt ? split_blocks(pl) : 0;
    const int work = std::max(npad, ncnt);
    const int tb = 256;
    pack_jstream_kernel<<<(work + tb - 1) / tb, tb, 0, stream>>>(posMass, js, (int)pl.n, npad, cnt,
                                                                  ncnt, pl.js_vpb, pl.js_log);
    return cudaGetLastError() == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

const char *config_name(int c) { return (c >= 0 && c < kNumConfigs) ? kConfigs[c].name : "?"; }
int num_configs() { return kNumConfigs; }

// Self-test of the bounded-wait path: one CTA waits on an mbarrier that
// nothing ever completes, with a limit of limit_ns; the wait gives up, sets
// NBGB_STATUS_WAIT_TIMEOUT and the kernel returns normally.
__global__ void selftest_wait_kernel(unsigned long long limit_ns, int *out) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&bar, 0u, limit_ns);
    if (threadIdx.x == 0)
        *out = ok ? 1 : 0;
}

static NBGB_STATUS_READER(read_status_force)

int read_and_clear_status(unsigned *bits) {
    *bits = 0;
    int rc = read_status_force(bits);
    if (rc == NBGB_OK)
        rc = read_status_ensemble(bits);
    if (rc == NBGB_OK)
        rc = read_status_integrate(bits);
    return rc;
}

// Workspace cache for the drop-in entry point (one per device, grow-only).
// The pointer belongs to the context it was allocated in: after a
// cudaDeviceReset (a new context id) it is dropped without being freed --
// the reset already released it.
struct WsCache {
    void *ptr = nullptr;
    size_t bytes = 0;
    unsigned long long ctx = 0;
};
static std::mutex g_ws_mu;
static WsCache g_ws[64];

static void *cached_workspace(size_t bytes) {
    int dev = 0;
    unsigned long long ctx = 0;
    if (current_context(&dev, &ctx) != NBGB_OK || dev < 0 || dev >= 64)
        return nullptr;
    std::lock_guard<std::mutex> lk(g_ws_mu);
    WsCache &w = g_ws[dev];
    if (w.ptr && w.ctx != ctx) {
        w.ptr = nullptr;
        w.bytes = 0;
    }
    if (w.bytes >= bytes && w.ptr)
        return w.ptr;
    if (w.ptr) {
        cudaFree(w.ptr);
        w.ptr = nullptr;
        w.bytes = 0;
    }
    w.ctx = ctx;
    if (cudaMalloc(&w.ptr, bytes) != cudaSuccess) {
        w.ptr = nullptr;
        return nullptr;
    }
    w.bytes = bytes;
    return w.ptr;
}

void release_workspaces() {
    std::lock_guard<std::mutex> lk(g_ws_mu);
    int cur = 0;
    cudaGetDevice(&cur);
    for (int d = 0; d < 64; d++) {
        if (g_ws[d].ptr) {
            int dev = -1;
            unsigned long long ctx = 0;
            // free only what the device's current context still owns
            if (cudaSetDevice(d) == cudaSuccess && current_context(&dev, &ctx) == NBGB_OK &&
                dev == d && ctx == g_ws[d].ctx)
                cudaFree(g_ws[d].ptr);
            g_ws[d].ptr = nullptr;
            g_ws[d].bytes = 0;
        }
    }
    cudaSetDevice(cur);
}

}  // namespace nbgb

using namespace nbgb;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

NBGB_API size_t nbgb_force_workspace_bytes(size_t N) {
    ForcePlan pl;
    if (plan_force(N, -1, -1, pl) != NBGB_OK)
        return 0;
    return pl.workspace_bytes;
}

// The planner without a GPU: the same decision for a device with `sms` SMs
// and occupancy[c] resident CTAs per SM of configuration c (all
// configurations; nbgb_force_device_info reports a real device's).
NBGB_API int nbgb_force_plan_on(size_t N, int sms, const int *occupancy, int nconfigs, int config,
                                int nsplit, int *out_config, int *out_nsplit, int *out_nfull,
                                size_t *out_workspace_bytes) {
    if (sms <= 0 || !occupancy || nconfigs != kNumConfigs)
        return NBGB_ERR_INVALID_ARGUMENT;
    DeviceInfo d;
    d.sms = sms;
    for (int c = 0; c < kNumConfigs; c++) {
        if (occupancy[c] < 0)
            return NBGB_ERR_INVALID_ARGUMENT;
        d.occ[c] = occupancy[c];
    }
    d.ok = true;
    ForcePlan pl;
    int rc = plan_force_on(N, config, nsplit, pl, &d);
    if (rc != NBGB_OK)
        return rc;
    if (out_config)
        *out_config = pl.config;
    if (out_nsplit)
        *out_nsplit = pl.nsplit;
    if (out_nfull)
        *out_nfull = pl.nfull;
    if (out_workspace_bytes)
        *out_workspace_bytes = pl.workspace_bytes;
    return NBGB_OK;
}

// The current device's SM count and resident CTAs per SM of every
// configuration (as the planner sees them).
NBGB_API int nbgb_force_device_info(int *sms, int *occupancy, int nconfigs) {
    if (!sms || !occupancy || nconfigs < kNumConfigs)
        return NBGB_ERR_INVALID_ARGUMENT;
    const DeviceInfo *d = device_info();
    if (!d)
        return NBGB_ERR_CUDA;
    *sms = d->sms;
    for (int c = 0; c < kNumConfigs; c++)
        occupancy[c] = d->occ[c];
    return NBGB_OK;
}

NBGB_API int nbgb_force_plan(size_t N, int config, int nsplit, int *out_config, int *out_nsplit,
                             size_t *out_workspace_bytes) {
    ForcePlan pl;
    int rc = plan_force(N, config, nsplit, pl);
    if (rc != NBGB_OK)
        return rc;
    if (out_config)
        *out_config = pl.config;
    if (out_nsplit)
        *out_nsplit = pl.nsplit;
    if (out_workspace_bytes)
        *out_workspace_bytes = pl.workspace_bytes;
    return NBGB_OK;
}

NBGB_API const char *nbgb_force_config_name(int config) { return config_name(config); }

NBGB_API int nbgb_force_set_speed(int config, double speed) {
    if (config < 0 || config >= kNumConfigs || !(speed > 0.0))
        return NBGB_ERR_INVALID_ARGUMENT;
    g_speed[config] = speed;
    return NBGB_OK;
}

NBGB_API double nbgb_force_get_speed(int config) {
    return (config >= 0 && config < kNumConfigs) ? g_speed[config] : 0.0;
}
NBGB_API int nbgb_force_num_configs(void) { return num_configs(); }

NBGB_API int nbgb_force_ex(float *force, const float *posMass, float softeningSquared, size_t N,
                           void *workspace, size_t workspace_bytes, int config, int nsplit,
                           void *stream) {
    if (N == 0)
        return NBGB_OK;
    if (!force || !posMass)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (((uintptr_t)force | (uintptr_t)posMass) & 15u)
        return NBGB_ERR_INVALID_ARGUMENT;
    ForcePlan pl;
    int rc = plan_force(N, config, nsplit, pl);
    if (rc != NBGB_OK)
        return rc;
    if (!workspace || workspace_bytes < pl.workspace_bytes || ((uintptr_t)workspace & 255u))
        return NBGB_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    rc = launch_pack(pl, (const float4 *)posMass, workspace, st);
    if (rc != NBGB_OK)
        return rc;
    return launch_force(pl, (float4 *)force, (const float4 *)posMass, nullptr, softeningSquared,
                        workspace, st);
}

NBGB_API int nbgb_force(float *force, const float *posMass, float softeningSquared, size_t N,
                        void *workspace, size_t workspace_bytes, void *stream) {
    return nbgb_force_ex(force, posMass, softeningSquared, N, workspace, workspace_bytes, -1, -1,
                         stream);
}

NBGB_API size_t nbgb_force_rows_workspace_bytes(size_t N, size_t rows) {
    ForcePlan pl;
    if (plan_force_rows(N, rows, pl) != NBGB_OK)
        return 0;
    return pl.workspace_bytes;
}

// Forces on the target rows [row_begin, row_end) of posMass against all N
// sources: one rank's share of a row-sharded evaluation.
NBGB_API int nbgb_force_rows(float *force_rows, const float *posMass, float softeningSquared,
                             size_t N, size_t row_begin, size_t row_end, void *workspace,
                             size_t workspace_bytes, void *stream) {
    if (row_end < row_begin || row_end > N)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (row_end == row_begin)
        return NBGB_OK;
    if (!force_rows || !posMass)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (((uintptr_t)force_rows | (uintptr_t)posMass) & 15u)
        return NBGB_ERR_INVALID_ARGUMENT;
    ForcePlan pl;
    int rc = plan_force_rows(N, row_end - row_begin, pl);
    if (rc != NBGB_OK)
        return rc;
    if (!workspace || workspace_bytes < pl.workspace_bytes || ((uintptr_t)workspace & 255u))
        return NBGB_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    rc = launch_pack(pl, (const float4 *)posMass, workspace, st);
    if (rc != NBGB_OK)
        return rc;
    return launch_force(pl, (float4 *)force_rows, (const float4 *)posMass + row_begin, nullptr,
                        softeningSquared, workspace, st);
}

NBGB_API float ComputeGravitation_GPU_GB300(float *force, float *posMass, float softeningSquared,
                                            size_t N) {
    float ms = 0.0f;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    ForcePlan pl;
    void *ws = nullptr;
    if (N == 0 || !force || !posMass)
        return 0.0f;
    if (plan_force(N, -1, -1, pl) != NBGB_OK)
        return 0.0f;
    ws = cached_workspace(pl.workspace_bytes);
    if (!ws)
        return 0.0f;
    if (cudaEventCreate(&ev0) != cudaSuccess || cudaEventCreate(&ev1) != cudaSuccess)
        goto done;
    if (cudaEventRecord(ev0, nullptr) != cudaSuccess)
        goto done;
    for (int attempt = 0; attempt < 2; attempt++) {
        if (launch_pack(pl, (const float4 *)posMass, ws, nullptr) != NBGB_OK)
            goto done;
        if (launch_force(pl, (float4 *)force, (const float4 *)posMass, nullptr, softeningSquared,
                         ws, nullptr) != NBGB_OK)
            goto done;
        if (cudaEventRecord(ev1, nullptr) != cudaSuccess)
            goto done;
        if (cudaDeviceSynchronize() != cudaSuccess)
            goto done;
        unsigned bits = 0;
        if (read_and_clear_status(&bits) != NBGB_OK)
            goto done;
        if (bits == 0)
            break;
        // Negative masses met a log-domain plan: evaluate again with rsqrt
        // only (the reference's arithmetic accepts any sign).
        if (bits != NBGB_STATUS_NEGATIVE_MASS || attempt > 0 ||
            plan_force_rsqrt(N, pl) != NBGB_OK || !(ws = cached_workspace(pl.workspace_bytes)) ||
            cudaEventRecord(ev0, nullptr) != cudaSuccess)
            goto done;
    }
    if (cudaEventElapsedTime(&ms, ev0, ev1) != cudaSuccess)
        ms = 0.0f;
done:
    if (ev1)
        cudaEventDestroy(ev1);
    if (ev0)
        cudaEventDestroy(ev0);
    return ms;
}

// Second table row: the Newton's-third-law variant with the same drop-in
// conventions (device pointers, legacy stream, ms returned, 0 on error,
// synchronised); scratch from the same per-device cache.
NBGB_API float ComputeGravitation_GPU_GB300_Newton3(float *force, float *posMass,
                                                    float softeningSquared, size_t N) {
    float ms = 0.0f;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    void *ws = nullptr;
    size_t bytes = 0;
    if (N == 0 || !force || !posMass)
        return 0.0f;
    bytes = nbgb_force_newton3_workspace_bytes(N);
    if (!bytes || !(ws = cached_workspace(bytes)))
        return 0.0f;
    if (cudaEventCreate(&ev0) != cudaSuccess || cudaEventCreate(&ev1) != cudaSuccess)
        goto done;
    if (cudaEventRecord(ev0, nullptr) != cudaSuccess)
        goto done;
    if (nbgb_force_newton3(force, posMass, softeningSquared, N, ws, bytes, nullptr) != NBGB_OK)
        goto done;
    if (cudaEventRecord(ev1, nullptr) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess)
        goto done;
    {
        unsigned bits = 0;
        if (read_and_clear_status(&bits) != NBGB_OK || bits != 0)
            goto done;
    }
    if (cudaEventElapsedTime(&ms, ev0, ev1) != cudaSuccess)
        ms = 0.0f;
done:
    if (ev1)
        cudaEventDestroy(ev1);
    if (ev0)
        cudaEventDestroy(ev0);
    return ms;
}

NBGB_API void nbgb_release_workspace(void) { release_workspaces(); }

NBGB_API int nbgb_last_status(void) {
    unsigned bits = 0;
    int rc = read_and_clear_status(&bits);
    return rc != NBGB_OK ? rc : (int)bits;
}

NBGB_API const char *nbgb_status_string(int code) {
    switch (code) {
    case NBGB_OK: return "ok";
    case NBGB_ERR_INVALID_ARGUMENT: return "invalid argument";
    case NBGB_ERR_WORKSPACE: return "workspace missing, misaligned or too small";
    case NBGB_ERR_CUDA: return "CUDA runtime error";
    case NBGB_ERR_DEVICE: return "a kernel reported a device status (bounded wait ran out)";
    case NBGB_ERR_UNSUPPORTED: return "unsupported device or configuration";
    case NBGB_ERR_NO_MEMORY: return "out of memory or over the memory budget";
    case NBGB_ERR_TOO_LARGE: return "size exceeds the documented maximum";
    default: return "unknown status";
    }
}

NBGB_API const char *nbgb_version(void) { return "nbody_gb300 0.1 (sm_103a)"; }

// Runs the bounded-wait self-test (limit in milliseconds, 0 < limit <= 1000)
// and returns the device status bits it left (NBGB_STATUS_WAIT_TIMEOUT
// expected), or a negative NBGB_ERR_* code.  Synchronous.
NBGB_API int nbgb_selftest_bounded_wait(double limit_ms) {
    if (!(limit_ms > 0.0) || limit_ms > 1000.0)
        return NBGB_ERR_INVALID_ARGUMENT;
    int *out = nullptr, h = -1;
    unsigned bits = 0;
    if (read_and_clear_status(&bits) != NBGB_OK)  // start from a clean word
        return NBGB_ERR_CUDA;
    if (cudaMalloc(&out, sizeof(int)) != cudaSuccess)
        return NBGB_ERR_CUDA;
    selftest_wait_kernel<<<1, 32>>>((unsigned long long)(limit_ms * 1e6), out);
    int rc = NBGB_OK;
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(&h, out, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = NBGB_ERR_CUDA;
    cudaFree(out);
    if (rc != NBGB_OK)
        return rc;
    if (read_and_clear_status(&bits) != NBGB_OK)
        return NBGB_ERR_CUDA;
    return h == 0 ? (int)bits : NBGB_ERR_DEVICE;
}

}  // extern "C"
