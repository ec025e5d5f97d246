// force_sym.cu -- the all-pairs force with Newton's third law: every pair of
// bodies is evaluated once and applied to both (the idea of the reference's
// unregistered tiled kernels, src/nbody_GPU_AOS_tiled.cu:93-179, which add
// every pair's contribution with per-pair warp reductions and float atomics).
//
// Here the unit of work is a block pair (bi, bj), bi <= bj, of 2048-body
// blocks, one CTA of 8 warps each (one CTA per SM: up to 255 registers a
// thread, spent on independent work per warp rather than on more warps;
// sizes whose pairs would not fill the GPU use 1024-body blocks with 4
// targets and 4 sources per lane, 2 CTAs per SM -- the same scheme at half
// the width):
//   * warp w holds 256 targets of block bi in registers (8 per lane, negated
//     and duplicated into f32x2 pairs, with their masses);
//   * block bj is visited as 8 source sets of 256 bodies; every lane loads 8
//     sources (4 f32x2 pairs of the j-stream) plus zeroed accumulators, and
//     for 32 steps evaluates its 8 targets against the 8 sources it holds,
//     then passes sources and their accumulators to the next lane
//     (__shfl_sync rotation).  After 32 steps each source has met every
//     target of the warp and is back in its lane with its accumulated
//     reaction.  Each step carries 32 independent pair evaluations per lane
//     for 28 shuffles of 64-bit values;
//   * per pair and target: d = p_j - p_i, s = (|d|^2 + eps2)^-3/2 (MUFU
//     rsqrt), a_i += m_j s d, a_j -= m_i s d: 16 f32x2 operations per 4
//     interactions instead of 24 for the one-sided kernel;
//   * the 8 warps' reactions on a source set are added in shared memory in
//     warp order (deterministic), then one FP64 atomic add per body and
//     component moves them to the global FP64 accumulator; the targets'
//     sums (compensated, FP32 TwoSum every 256 sources) are added the same
//     way at the end of the block pair;
//   * diagonal block pairs (bi == bj): warp w skips source sets s < w and
//     evaluates s == w one-sided (every ordered pair of the set once, the
//     self pair contributing 0).
// A final kernel rounds the FP64 accumulators to FP32 forces.  The FP64 sums
// receive ~2 N / 2048 contributions per body in an order set by scheduling;
// FP64 keeps the result order-independent to well below FP32 resolution.
#include <cuda_runtime.h>

#include <cstdint>

#include "nbgb_device.cuh"
#include "nbgb_internal.h"
#include "nbody_gb300.h"

namespace nbgb {
namespace sym {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;

// Geometry: KI targets and KJ = KI sources per lane.  KI = 8: 2048-body
// blocks, one CTA per SM (up to 255 registers); KI = 4: 1024-body blocks,
// two CTAs per SM (128 registers), four times the block pairs for sizes
// whose 2048-body pairs would not fill the GPU.
template <int KI_>
struct Geo {
    static constexpr int KI = KI_;                  // targets per lane
    static constexpr int KJ = KI_;                  // sources per lane
    static constexpr int NC = KJ / 2;               // f32x2 source pairs per lane
    static constexpr int kMinBlocks = KI_ >= 8 ? 1 : 2;  // resident CTAs per SM
    static constexpr int kSet = 32 * KJ;            // sources per set
    static constexpr int kBlock = kWarps * 32 * KI; // bodies per block
    static constexpr int kFoldSets = kSet >= 256 ? 1 : 256 / kSet;  // sets per fold
    static_assert(kBlock == kWarps * kSet, "a block is 8 source sets");
    static_assert(kWarps % kFoldSets == 0, "folds end with the block's last set");
};
constexpr int kWideKI = 8, kNarrowKI = 4;

struct Params {
    const float4 *__restrict__ pm;  // AOS posMass (targets), n bodies
    const float4 *__restrict__ js;  // paired j-stream, npad bodies
    double *__restrict__ acc;       // [3][npad] FP64 accumulators
    int n, npad, nblocks;
    float eps2;
};

// pair index p -> (bi, bj) with bi <= bj over an nb x nb upper triangle,
// rows of decreasing length.
__device__ __forceinline__ void pair_of(long long p, int nb, int &bi, int &bj) {
    // row r holds nb - r pairs; rows before r hold r*nb - r(r-1)/2
    double b = 2.0 * nb + 1.0;
    int r = (int)((b - sqrt(b * b - 8.0 * (double)p)) * 0.5);
    if (r < 0)
        r = 0;
    if (r >= nb)
        r = nb - 1;
    auto start = [&](int rr) { return (long long)rr * nb - (long long)rr * (rr - 1) / 2; };
    while (r > 0 && start(r) > p)
        r--;
    while (r + 1 < nb && start(r + 1) <= p)
        r++;
    bi = r;
    bj = r + (int)(p - start(r));
}

// 32 rotation steps over one source set.  REACT: also accumulate the
// sources' reactions (both sides); otherwise only the targets' sums.  The
// branch on REACT is resolved at compile time, outside the step loop.
template <bool REACT, int KI, int NC = KI / 2>
__device__ __forceinline__ void rotate_set(f2 (&sx)[NC], f2 (&sy)[NC], f2 (&sz)[NC],
                                           f2 (&sm)[NC], f2 (&rx)[NC], f2 (&ry)[NC],
                                           f2 (&rz)[NC],
                                           const f2 (&nx)[KI], const f2 (&ny)[KI],
                                           const f2 (&nz)[KI], const f2 (&nm)[KI], f2 (&ax)[KI],
                                           f2 (&ay)[KI], f2 (&az)[KI], f2 eps2p, int lane) {
    const int from = (lane + 1) & 31;
#pragma unroll 2
    for (int step = 0; step < 32; step++) {
#pragma unroll
        for (int c = 0; c < NC; c++) {
#pragma unroll
            for (int k = 0; k < KI; k++) {
                f2 dx = f2_add(sx[c], nx[k]);
                f2 dy = f2_add(sy[c], ny[k]);
                f2 dz = f2_add(sz[c], nz[k]);
                f2 d2 = f2_fma(dx, dx, eps2p);
                d2 = f2_fma(dy, dy, d2);
                d2 = f2_fma(dz, dz, d2);
                float d2l, d2h;
                f2_unpack(d2, d2l, d2h);
                const f2 inv = f2_pack(rsqrt_mufu(d2l), rsqrt_mufu(d2h));
                const f2 inv2 = f2_mul(inv, inv);
                const f2 sc = f2_mul(inv, inv2);  // (|d|^2+eps2)^-3/2
                const f2 wi = f2_mul(sm[c], sc);  // m_j s
                ax[k] = f2_fma(dx, wi, ax[k]);
                ay[k] = f2_fma(dy, wi, ay[k]);
                az[k] = f2_fma(dz, wi, az[k]);
                if (REACT) {
                    const f2 wj = f2_mul(nm[k], sc);  // -m_i s
                    rx[c] = f2_fma(dx, wj, rx[c]);
                    ry[c] = f2_fma(dy, wj, ry[c]);
                    rz[c] = f2_fma(dz, wj, rz[c]);
                }
            }
        }
        // pass sources (and their reactions) to the next lane
#pragma unroll
        for (int c = 0; c < NC; c++) {
            sx[c] = __shfl_sync(0xffffffffu, sx[c], from);
            sy[c] = __shfl_sync(0xffffffffu, sy[c], from);
            sz[c] = __shfl_sync(0xffffffffu, sz[c], from);
            sm[c] = __shfl_sync(0xffffffffu, sm[c], from);
            if (REACT) {
                rx[c] = __shfl_sync(0xffffffffu, rx[c], from);
                ry[c] = __shfl_sync(0xffffffffu, ry[c], from);
                rz[c] = __shfl_sync(0xffffffffu, rz[c], from);
            }
        }
    }
}

// One block pair (bi, bj) of one system, by the whole CTA.
template <int KI_>
__device__ __forceinline__ void sym_block_pair(const Params &P, int bi, int bj) {
    using G = Geo<KI_>;
    constexpr int KI = G::KI, KJ = G::KJ, NC = G::NC, kSet = G::kSet, kBlock = G::kBlock,
                  kFoldSets = G::kFoldSets;
    __shared__ float red[kWarps][3][kSet];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool diag = (bi == bj);

    // targets: lane owns bodies bi*kBlock + warp*32*KI + lane + 32*k
    f2 nx[KI], ny[KI], nz[KI], nm[KI];
    f2 ax[KI], ay[KI], az[KI];
    float hx[KI], hy[KI], hz[KI], lx[KI], ly[KI], lz[KI];
#pragma unroll
    for (int k = 0; k < KI; k++) {
        const int i = bi * kBlock + warp * 32 * KI + lane + 32 * k;
        const float4 b = (i < P.n) ? P.pm[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        nx[k] = f2_pack(-b.x, -b.x);
        ny[k] = f2_pack(-b.y, -b.y);
        nz[k] = f2_pack(-b.z, -b.z);
        nm[k] = f2_pack(-b.w, -b.w);
        hx[k] = hy[k] = hz[k] = lx[k] = ly[k] = lz[k] = 0.f;
    }
    const f2 eps2p = f2_pack(P.eps2, P.eps2);
    const f2 zero2 = f2_pack(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < KI; k++)
        ax[k] = ay[k] = az[k] = zero2;

    for (int s = 0; s < kWarps; s++) {
        // mode: 2 both sides, 1 targets only (the warp's own set), 0 skip
        const int mode = !diag ? 2 : (s > warp ? 2 : (s == warp ? 1 : 0));
        // sources of set s: lane holds bodies base .. base + KJ - 1 (NC pairs)
        const int base = bj * kBlock + s * kSet + lane * KJ;
        f2 sx[NC], sy[NC], sz[NC], sm[NC], rx[NC], ry[NC], rz[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const ulonglong2 a = reinterpret_cast<const ulonglong2 *>(P.js)[base + 2 * c];
            const ulonglong2 b = reinterpret_cast<const ulonglong2 *>(P.js)[base + 2 * c + 1];
            sx[c] = a.x;
            sy[c] = a.y;
            sz[c] = b.x;
            sm[c] = b.y;
            rx[c] = ry[c] = rz[c] = zero2;
        }
        if (mode == 2)
            rotate_set<true, KI>(sx, sy, sz, sm, rx, ry, rz, nx, ny, nz, nm, ax, ay, az, eps2p,
                                 lane);
        else if (mode == 1)
            rotate_set<false, KI>(sx, sy, sz, sm, rx, ry, rz, nx, ny, nz, nm, ax, ay, az, eps2p,
                                  lane);
        // fold target sums into the compensated sums every 256 sources
        if ((s + 1) % kFoldSets == 0) {
#pragma unroll
            for (int k = 0; k < KI; k++) {
                float l, h;
                f2_unpack(ax[k], l, h);
                comp_add(hx[k], lx[k], l + h);
                f2_unpack(ay[k], l, h);
                comp_add(hy[k], ly[k], l + h);
                f2_unpack(az[k], l, h);
                comp_add(hz[k], lz[k], l + h);
                ax[k] = ay[k] = az[k] = zero2;
            }
        }
        // reactions on set s: stage per warp, add in warp order, FP64 atomics
#pragma unroll
        for (int c = 0; c < NC; c++) {
            float l, h;
            f2_unpack(rx[c], l, h);
            red[warp][0][lane * KJ + 2 * c] = l;
            red[warp][0][lane * KJ + 2 * c + 1] = h;
            f2_unpack(ry[c], l, h);
            red[warp][1][lane * KJ + 2 * c] = l;
            red[warp][1][lane * KJ + 2 * c + 1] = h;
            f2_unpack(rz[c], l, h);
            red[warp][2][lane * KJ + 2 * c] = l;
            red[warp][2][lane * KJ + 2 * c + 1] = h;
        }
        __syncthreads();
        for (int q = tid; q < 3 * kSet; q += kThreads) {
            const int comp = q / kSet, jj = q - comp * kSet;
            float t = 0.f;
#pragma unroll
            for (int w = 0; w < kWarps; w++)
                t += red[w][comp][jj];
            const int j = bj * kBlock + s * kSet + jj;
            if (t != 0.f && j < P.n)
                atomicAdd(&P.acc[(size_t)comp * P.npad + j], (double)t);
        }
        __syncthreads();
    }
    // targets' sums -> FP64 accumulators
#pragma unroll
    for (int k = 0; k < KI; k++) {
        const int i = bi * kBlock + warp * 32 * KI + lane + 32 * k;
        if (i < P.n) {
            atomicAdd(&P.acc[i], (double)hx[k] + (double)lx[k]);
            atomicAdd(&P.acc[(size_t)P.npad + i], (double)hy[k] + (double)ly[k]);
            atomicAdd(&P.acc[2 * (size_t)P.npad + i], (double)hz[k] + (double)lz[k]);
        }
    }
}

template <int KI_>
__global__ void __launch_bounds__(kThreads, Geo<KI_>::kMinBlocks) sym_kernel(Params P) {
    int bi, bj;
    pair_of(blockIdx.x, P.nblocks, bi, bj);
    sym_block_pair<KI_>(P, bi, bj);
}

// Many systems in one launch (the ensemble's Newton-3 systems): CTA b takes
// block pair b - pair_begin[s] of the system s whose range holds b (binary
// search over the systems' prefix counts).
__global__ void __launch_bounds__(kThreads, Geo<kWideKI>::kMinBlocks)
    sym_systems_kernel(const SymSystem *__restrict__ tab, int nsys) {
    const long long b = blockIdx.x;
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tab[mid].pair_begin <= b)
            lo = mid;
        else
            hi = mid - 1;
    }
    const SymSystem &t = tab[lo];
    Params P;
    P.pm = t.pm;
    P.js = t.js;
    P.acc = t.acc;
    P.n = t.n;
    P.npad = t.npad;
    P.nblocks = t.nblocks;
    P.eps2 = t.eps2;
    int bi, bj;
    pair_of(b - t.pair_begin, t.nblocks, bi, bj);
    sym_block_pair<kWideKI>(P, bi, bj);
}

// FP64 sums -> FP32 accelerations {ax, ay, az, 0}, and the sums zeroed for
// the next evaluation.
__global__ void sym_finish_zero_kernel(double *__restrict__ acc, int n, int npad,
                                       float4 *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        out[i] = make_float4((float)acc[i], (float)acc[(size_t)npad + i],
                             (float)acc[2 * (size_t)npad + i], 0.f);
        acc[i] = acc[(size_t)npad + i] = acc[2 * (size_t)npad + i] = 0.0;
    }
}

__global__ void sym_finish_kernel(const double *__restrict__ acc, int n, int npad,
                                  float4 *__restrict__ force) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        force[i] = make_float4((float)acc[i], (float)acc[(size_t)npad + i],
                               (float)acc[2 * (size_t)npad + i], 0.f);
}

}  // namespace sym

int launch_sym_systems(const SymSystem *d_tab, const SymSystem *h_tab, int nsys,
                       cudaStream_t st) {
    if (nsys <= 0)
        return NBGB_OK;
    const long long pairs = h_tab[nsys - 1].pair_begin +
                            (long long)h_tab[nsys - 1].nblocks * (h_tab[nsys - 1].nblocks + 1) / 2;
    if (pairs > (1ll << 31) - 1)
        return NBGB_ERR_TOO_LARGE;
    sym::sym_systems_kernel<<<(unsigned)pairs, sym::kThreads, 0, st>>>(d_tab, nsys);
    for (int s = 0; s < nsys; s++)
        sym::sym_finish_zero_kernel<<<(unsigned)((h_tab[s].n + 255) / 256), 256, 0, st>>>(
            h_tab[s].acc, h_tab[s].n, h_tab[s].npad, h_tab[s].out);
    return cudaGetLastError() == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

int sym_block_bodies() { return sym::Geo<sym::kWideKI>::kBlock; }

}  // namespace nbgb

namespace {

struct SymLayout {
    int ki, block;  // geometry: targets per lane, bodies per block
    int nblocks, npad;
    size_t off_js, off_acc, bytes;
};

int device_sms() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0) {
        cudaGetLastError();  // no device: plan for a 152-SM GB300
        sms = 152;
    }
    return sms;
}

// The wide geometry (2048-body blocks, one CTA per SM) when its block pairs
// give every SM at least two; the narrow one (1024-body blocks, four times
// the pairs) below that.
SymLayout sym_layout(size_t n) {
    using Wide = nbgb::sym::Geo<nbgb::sym::kWideKI>;
    using Narrow = nbgb::sym::Geo<nbgb::sym::kNarrowKI>;
    SymLayout L;
    const long long nbw = (long long)((n + Wide::kBlock - 1) / Wide::kBlock);
    const bool wide = nbw * (nbw + 1) / 2 >= 2LL * device_sms();
    L.ki = wide ? Wide::KI : Narrow::KI;
    L.block = wide ? Wide::kBlock : Narrow::kBlock;
    L.nblocks = (int)((n + L.block - 1) / L.block);
    L.npad = L.nblocks * L.block;
    L.off_js = 0;
    L.off_acc = ((size_t)L.npad * 16 + 255) / 256 * 256;
    L.bytes = L.off_acc + (size_t)3 * L.npad * sizeof(double);
    return L;
}

}  // namespace

extern "C" {

NBGB_API size_t nbgb_force_newton3_workspace_bytes(size_t N) {
    if (N == 0 || N > nbgb::kMaxBodies)
        return 0;
    return sym_layout(N).bytes;
}

NBGB_API int nbgb_force_newton3(float *force, const float *posMass, float softeningSquared,
                                size_t N, void *workspace, size_t workspace_bytes, void *stream) {
    if (N == 0)
        return NBGB_OK;
    if (!force || !posMass || N > nbgb::kMaxBodies)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (((uintptr_t)force | (uintptr_t)posMass) & 15u)
        return NBGB_ERR_INVALID_ARGUMENT;
    const SymLayout L = sym_layout(N);
    if (!workspace || workspace_bytes < L.bytes || ((uintptr_t)workspace & 255u))
        return NBGB_ERR_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)workspace;
    // the j-stream (paired layout, zero-mass padding to whole blocks)
    nbgb::ForcePlan pl;
    pl.n = N;
    pl.ntiles = L.nblocks;
    pl.tile_bodies = L.block;
    pl.js_vpb = 1;
    pl.nsplit = 1;
    pl.off_js = L.off_js;
    int rc = nbgb::launch_pack(pl, (const float4 *)posMass, ws, st);
    if (rc != NBGB_OK)
        return rc;
    double *acc = (double *)(ws + L.off_acc);
    if (cudaMemsetAsync(acc, 0, (size_t)3 * L.npad * sizeof(double), st) != cudaSuccess)
        return NBGB_ERR_CUDA;
    nbgb::sym::Params P;
    P.pm = (const float4 *)posMass;
    P.js = (const float4 *)(ws + L.off_js);
    P.acc = acc;
    P.n = (int)N;
    P.npad = L.npad;
    P.nblocks = L.nblocks;
    P.eps2 = softeningSquared;
    const long long pairs = (long long)L.nblocks * (L.nblocks + 1) / 2;
    if (pairs > (1ll << 31) - 1)
        return NBGB_ERR_TOO_LARGE;
    if (L.ki == nbgb::sym::kWideKI)
        nbgb::sym::sym_kernel<nbgb::sym::kWideKI><<<(unsigned)pairs, nbgb::sym::kThreads, 0, st>>>(P);
    else
        nbgb::sym::sym_kernel<nbgb::sym::kNarrowKI>
            <<<(unsigned)pairs, nbgb::sym::kThreads, 0, st>>>(P);
    nbgb::sym::sym_finish_kernel<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(
        acc, (int)N, L.npad, (float4 *)force);
    return cudaGetLastError() == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

}  // extern "C"
