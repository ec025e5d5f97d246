// ensemble.cu -- many independent systems of uneven N on one GPU.
//
// The reference evaluates one system per call (its algorithms take one
// posMass array, src/nbody.h:68); running thousands of small systems that way
// costs a launch (and a host round trip) per system per step and leaves most
// of the GPU idle.  Here every active system's state is resident in one arena
// and a tick advances all of them by one FP64 kick-drift-kick step with three
// launches:
//
//   ens_kick_drift   v += a dt/2; x += v dt (FP64) for moving systems, and
//                    rewrite every active system's FP32 posMass and j-stream
//   ens_force        ONE persistent launch: CTAs take work items (system,
//                    i-block, j-split) from a device queue with an atomic
//                    counter, largest items first, and evaluate them with the
//                    same TMA ring, f32x2 pair interaction (every fourth
//                    source pair in the log domain for systems whose masses
//                    are all >= 0) and TwoSum accumulation as the
//                    single-system kernel; a system whose
//                    j-range is split combines its partials in fixed order
//                    (last item of the i-block, atomic counter)
//   ens_kick         v += a dt/2 for moving systems
//
// Newton-3 systems (opt-in, nbgb_ensemble_set_newton3_min): systems of at
// least that many bodies skip the work queue; pass 0 of each tick evaluates
// them with the Newton's-third-law kernel (block pairs, FP64 sums; one launch
// for all of them) and rounds their sums to FP32 accelerations.  Their
// results repeat to FP64 rounding order (not bit for bit).
//
// Sub-cycling: a system may take up to kMaxSub steps per tick (its `sub`).
// A tick then runs passes p = 0 .. max sub - 1, each the three launches above
// over the systems whose effective sub (min(sub, steps left)) exceeds p, so
// small systems advance several steps while large ones advance one.  Pass p's
// work items are a suffix of one list sorted by effective sub (ascending),
// then cost (descending).
//
// A system's decomposition (kernel variant, tile size, j-split) depends only
// on its own N, so its result is bit-identical whether it runs alone or in
// any mix (with any sub).  Newly admitted systems spend their first tick in the force pass
// only (their initial accelerations); systems whose steps are done leave the
// tick.  While the membership is unchanged the tick is replayed from a CUDA
// graph.  Admission is bounded by a slot count and a device-memory budget.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "nbgb_device.cuh"
#include "nbgb_internal.h"
#include "nbody_gb300.h"

namespace nbgb {
namespace ens {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
constexpr int kStages = 3;
constexpr int kMaxJT = 1024;  // largest tile (bodies); ring stage = 16 KiB
constexpr uint32_t kStageBytes = kMaxJT * 16u;

// kLogMass: j-stream pairs q % 4 == 0 (system-local) hold log2 masses and
// are evaluated in the log domain (set when every mass is >= 0).
enum : int { kMove = 1, kInForce = 2, kLogMass = 4 };
constexpr int kMaxSub = 8;  // steps per tick of one system, at most

// Device descriptor of one system slot.
struct Desc {
    int n;         // bodies
    int body_off;  // into the body arrays
    int js_off;    // into the j-stream arena (float4 units, even)
    int ntiles;
    int jt;        // bodies per tile
    int variant;   // targets/thread and unroll: 0 (1, 8), 1 (2, 4), 2 (1, 4), 3 (2, 8)
    int nsplit;
    int nblocks;
    long long part_off;  // into the partial arena (float4 units); lo follows hi
    int cnt_off;         // into the counter arena
    int ni_pad;          // nblocks * block bodies
    int flags;           // kMove | kInForce | kLogMass
    int sub;             // passes of this tick the system moves in (1..kMaxSub)
    float eps2;
    double dt;
};

struct Params {
    const Desc *desc;
    const int4 *items;  // {system, i-block, split, 0}
    int n_items;
    unsigned *head;     // queue counter (zeroed before the launch)
    const float4 *pm;   // all bodies
    const float4 *js;   // all j-streams
    float4 *acc;        // all bodies
    float4 *part;       // partial arena
    unsigned *cnt;      // counter arena
};

// One work item with K targets per thread.  tile_base: tiles this CTA has
// streamed through its ring before this item (keeps stage phases continuous
// across items).  Returns false if a bounded wait ran out.
template <int K, int UNROLL, bool LOGM>
__device__ bool process_item(const Params &P, const Desc &d, int ib, int r, unsigned tile_base,
                             float4 *ring, uint64_t *full, unsigned *released, int *stage_tile,
                             int *abort_flag, int *s_last) {
    constexpr int BI = kThreads * K;
    const int tid = threadIdx.x, lane = tid & 31;
    const int t_begin = (int)(((long long)r * d.ntiles) / d.nsplit);
    const int t_end = (int)(((long long)(r + 1) * d.ntiles) / d.nsplit);
    const int nt = t_end - t_begin;
    const int jt = d.jt;
    const uint32_t tile_bytes = (uint32_t)jt * 16u;
    const float4 *js = P.js + d.js_off;

    if (tid == 0) {
        // the previous item read these stages through the generic proxy
        fence_proxy_async_shared();
        for (int u = 0; u < kStages && u < nt; u++) {
            const unsigned g = tile_base + (unsigned)u;
            const int s = (int)(g % kStages);
            mbar_expect_tx(&full[s], tile_bytes);
            bulk_g2s(ring + (size_t)s * kMaxJT, js + (size_t)(t_begin + u) * jt, tile_bytes,
                     &full[s]);
            stage_tile[s] = (int)g;
        }
    }

    f2 nx[K], ny[K], nz[K];
    float hx[K], hy[K], hz[K], lx[K], ly[K], lz[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int i = ib * BI + k * kThreads + tid;
        const float4 b = (i < d.n) ? P.pm[d.body_off + i] : make_float4(0.f, 0.f, 0.f, 0.f);
        nx[k] = f2_pack(-b.x, -b.x);
        ny[k] = f2_pack(-b.y, -b.y);
        nz[k] = f2_pack(-b.z, -b.z);
        hx[k] = hy[k] = hz[k] = lx[k] = ly[k] = lz[k] = 0.f;
    }
    const f2 eps2p = f2_pack(d.eps2, d.eps2);
    const f2 zero2 = f2_pack(0.f, 0.f);
    const f2 m15 = f2_pack(-1.5f, -1.5f);

    bool failed = false;
    for (int t = 0; t < nt; t++) {
        const unsigned g = tile_base + (unsigned)t;
        const int s = (int)(g % kStages);
        const uint32_t parity = (g / kStages) & 1u;
        if (__any_sync(0xffffffffu, *(volatile int *)abort_flag != 0)) {
            failed = true;
            break;
        }
        if (!__all_sync(0xffffffffu, mbar_wait_bounded(&full[s], parity))) {
            if (lane == 0)
                *(volatile int *)abort_flag = 1;
            failed = true;
            break;
        }
        const ulonglong2 *tp = reinterpret_cast<const ulonglong2 *>(ring + (size_t)s * kMaxJT);
        f2 ax[K], ay[K], az[K];
        // fold into the compensated sum every 256 sources (or per tile)
        const int fpairs = jt / 2 < 128 ? jt / 2 : 128;
        for (int q0 = 0; q0 < jt / 2; q0 += fpairs) {
#pragma unroll
            for (int k = 0; k < K; k++)
                ax[k] = ay[k] = az[k] = zero2;
            if constexpr (LOGM) {  // groups of 4 pairs, the first in the log domain
                constexpr int GROUPS = UNROLL >= 4 ? UNROLL / 4 : 1;
#pragma unroll GROUPS
                for (int q = q0; q < q0 + fpairs; q += 4) {
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
            } else {
#pragma unroll UNROLL
                for (int q = q0; q < q0 + fpairs; q++) {
                    const ulonglong2 a = tp[2 * q];
                    const ulonglong2 b = tp[2 * q + 1];
#pragma unroll
                    for (int k = 0; k < K; k++)
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
        __syncwarp();
        if (lane == 0) {
            const unsigned round = g / kStages + 1u;
            const unsigned prev = atom_add_acqrel_shared(&released[s], 1u);
            if (prev == round * kWarps - 1u && t + kStages < nt) {
                fence_proxy_async_shared();
                mbar_expect_tx(&full[s], tile_bytes);
                bulk_g2s(ring + (size_t)s * kMaxJT, js + (size_t)(t_begin + t + kStages) * jt,
                         tile_bytes, &full[s]);
                stage_tile[s] = (int)(g + kStages);
            }
        }
    }
    if (__syncthreads_or(failed))
        return false;

    float4 *out = P.acc + d.body_off;
    if (d.nsplit == 1) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int i = ib * BI + k * kThreads + tid;
            if (i < d.n)
                out[i] = make_float4(hx[k] + lx[k], hy[k] + ly[k], hz[k] + lz[k], 0.f);
        }
        return true;
    }
    float4 *hi = P.part + d.part_off;
    float4 *lo = hi + (size_t)d.nsplit * d.ni_pad;
#pragma unroll
    for (int k = 0; k < K; k++) {
        const size_t o = (size_t)r * d.ni_pad + (size_t)(ib * BI + k * kThreads + tid);
        hi[o] = make_float4(hx[k], hy[k], hz[k], 0.f);
        lo[o] = make_float4(lx[k], ly[k], lz[k], 0.f);
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        unsigned *c = P.cnt + d.cnt_off + ib;
        const unsigned prev = atomicAdd(c, 1u);
        *s_last = (prev == (unsigned)(d.nsplit - 1));
        if (*s_last)
            *c = 0u;
    }
    __syncthreads();
    if (!*s_last)
        return true;
    __threadfence();
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int i = ib * BI + k * kThreads + tid;
        if (i >= d.n)
            continue;
        float Hx = 0.f, Hy = 0.f, Hz = 0.f, Lx = 0.f, Ly = 0.f, Lz = 0.f;
        for (int rr = 0; rr < d.nsplit; rr++) {
            float4 h, l;
            if (rr == r) {
                h = make_float4(hx[k], hy[k], hz[k], 0.f);
                l = make_float4(lx[k], ly[k], lz[k], 0.f);
            } else {
                const size_t o = (size_t)rr * d.ni_pad + (size_t)i;
                h = __ldcg(hi + o);
                l = __ldcg(lo + o);
            }
            comp_add(Hx, Lx, h.x);
            comp_add(Hy, Ly, h.y);
            comp_add(Hz, Lz, h.z);
            Lx += l.x;
            Ly += l.y;
            Lz += l.z;
        }
        out[i] = make_float4(Hx + Lx, Hy + Ly, Hz + Lz, 0.f);
    }
    return true;
}

__global__ void __launch_bounds__(kThreads, 2) ens_force_kernel(Params P) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float4 *ring = reinterpret_cast<float4 *>(smem_raw);
    __shared__ __align__(8) uint64_t full[kStages];
    __shared__ unsigned released[kStages];
    __shared__ int stage_tile[kStages];
    __shared__ int abort_flag, s_last, s_item;
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int s = 0; s < kStages; s++) {
            mbar_init(&full[s], 1);
            released[s] = 0u;
            stage_tile[s] = -1;
        }
        abort_flag = 0;
        fence_mbar_init();
    }
    unsigned tile_base = 0;
    bool ok = true;
    for (;;) {
        __syncthreads();  // previous item fully consumed; ring free
        if (tid == 0)
            s_item = (int)atomicAdd(P.head, 1u);
        __syncthreads();
        const int it = s_item;
        if (it >= P.n_items)
            break;
        const int4 item = P.items[it];
        const Desc d = P.desc[item.x];
        const bool lg = (d.flags & kLogMass) != 0;
#define NBGB_ENS_ITEM(K, U)                                                                \
    (lg ? process_item<K, U, true>(P, d, item.y, item.z, tile_base, ring, full, released,  \
                                   stage_tile, &abort_flag, &s_last)                       \
        : process_item<K, U, false>(P, d, item.y, item.z, tile_base, ring, full, released, \
                                    stage_tile, &abort_flag, &s_last))
        switch (d.variant) {
        case 0:
            ok = NBGB_ENS_ITEM(1, 8);
            break;
        case 1:
            ok = NBGB_ENS_ITEM(2, 4);
            break;
        case 2:
            ok = NBGB_ENS_ITEM(1, 4);
            break;
        default:
            ok = NBGB_ENS_ITEM(2, 8);
            break;
        }
#undef NBGB_ENS_ITEM
        if (!ok)
            break;
        const int t_begin = (int)(((long long)item.z * d.ntiles) / d.nsplit);
        const int t_end = (int)(((long long)(item.z + 1) * d.ntiles) / d.nsplit);
        tile_base += (unsigned)(t_end - t_begin);
    }
    if (!ok && tid == 0)
        for (int s = 0; s < kStages; s++)
            if (stage_tile[s] >= 0)
                (void)mbar_wait_bounded(&full[s], (uint32_t)((stage_tile[s] / kStages) & 1),
                                        100000000ull);
}

// Thread q owns j-stream pair slot q (bodies 2p, 2p+1 of system slot_sys[q]).
// mode 0: kick half + drift for moving systems, then write posMass and the
// j-stream of every active system; mode 1: kick half only.  pass > 0: only
// moving systems with sub > pass take part.
__global__ void ens_kdk_kernel(const Desc *__restrict__ desc, const int *__restrict__ slot_sys,
                               int n_slots, double *__restrict__ x64, size_t stride,
                               const float *__restrict__ mass, const float4 *__restrict__ acc,
                               float4 *__restrict__ pm, float4 *__restrict__ js, int mode,
                               int pass) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_slots)
        return;
    const int sys = slot_sys[q];
    if (sys < 0)
        return;
    const Desc d = desc[sys];
    if (!(d.flags & kInForce))
        return;
    if (pass > 0 && (!(d.flags & kMove) || d.sub <= pass))
        return;
    const bool move = (d.flags & kMove) != 0;
    const int lp = q - d.js_off / 2;
    float4 out[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int b = 2 * lp + h;
        if (b < d.n) {
            const size_t i = (size_t)d.body_off + b;
            double x = x64[i], y = x64[stride + i], z = x64[2 * stride + i];
            if (move) {
                const float4 a = acc[i];
                const double kdt = 0.5 * d.dt;
                // conversions on the integer pipe: GB300's FP64 pipe is narrow
                double u = fma(widen_f32(a.x), kdt, x64[3 * stride + i]);
                double v = fma(widen_f32(a.y), kdt, x64[4 * stride + i]);
                double w = fma(widen_f32(a.z), kdt, x64[5 * stride + i]);
                x64[3 * stride + i] = u;
                x64[4 * stride + i] = v;
                x64[5 * stride + i] = w;
                if (mode == 0) {
                    x = fma(u, d.dt, x);
                    y = fma(v, d.dt, y);
                    z = fma(w, d.dt, z);
                    x64[i] = x;
                    x64[stride + i] = y;
                    x64[2 * stride + i] = z;
                }
            }
            out[h] = make_float4(narrow_f64(x), narrow_f64(y), narrow_f64(z), mass[i]);
            if (mode == 0)
                pm[i] = out[h];
        } else {
            out[h] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    if (mode == 0) {
        if ((d.flags & kLogMass) && (lp & 3) == 0) {  // log-domain pair (padding: -inf)
            out[0].w = jstream_log_mass(out[0].w);
            out[1].w = jstream_log_mass(out[1].w);
        }
        js[2 * q] = make_float4(out[0].x, out[1].x, out[0].y, out[1].y);
        js[2 * q + 1] = make_float4(out[0].z, out[1].z, out[0].w, out[1].w);
    }
}

static NBGB_STATUS_READER(read_status_ens)

}  // namespace ens

int read_status_ensemble(unsigned *bits) { return ens::read_status_ens(bits); }

}  // namespace nbgb

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
using nbgb::ens::Desc;

namespace {

// First-fit allocator over [0, capacity) in abstract units.
struct RangeAlloc {
    struct R {
        size_t off, len;
    };
    size_t capacity = 0;
    std::vector<R> free_list;
    void init(size_t cap) {
        capacity = cap;
        free_list.assign(1, R{0, cap});
    }
    bool alloc(size_t len, size_t align, size_t &off) {
        if (len == 0) {
            off = 0;
            return true;
        }
        for (size_t k = 0; k < free_list.size(); k++) {
            R &f = free_list[k];
            const size_t a = (f.off + align - 1) / align * align;
            if (a + len <= f.off + f.len) {
                const size_t tail = f.off + f.len - (a + len);
                const size_t head = a - f.off;
                off = a;
                if (head && tail) {
                    f.len = head;
                    free_list.insert(free_list.begin() + k + 1, R{a + len, tail});
                } else if (head) {
                    f.len = head;
                } else if (tail) {
                    f.off = a + len;
                    f.len = tail;
                } else {
                    free_list.erase(free_list.begin() + k);
                }
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t len) {
        if (len == 0)
            return;
        R r{off, len};
        auto it = std::lower_bound(free_list.begin(), free_list.end(), r,
                                   [](const R &a, const R &b) { return a.off < b.off; });
        it = free_list.insert(it, r);
        // merge with neighbours
        if (it + 1 != free_list.end() && it->off + it->len == (it + 1)->off) {
            it->len += (it + 1)->len;
            free_list.erase(it + 1);
        }
        if (it != free_list.begin() && (it - 1)->off + (it - 1)->len == it->off) {
            (it - 1)->len += it->len;
            free_list.erase(it);
        }
    }
};

struct HostSys {
    bool used = false;
    int n = 0;
    size_t body_off = 0, js_off = 0, part_off = 0, cnt_off = 0;
    size_t body_len = 0, js_len = 0, part_len = 0, cnt_len = 0;
    int variant = 1, jt = 256, nsplit = 1, nblocks = 0, ntiles = 0, ni_pad = 0;
    double dt = 0.0;
    long long steps_left = 0;
    bool started = false;  // has initial accelerations
    long long steps_done = 0;
    bool log_mass = false;  // every mass >= 0: log-domain pairs (kLogMass)
    int sub = 1;            // steps per tick (1..kMaxSub)
    bool n3 = false;        // Newton-3 system (no work items)
    size_t acc_off = 0, acc_len = 0;  // its FP64 sums ([3][npad] doubles)
};

// Steps a system takes in the coming tick (0 before its initial forces).
inline int sub_eff(const HostSys &h) {
    if (!h.started || h.n3)
        return 1;  // the initial-force pass; Newton-3 systems run in pass 0 only
    return (int)std::min<long long>(h.sub, h.steps_left);
}

// Per-N-bucket plan: bucket b covers N in [2^b, 2^(b+1)).
struct BucketPlan {
    int variant = -1, jt = 0, nsplit = 0;  // -1: default rule
};

}  // namespace

struct nbgb_ensemble {
    int device = 0;
    cudaStream_t stream = nullptr;
    float eps2 = 1e-4f;
    int max_systems = 0;
    size_t max_bodies = 0, js_cap = 0, part_cap = 0, cnt_cap = 0;
    // device arena
    double *x64 = nullptr;  // 6 * max_bodies
    float *mass = nullptr;
    float4 *pm = nullptr, *acc = nullptr, *js = nullptr, *part = nullptr;
    unsigned *cnt = nullptr, *head = nullptr;
    Desc *d_desc = nullptr;
    int4 *d_items = nullptr;
    int *d_slot_sys = nullptr;
    size_t items_cap = 0;
    // pinned host mirrors for uploads
    Desc *h_desc = nullptr;
    int4 *h_items = nullptr;
    int *h_slot_sys = nullptr;
    // host bookkeeping
    std::vector<HostSys> sys;
    RangeAlloc a_body, a_js, a_part, a_cnt;
    BucketPlan bucket[32];
    int n_items = 0, n_slots = 0;
    int n_pass = 1;                       // passes per tick (max effective sub)
    // Newton-3 systems
    size_t n3_min = 0;                    // 0: off
    double *acc64 = nullptr;              // FP64 sums arena (allocated when enabled)
    size_t acc64_cap = 0;
    RangeAlloc a_acc;
    nbgb::SymSystem *d_sym = nullptr, *h_sym = nullptr;
    int n_sym = 0;
    int pass_first[nbgb::ens::kMaxSub];   // first item of pass p (items sorted by sub)
    bool dirty = true;
    cudaGraphExec_t graph = nullptr;
    bool use_graph = true;
    int stable_ticks = 0;  // ticks since the membership last changed
    int grid = 0;      // CTAs of the persistent force launch
    int grid_max = 0;  // SMs x resident CTAs per SM
    size_t bytes_total = 0;
    long long ticks = 0;
};

namespace {

int bucket_of(int n) {
    int b = 0;
    while ((2 << b) <= n && b < 31)
        b++;
    return b;
}

// Default per-bucket rule (used until an autotuner sets bucket plans): small
// systems 1 target per thread and 128-body tiles, larger ones 2 per thread
// with tiles up to 512 bodies; no j-split below 16 i-blocks.
void choose_plan(nbgb_ensemble *e, int n, HostSys &h) {
    const BucketPlan &bp = e->bucket[bucket_of(n)];
    int variant = bp.variant, jt = bp.jt, nsplit = bp.nsplit;
    if (variant < 0) {
        variant = n <= 1024 ? 0 : 1;
        jt = n <= 512 ? 128 : (n <= 4096 ? 256 : 512);
        nsplit = 1;
    }
    const int bi = nbgb::ens::kThreads * ((variant == 0 || variant == 2) ? 1 : 2);
    h.variant = variant;
    h.jt = jt;
    h.nblocks = (n + bi - 1) / bi;
    h.ntiles = (n + jt - 1) / jt;
    h.nsplit = std::max(1, std::min(std::min(nsplit, 4), h.ntiles));
    h.ni_pad = h.nblocks * bi;
}

void fill_desc(nbgb_ensemble *e, int slot, Desc &d) {
    const HostSys &h = e->sys[slot];
    d.n = h.n;
    d.body_off = (int)h.body_off;
    d.js_off = (int)h.js_off;
    d.ntiles = h.ntiles;
    d.jt = h.jt;
    d.variant = h.variant;
    d.nsplit = h.nsplit;
    d.nblocks = h.nblocks;
    d.part_off = (long long)h.part_off;
    d.cnt_off = (int)h.cnt_off;
    d.ni_pad = h.ni_pad;
    d.flags = h.used ? (nbgb::ens::kInForce | (h.started && h.steps_left > 0 ? nbgb::ens::kMove : 0) |
                        (h.log_mass ? nbgb::ens::kLogMass : 0))
                     : 0;
    d.sub = h.used ? sub_eff(h) : 1;
    d.eps2 = e->eps2;
    d.dt = h.dt;
}

// Rebuild descriptors, the j-stream slot map and the largest-first item list.
// The pinned staging buffers are re-filled, so uploads (and ticks) still queued
// from an earlier rebuild must have run first: synchronise the stream.
int rebuild(nbgb_ensemble *e) {
    if (cudaStreamSynchronize(e->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    struct It {
        int4 v;
        double cost;
        int sub;
    };
    std::vector<It> items;
    for (int s = 0; s < e->max_systems; s++) {
        fill_desc(e, s, e->h_desc[s]);
        const HostSys &h = e->sys[s];
        if (!h.used)
            continue;
        const bool in_force = h.steps_left > 0 || !h.started;
        if (!in_force) {
            e->h_desc[s].flags = 0;
            continue;
        }
        if (h.n3)
            continue;  // evaluated by the Newton-3 launch
        const int bi = nbgb::ens::kThreads * ((h.variant == 0 || h.variant == 2) ? 1 : 2);
        for (int b = 0; b < h.nblocks; b++)
            for (int r = 0; r < h.nsplit; r++) {
                const int tb = (int)(((long long)r * h.ntiles) / h.nsplit);
                const int te = (int)(((long long)(r + 1) * h.ntiles) / h.nsplit);
                items.push_back(It{make_int4(s, b, r, 0),
                                   (double)(te - tb) * h.jt * bi + 4096.0, sub_eff(h)});
            }
    }
    // by effective sub (ascending), then largest first: pass p's items are
    // the suffix of systems with sub > p
    std::stable_sort(items.begin(), items.end(), [](const It &a, const It &b) {
        return a.sub != b.sub ? a.sub < b.sub : a.cost > b.cost;
    });
    if (items.size() > e->items_cap)
        return NBGB_ERR_NO_MEMORY;
    for (size_t k = 0; k < items.size(); k++)
        e->h_items[k] = items[k].v;
    e->n_items = (int)items.size();
    e->n_pass = 1;
    for (const It &it : items)
        e->n_pass = std::max(e->n_pass, it.sub);
    for (int p = 0; p < nbgb::ens::kMaxSub; p++) {
        int k = 0;
        while (k < e->n_items && items[k].sub <= p)
            k++;
        e->pass_first[p] = p == 0 ? 0 : k;
    }
    // slot map over the used part of the j-stream arena (pairs)
    size_t end = 0;
    for (int s = 0; s < e->max_systems; s++)
        if (e->sys[s].used)
            end = std::max(end, (e->sys[s].js_off + e->sys[s].js_len) / 2);
    const int n_pairs = (int)end;
    std::fill(e->h_slot_sys, e->h_slot_sys + n_pairs, -1);
    for (int s = 0; s < e->max_systems; s++) {
        const HostSys &h = e->sys[s];
        if (!h.used)
            continue;
        for (size_t q = h.js_off / 2; q < (h.js_off + h.js_len) / 2; q++)
            e->h_slot_sys[q] = s;
    }
    e->n_slots = n_pairs;
    // Newton-3 systems of this tick, with their block-pair prefix counts
    e->n_sym = 0;
    long long pairs = 0;
    const int sb = nbgb::sym_block_bodies();
    for (int s = 0; s < e->max_systems; s++) {
        const HostSys &h = e->sys[s];
        if (!h.used || !h.n3 || !(h.steps_left > 0 || !h.started))
            continue;
        nbgb::SymSystem &t = e->h_sym[e->n_sym++];
        t.pm = e->pm + h.body_off;
        t.js = e->js + h.js_off;
        t.acc = e->acc64 + h.acc_off;
        t.out = e->acc + h.body_off;
        t.n = h.n;
        t.npad = (int)(h.js_len);
        t.nblocks = (int)(h.js_len / sb);
        t.eps2 = e->eps2;
        t.pair_begin = pairs;
        pairs += (long long)t.nblocks * (t.nblocks + 1) / 2;
    }
    cudaStream_t st = e->stream;
    if (e->n_sym && cudaMemcpyAsync(e->d_sym, e->h_sym, sizeof(nbgb::SymSystem) * e->n_sym,
                                    cudaMemcpyHostToDevice, st) != cudaSuccess)
        return NBGB_ERR_CUDA;
    if (cudaMemcpyAsync(e->d_desc, e->h_desc, sizeof(Desc) * e->max_systems,
                        cudaMemcpyHostToDevice, st) != cudaSuccess ||
        (e->n_items &&
         cudaMemcpyAsync(e->d_items, e->h_items, sizeof(int4) * e->n_items, cudaMemcpyHostToDevice,
                         st) != cudaSuccess) ||
        (n_pairs && cudaMemcpyAsync(e->d_slot_sys, e->h_slot_sys, sizeof(int) * n_pairs,
                                    cudaMemcpyHostToDevice, st) != cudaSuccess))
        return NBGB_ERR_CUDA;
    if (e->graph) {
        cudaGraphExecDestroy(e->graph);
        e->graph = nullptr;
    }
    e->dirty = false;
    return NBGB_OK;
}

int launch_tick(nbgb_ensemble *e) {
    cudaStream_t st = e->stream;
    const int tb = 256;
    const int nb = std::max(1, (e->n_slots + tb - 1) / tb);
    for (int pass = 0; pass < e->n_pass; pass++) {
        const int first = e->pass_first[pass];
        const int n_items = e->n_items - first;
        if (pass > 0 && n_items <= 0)
            break;
        nbgb::ens::ens_kdk_kernel<<<nb, tb, 0, st>>>(e->d_desc, e->d_slot_sys, e->n_slots,
                                                     e->x64, e->max_bodies, e->mass, e->acc,
                                                     e->pm, e->js, 0, pass);
        if (cudaMemsetAsync(e->head, 0, sizeof(unsigned), st) != cudaSuccess)
            return NBGB_ERR_CUDA;
        nbgb::ens::Params P;
        P.desc = e->d_desc;
        P.items = e->d_items + first;
        P.n_items = n_items;
        P.head = e->head;
        P.pm = e->pm;
        P.js = e->js;
        P.acc = e->acc;
        P.part = e->part;
        P.cnt = e->cnt;
        if (n_items > 0)
            nbgb::ens::ens_force_kernel<<<e->grid, nbgb::ens::kThreads,
                                          nbgb::ens::kStages * nbgb::ens::kStageBytes, st>>>(P);
        if (pass == 0 && e->n_sym > 0) {
            const int rc = nbgb::launch_sym_systems(e->d_sym, e->h_sym, e->n_sym, st);
            if (rc != NBGB_OK)
                return rc;
        }
        nbgb::ens::ens_kdk_kernel<<<nb, tb, 0, st>>>(e->d_desc, e->d_slot_sys, e->n_slots,
                                                     e->x64, e->max_bodies, e->mass, e->acc,
                                                     e->pm, e->js, 1, pass);
    }
    return cudaGetLastError() == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

void free_ens(nbgb_ensemble *e) {
    if (e->graph)
        cudaGraphExecDestroy(e->graph);
    cudaFree(e->x64);
    cudaFree(e->mass);
    cudaFree(e->pm);
    cudaFree(e->acc);
    cudaFree(e->js);
    cudaFree(e->part);
    cudaFree(e->cnt);
    cudaFree(e->head);
    cudaFree(e->d_desc);
    cudaFree(e->d_items);
    cudaFree(e->d_slot_sys);
    cudaFree(e->acc64);
    cudaFree(e->d_sym);
    cudaFreeHost(e->h_sym);
    cudaFreeHost(e->h_desc);
    cudaFreeHost(e->h_items);
    cudaFreeHost(e->h_slot_sys);
    if (e->stream)
        cudaStreamDestroy(e->stream);
}

}  // namespace

extern "C" {

// Capacity: max_bodies bodies in total, max_systems concurrent systems.  The
// device arena is allocated once here (about 250 B per body of capacity,
// including partials for j-splits of up to 4); admission never allocates.
NBGB_API nbgb_ensemble *nbgb_ensemble_create(size_t max_bodies, int max_systems,
                                             float softeningSquared) {
    if (max_bodies == 0 || max_bodies > ((size_t)1 << 30) || max_systems <= 0)
        return nullptr;
    nbgb_ensemble *e = new (std::nothrow) nbgb_ensemble();
    if (!e)
        return nullptr;
    e->eps2 = softeningSquared;
    e->max_systems = max_systems;
    e->max_bodies = max_bodies;
    // j-stream: bodies rounded up to tiles (<= 1024 per system) or to
    // Newton-3 blocks, and to pairs
    e->js_cap = max_bodies +
                (size_t)max_systems * std::max(nbgb::ens::kMaxJT, nbgb::sym_block_bodies());
    e->js_cap += e->js_cap & 1;
    // split partials: hi + lo for up to 4-way j-splits of every body (plus
    // block padding); counters and items for up to 4 splits of 256-body blocks
    e->part_cap = 8 * (max_bodies + (size_t)max_systems * 512);
    e->cnt_cap = max_bodies / 256 + (size_t)max_systems + 1;
    e->items_cap = 4 * (max_bodies / 256 + (size_t)max_systems) + 64;
    e->sys.assign(max_systems, HostSys());
    e->a_body.init(max_bodies);
    e->a_js.init(e->js_cap);
    e->a_part.init(e->part_cap);
    e->a_cnt.init(e->cnt_cap);
    cudaGetDevice(&e->device);
    bool ok = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaMalloc(&e->x64, 6 * max_bodies * sizeof(double)) == cudaSuccess;
    ok = ok && cudaMalloc(&e->mass, max_bodies * sizeof(float)) == cudaSuccess;
    ok = ok && cudaMalloc(&e->pm, max_bodies * 16) == cudaSuccess;
    ok = ok && cudaMalloc(&e->acc, max_bodies * 16) == cudaSuccess;
    ok = ok && cudaMalloc(&e->js, e->js_cap * 16) == cudaSuccess;
    ok = ok && cudaMalloc(&e->part, e->part_cap * 16) == cudaSuccess;
    ok = ok && cudaMalloc(&e->cnt, e->cnt_cap * 4) == cudaSuccess;
    ok = ok && cudaMalloc(&e->head, 256) == cudaSuccess;
    ok = ok && cudaMalloc(&e->d_desc, sizeof(Desc) * max_systems) == cudaSuccess;
    ok = ok && cudaMalloc(&e->d_items, sizeof(int4) * e->items_cap) == cudaSuccess;
    ok = ok && cudaMalloc(&e->d_slot_sys, sizeof(int) * (e->js_cap / 2)) == cudaSuccess;
    ok = ok && cudaMallocHost(&e->h_desc, sizeof(Desc) * max_systems) == cudaSuccess;
    ok = ok && cudaMallocHost(&e->h_items, sizeof(int4) * e->items_cap) == cudaSuccess;
    ok = ok && cudaMallocHost(&e->h_slot_sys, sizeof(int) * (e->js_cap / 2)) == cudaSuccess;
    ok = ok && cudaMalloc(&e->d_sym, sizeof(nbgb::SymSystem) * max_systems) == cudaSuccess;
    ok = ok && cudaMallocHost(&e->h_sym, sizeof(nbgb::SymSystem) * max_systems) == cudaSuccess;
    ok = ok && cudaMemsetAsync(e->cnt, 0, e->cnt_cap * 4, e->stream) == cudaSuccess;
    ok = ok && cudaMemsetAsync(e->js, 0, e->js_cap * 16, e->stream) == cudaSuccess;
    ok = ok && cudaFuncSetAttribute(nbgb::ens::ens_force_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    nbgb::ens::kStages * nbgb::ens::kStageBytes) == cudaSuccess;
    int occ = 0, sms = 0;
    ok = ok && cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                   &occ, nbgb::ens::ens_force_kernel, nbgb::ens::kThreads,
                   nbgb::ens::kStages * nbgb::ens::kStageBytes) == cudaSuccess;
    ok = ok && cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->device) ==
                   cudaSuccess;
    ok = ok && cudaStreamSynchronize(e->stream) == cudaSuccess && occ > 0;
    if (!ok) {
        free_ens(e);
        delete e;
        return nullptr;
    }
    e->grid = sms * occ;
    e->grid_max = e->grid;
    e->bytes_total = max_bodies * (6 * 8 + 4 + 16 + 16) + e->js_cap * 16 + e->part_cap * 16 +
                     e->cnt_cap * 4;
    return e;
}

NBGB_API void nbgb_ensemble_destroy(nbgb_ensemble *e) {
    if (!e)
        return;
    cudaStreamSynchronize(e->stream);
    free_ens(e);
    delete e;
}

NBGB_API size_t nbgb_ensemble_device_bytes(nbgb_ensemble *e) { return e ? e->bytes_total : 0; }

// Per-bucket plan (bucket b: N in [2^b, 2^(b+1))): variant 0..3 (targets per
// thread and unroll: (1,8) (2,4) (1,4) (2,8)), tile a power of two in
// 16..1024 bodies, j-split 1..4; variant -1 restores the default rule.
// Applies to systems admitted afterwards.
NBGB_API int nbgb_ensemble_set_bucket_plan(nbgb_ensemble *e, int bucket, int variant, int jt,
                                           int nsplit) {
    if (!e || bucket < 0 || bucket >= 32 || variant < -1 || variant > 3)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (variant >= 0 &&
        (jt < 16 || jt > nbgb::ens::kMaxJT || (jt & (jt - 1)) || nsplit < 1 || nsplit > 4))
        return NBGB_ERR_INVALID_ARGUMENT;
    e->bucket[bucket].variant = variant;
    e->bucket[bucket].jt = jt;
    e->bucket[bucket].nsplit = nsplit;
    return NBGB_OK;
}

// Admit one system: HOST FP64 positions/velocities double[n][3], float masses.
// Returns NBGB_ERR_NO_MEMORY when no slot or not enough arena is free (the
// caller retries after systems retire).  *slot receives the system's slot.
NBGB_API int nbgb_ensemble_add(nbgb_ensemble *e, const double *pos3, const double *vel3,
                               const float *mass, size_t n, double dt, long long steps,
                               int *slot) {
    if (!e || !pos3 || !vel3 || !mass || !slot || n == 0 || n > e->max_bodies || steps < 0)
        return NBGB_ERR_INVALID_ARGUMENT;
    int s = -1;
    for (int k = 0; k < e->max_systems; k++)
        if (!e->sys[k].used) {
            s = k;
            break;
        }
    if (s < 0)
        return NBGB_ERR_NO_MEMORY;
    HostSys h;
    h.n = (int)n;
    choose_plan(e, (int)n, h);
    h.body_len = n;
    h.n3 = e->n3_min > 0 && n >= e->n3_min;
    if (h.n3) {  // j-stream padded to whole Newton-3 blocks, FP64 sums
        const size_t sb = (size_t)nbgb::sym_block_bodies();
        h.js_len = (n + sb - 1) / sb * sb;
        h.acc_len = 3 * h.js_len;
        h.part_len = h.cnt_len = 0;
    } else {
        h.js_len = (size_t)h.ntiles * h.jt;
        h.js_len += h.js_len & 1;
        h.part_len = h.nsplit > 1 ? 2 * (size_t)h.nsplit * h.ni_pad : 0;
        h.cnt_len = h.nsplit > 1 ? (size_t)h.nblocks : 0;
    }
    size_t ob, oj, op = 0, oc = 0, oa = 0;
    if (h.acc_len && !e->a_acc.alloc(h.acc_len, 32, oa))
        return NBGB_ERR_NO_MEMORY;
    if (!e->a_body.alloc(h.body_len, 1, ob)) {
        if (h.acc_len)
            e->a_acc.release(oa, h.acc_len);
        return NBGB_ERR_NO_MEMORY;
    }
    if (!e->a_js.alloc(h.js_len, 2, oj)) {
        e->a_body.release(ob, h.body_len);
        if (h.acc_len)
            e->a_acc.release(oa, h.acc_len);
        return NBGB_ERR_NO_MEMORY;
    }
    if (h.part_len && !e->a_part.alloc(h.part_len, 2, op)) {
        e->a_body.release(ob, h.body_len);
        e->a_js.release(oj, h.js_len);
        return NBGB_ERR_NO_MEMORY;
    }
    if (h.cnt_len && !e->a_cnt.alloc(h.cnt_len, 1, oc)) {
        e->a_body.release(ob, h.body_len);
        e->a_js.release(oj, h.js_len);
        if (h.part_len)
            e->a_part.release(op, h.part_len);
        return NBGB_ERR_NO_MEMORY;
    }
    h.acc_off = oa;
    h.body_off = ob;
    h.js_off = oj;
    h.part_off = op;
    h.cnt_off = oc;
    h.dt = dt;
    h.steps_left = steps;
    h.used = true;
    h.log_mass = !h.n3;  // the Newton-3 kernel reads plain masses
    for (size_t i = 0; i < n && h.log_mass; i++)
        h.log_mass = mass[i] >= 0.f;
    // upload state (SoA FP64, masses), zero the j-stream range
    std::vector<double> tmp(n);
    cudaStream_t st = e->stream;
    for (int c = 0; c < 6; c++) {
        const double *src = c < 3 ? pos3 : vel3;
        for (size_t i = 0; i < n; i++)
            tmp[i] = src[3 * i + (c % 3)];
        if (cudaMemcpyAsync(e->x64 + (size_t)c * e->max_bodies + ob, tmp.data(),
                            n * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return NBGB_ERR_CUDA;
    }
    if (cudaMemcpyAsync(e->mass + ob, mass, n * sizeof(float), cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaMemsetAsync(e->js + oj, 0, h.js_len * 16, st) != cudaSuccess ||
        (h.acc_len &&
         cudaMemsetAsync(e->acc64 + oa, 0, h.acc_len * sizeof(double), st) != cudaSuccess) ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return NBGB_ERR_CUDA;
    e->sys[s] = h;
    e->dirty = true;
    *slot = s;
    return NBGB_OK;
}

// One tick: every admitted system either gets its initial accelerations (its
// first tick) or advances one FP64 KDK step.  Asynchronous.
NBGB_API int nbgb_ensemble_tick(nbgb_ensemble *e, int nticks) {
    if (!e || nticks < 0)
        return NBGB_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < nticks; k++) {
        if (e->dirty) {
            int rc = rebuild(e);
            if (rc != NBGB_OK)
                return rc;
            e->stable_ticks = 0;
        }
        // A graph pays off only when it is replayed: capture it once the
        // membership has been unchanged for two ticks, launch eagerly before.
        if (e->use_graph && e->stable_ticks >= 2) {
            if (!e->graph) {
                cudaGraph_t g = nullptr;
                if (cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal) !=
                    cudaSuccess)
                    return NBGB_ERR_CUDA;
                int rc = launch_tick(e);
                cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
                if (rc != NBGB_OK || ce != cudaSuccess) {
                    if (g)
                        cudaGraphDestroy(g);
                    return NBGB_ERR_CUDA;
                }
                ce = cudaGraphInstantiate(&e->graph, g, 0);
                cudaGraphDestroy(g);
                if (ce != cudaSuccess)
                    return NBGB_ERR_CUDA;
            }
            if (cudaGraphLaunch(e->graph, e->stream) != cudaSuccess)
                return NBGB_ERR_CUDA;
        } else {
            int rc = launch_tick(e);
            if (rc != NBGB_OK)
                return rc;
        }
        e->stable_ticks++;
        e->ticks++;
        // host bookkeeping of this tick
        for (auto &h : e->sys) {
            if (!h.used)
                continue;
            if (!h.started) {
                h.started = true;
                e->dirty = true;  // moves from the next tick on
            } else if (h.steps_left > 0) {
                const int k = sub_eff(h);
                h.steps_left -= k;
                h.steps_done += k;
                if (h.steps_left < h.sub)
                    e->dirty = true;  // leaves the tick, or fewer steps next tick
            }
        }
    }
    return NBGB_OK;
}

// CTAs of the persistent force launch (1 .. SMs x resident CTAs; 0 = all).
// Two ensembles on one GPU can run side by side when their grids together
// fit the GPU's resident CTA slots.
NBGB_API int nbgb_ensemble_set_grid(nbgb_ensemble *e, int ctas) {
    if (!e || ctas < 0 || ctas > e->grid_max)
        return NBGB_ERR_INVALID_ARGUMENT;
    const int g = ctas == 0 ? e->grid_max : ctas;
    if (g != e->grid) {
        e->grid = g;
        if (e->graph) {  // the captured tick launches the old grid
            cudaGraphExecDestroy(e->graph);
            e->graph = nullptr;
        }
    }
    return NBGB_OK;
}

// Resident CTA slots of the persistent force launch on this device.
NBGB_API int nbgb_ensemble_max_grid(nbgb_ensemble *e) { return e ? e->grid_max : 0; }

NBGB_API int nbgb_ensemble_set_graph(nbgb_ensemble *e, int enable) {
    if (!e)
        return NBGB_ERR_INVALID_ARGUMENT;
    e->use_graph = enable != 0;
    return NBGB_OK;
}

NBGB_API int nbgb_ensemble_synchronize(nbgb_ensemble *e) {
    if (!e)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (cudaStreamSynchronize(e->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    unsigned bits = 0;
    if (nbgb::read_status_ensemble(&bits) != NBGB_OK)
        return NBGB_ERR_CUDA;
    return bits ? NBGB_ERR_DEVICE : NBGB_OK;
}

// Slots whose steps are all done (state synchronised in time), up to max.
NBGB_API int nbgb_ensemble_finished(nbgb_ensemble *e, int *slots, int max) {
    if (!e || (max > 0 && !slots))
        return NBGB_ERR_INVALID_ARGUMENT;
    int k = 0;
    for (int s = 0; s < e->max_systems && k < max; s++)
        if (e->sys[s].used && e->sys[s].started && e->sys[s].steps_left == 0)
            slots[k++] = s;
    return k;
}

// State of a slot (HOST double[n][3]); synchronises the stream first.
NBGB_API int nbgb_ensemble_get_state(nbgb_ensemble *e, int slot, double *pos3, double *vel3,
                                     float *acc4) {
    if (!e || slot < 0 || slot >= e->max_systems || !e->sys[slot].used)
        return NBGB_ERR_INVALID_ARGUMENT;
    const HostSys &h = e->sys[slot];
    const size_t n = h.n;
    std::vector<double> tmp(6 * n);
    cudaStream_t st = e->stream;
    for (int c = 0; c < 6; c++)
        if (cudaMemcpyAsync(tmp.data() + c * n, e->x64 + (size_t)c * e->max_bodies + h.body_off,
                            n * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
            return NBGB_ERR_CUDA;
    if (acc4 && cudaMemcpyAsync(acc4, e->acc + h.body_off, n * 16, cudaMemcpyDeviceToHost, st) !=
                    cudaSuccess)
        return NBGB_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess)
        return NBGB_ERR_CUDA;
    for (size_t i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) {
            if (pos3)
                pos3[3 * i + c] = tmp[c * n + i];
            if (vel3)
                vel3[3 * i + c] = tmp[(3 + c) * n + i];
        }
    return NBGB_OK;
}

// Slot info: bodies, steps done, steps left, plan (variant, tile, split).
NBGB_API int nbgb_ensemble_slot_info(nbgb_ensemble *e, int slot, long long *info6) {
    if (!e || slot < 0 || slot >= e->max_systems || !info6)
        return NBGB_ERR_INVALID_ARGUMENT;
    const HostSys &h = e->sys[slot];
    info6[0] = h.used ? h.n : 0;
    info6[1] = h.steps_done;
    info6[2] = h.steps_left;
    info6[3] = h.variant;
    info6[4] = h.jt;
    info6[5] = h.nsplit;
    return NBGB_OK;
}

// Steps per tick of one system (1..8); takes effect from the next tick.
NBGB_API int nbgb_ensemble_set_substeps(nbgb_ensemble *e, int slot, int sub) {
    if (!e || slot < 0 || slot >= e->max_systems || !e->sys[slot].used || sub < 1 ||
        sub > nbgb::ens::kMaxSub)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (e->sys[slot].sub != sub) {
        e->sys[slot].sub = sub;
        e->dirty = true;
    }
    return NBGB_OK;
}

// Stream priority of the ensemble's work: high = the device's greatest
// priority, so that its CTAs are dispatched ahead of other streams' pending
// CTAs as SMs free up (an ensemble beside a busier one).  Recreates the
// stream (after draining it).
NBGB_API int nbgb_ensemble_set_priority(nbgb_ensemble *e, int high) {
    if (!e)
        return NBGB_ERR_INVALID_ARGUMENT;
    int lo = 0, hi = 0;
    if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess ||
        cudaStreamSynchronize(e->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, high ? hi : lo) != cudaSuccess)
        return NBGB_ERR_CUDA;
    if (e->graph) {
        cudaGraphExecDestroy(e->graph);
        e->graph = nullptr;
    }
    cudaStreamDestroy(e->stream);
    e->stream = st;
    return NBGB_OK;
}

// Systems admitted from now on with at least nmin bodies use the Newton-3
// kernel (0: none).  The first nonzero call allocates the FP64 sums arena
// (24 B per body of capacity).
NBGB_API int nbgb_ensemble_set_newton3_min(nbgb_ensemble *e, size_t nmin) {
    if (!e)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (nmin > 0 && !e->acc64) {
        const size_t cap = 3 * (e->max_bodies + (size_t)e->max_systems *
                                                    (size_t)nbgb::sym_block_bodies());
        if (cudaMalloc(&e->acc64, cap * sizeof(double)) != cudaSuccess) {
            e->acc64 = nullptr;
            return NBGB_ERR_NO_MEMORY;
        }
        e->acc64_cap = cap;
        e->a_acc.init(cap);
        e->bytes_total += cap * sizeof(double);
    }
    e->n3_min = nmin;
    return NBGB_OK;
}

// Retire a slot: its arena ranges and slot become free for admission.
NBGB_API int nbgb_ensemble_remove(nbgb_ensemble *e, int slot) {
    if (!e || slot < 0 || slot >= e->max_systems || !e->sys[slot].used)
        return NBGB_ERR_INVALID_ARGUMENT;
    HostSys &h = e->sys[slot];
    // the stream may still run a tick that reads this slot's ranges
    if (cudaStreamSynchronize(e->stream) != cudaSuccess)
        return NBGB_ERR_CUDA;
    e->a_body.release(h.body_off, h.body_len);
    e->a_js.release(h.js_off, h.js_len);
    if (h.part_len)
        e->a_part.release(h.part_off, h.part_len);
    if (h.cnt_len)
        e->a_cnt.release(h.cnt_off, h.cnt_len);
    if (h.acc_len)
        e->a_acc.release(h.acc_off, h.acc_len);
    h = HostSys();
    e->dirty = true;
    return NBGB_OK;
}

NBGB_API int nbgb_ensemble_active(nbgb_ensemble *e) {
    if (!e)
        return 0;
    int k = 0;
    for (auto &h : e->sys)
        k += h.used ? 1 : 0;
    return k;
}

NBGB_API void *nbgb_ensemble_stream(nbgb_ensemble *e) { return e ? e->stream : nullptr; }

}  // extern "C"
