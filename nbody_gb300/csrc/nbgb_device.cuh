// nbgb_device.cuh -- device-side building blocks shared by the GB300 kernels.
//
//  * the pair interaction of src/bodybodyInteraction.cuh:40-65, in a scalar
//    form and in a packed form that evaluates two interactions per
//    instruction with the sm_100-family f32x2 FP32 instructions;
//  * Knuth's TwoSum for compensated accumulation across j-tiles;
//  * mbarrier + 1-D bulk-copy (TMA) wrappers whose waits are bounded in time:
//    a wait that runs out sets a bit in the device status word and returns
//    false instead of spinning forever.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "nbgb_status.h"

namespace nbgb {

// Device status word: bits from nbgb_status.h, OR-ed in by kernels that hit a
// bounded wait or an internal consistency check.  Each translation unit has
// its own copy (no relocatable device code); NBGB_STATUS_READER defines the
// host function that reads and clears it, and nbgb_last_status() ORs them.
static __device__ unsigned int g_status = 0;

#define NBGB_STATUS_READER(name)                                                   \
    int name(unsigned *bits) {                                                     \
        unsigned v = 0, z = 0;                                                     \
        if (cudaMemcpyFromSymbol(&v, g_status, sizeof(v)) != cudaSuccess)          \
            return NBGB_ERR_CUDA;                                                  \
        if (v && cudaMemcpyToSymbol(g_status, &z, sizeof(z)) != cudaSuccess)       \
            return NBGB_ERR_CUDA;                                                  \
        *bits |= v;                                                                \
        return NBGB_OK;                                                            \
    }

// ---------------------------------------------------------------------------
// Packed FP32 pairs.  A u64 holds (lo, hi) = two binary32 values in adjacent
// registers; add/fma/mul.f32x2 run both halves in one instruction.
// ---------------------------------------------------------------------------
typedef unsigned long long f2;

__device__ __forceinline__ f2 f2_pack(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
    f2 d;
    asm("add.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// MUFU reciprocal square root (the reference's rsqrtf on the SFU pipe).
__device__ __forceinline__ float rsqrt_mufu(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Two interactions at once: sources (x0,x1),(y0,y1),(z0,z1),(m0,m1) against
// one target whose negated position is held duplicated in (nx,nx) etc.
// Same arithmetic as bodyBodyInteraction, with eps2 folded into the first FMA
// of the squared distance.
__device__ __forceinline__ void pair_interact2(f2 sx, f2 sy, f2 sz, f2 sm,
                                               f2 nx, f2 ny, f2 nz, f2 eps2,
                                               f2 &ax, f2 &ay, f2 &az) {
    f2 dx = f2_add(sx, nx);
    f2 dy = f2_add(sy, ny);
    f2 dz = f2_add(sz, nz);
    f2 d2 = f2_fma(dx, dx, eps2);
    d2 = f2_fma(dy, dy, d2);
    d2 = f2_fma(dz, dz, d2);
    float d2l, d2h;
    f2_unpack(d2, d2l, d2h);
    f2 inv = f2_pack(rsqrt_mufu(d2l), rsqrt_mufu(d2h));
    f2 inv2 = f2_mul(inv, inv);
    f2 s = f2_mul(sm, inv);
    s = f2_mul(s, inv2);
    ax = f2_fma(dx, s, ax);
    ay = f2_fma(dy, s, ay);
    az = f2_fma(dz, s, az);
}

// pair_interact2 plus the potential sum ap += m * rsqrt(d2).
__device__ __forceinline__ void pair_interact2_pot(f2 sx, f2 sy, f2 sz, f2 sm, f2 nx, f2 ny,
                                                   f2 nz, f2 eps2, f2 &ax, f2 &ay, f2 &az,
                                                   f2 &ap) {
    f2 dx = f2_add(sx, nx);
    f2 dy = f2_add(sy, ny);
    f2 dz = f2_add(sz, nz);
    f2 d2 = f2_fma(dx, dx, eps2);
    d2 = f2_fma(dy, dy, d2);
    d2 = f2_fma(dz, dz, d2);
    float d2l, d2h;
    f2_unpack(d2, d2l, d2h);
    f2 inv = f2_pack(rsqrt_mufu(d2l), rsqrt_mufu(d2h));
    f2 inv2 = f2_mul(inv, inv);
    f2 s = f2_mul(sm, inv);
    ap = f2_add(ap, s);
    s = f2_mul(s, inv2);
    ax = f2_fma(dx, s, ax);
    ay = f2_fma(dy, s, ay);
    az = f2_fma(dz, s, az);
}

// As pair_interact2, but every add and multiply is issued as an FMA
// (a + b = fma(a, 1, b), a * b = fma(a, b, 0)); results are identical because
// each FMA still rounds once.
__device__ __forceinline__ void pair_interact2_fma(f2 sx, f2 sy, f2 sz, f2 sm,
                                                   f2 nx, f2 ny, f2 nz, f2 eps2, f2 one,
                                                   f2 zero, f2 &ax, f2 &ay, f2 &az) {
    f2 dx = f2_fma(sx, one, nx);
    f2 dy = f2_fma(sy, one, ny);
    f2 dz = f2_fma(sz, one, nz);
    f2 d2 = f2_fma(dx, dx, eps2);
    d2 = f2_fma(dy, dy, d2);
    d2 = f2_fma(dz, dz, d2);
    float d2l, d2h;
    f2_unpack(d2, d2l, d2h);
    f2 inv = f2_pack(rsqrt_mufu(d2l), rsqrt_mufu(d2h));
    f2 inv2 = f2_fma(inv, inv, zero);
    f2 s = f2_fma(sm, inv, zero);
    s = f2_fma(s, inv2, zero);
    ax = f2_fma(dx, s, ax);
    ay = f2_fma(dy, s, ay);
    az = f2_fma(dz, s, az);
}

// MUFU base-2 exponential and logarithm.
__device__ __forceinline__ float ex2_mufu(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float lg2_mufu(float x) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// pair_interact2 with the scale m * d2^(-3/2) taken in the log domain:
// s = 2^(log2 m - 1.5 log2 d2), where the source slot holds lm = log2 m
// (-inf for a zero mass, giving s = 0).  One packed FMA, two MUFU lg2 and two
// MUFU ex2 replace two MUFU rsqrt and three packed multiplies.  On sm_103 ex2
// issues at twice the rsqrt / lg2 rate, so mixing both forms moves work from
// the FMA pipe (the bound) to the MUFU pipe.
__device__ __forceinline__ void pair_interact2_log(f2 sx, f2 sy, f2 sz, f2 lm, f2 nx, f2 ny,
                                                   f2 nz, f2 eps2, f2 m15, f2 &ax, f2 &ay,
                                                   f2 &az) {
    f2 dx = f2_add(sx, nx);
    f2 dy = f2_add(sy, ny);
    f2 dz = f2_add(sz, nz);
    f2 d2 = f2_fma(dx, dx, eps2);
    d2 = f2_fma(dy, dy, d2);
    d2 = f2_fma(dz, dz, d2);
    float d2l, d2h;
    f2_unpack(d2, d2l, d2h);
    f2 e = f2_fma(f2_pack(lg2_mufu(d2l), lg2_mufu(d2h)), m15, lm);
    float el, eh;
    f2_unpack(e, el, eh);
    f2 s = f2_pack(ex2_mufu(el), ex2_mufu(eh));
    ax = f2_fma(dx, s, ax);
    ay = f2_fma(dy, s, ay);
    az = f2_fma(dz, s, az);
}

// j-stream pairs that carry log2 masses in log-domain (mode 6) plans: pair q
// with q % 4 == 0 (tiles hold whole groups of 4 pairs, so the tile-local and
// the global pair index agree modulo 4).
__device__ __forceinline__ bool jstream_log_slot(int q) { return (q & 3) == 0; }

// log2 m for those pairs: -inf for m == 0 (the pair then contributes 0, as
// zero-mass padding must).  A negative (or NaN) mass has no logarithm: NaN is
// stored, so the forces come out NaN, and NBGB_STATUS_NEGATIVE_MASS is set.
__device__ __forceinline__ float jstream_log_mass(float m) {
    if (m > 0.f)
        return log2f(m);
    if (m == 0.f)
        return __int_as_float(0xff800000);  // -inf
    atomicOr(&g_status, NBGB_STATUS_NEGATIVE_MASS);
    return __int_as_float(0x7fc00000);  // NaN
}

// Body i's entry of the j-stream, written by the thread that owns body i (one
// body per thread, consecutive threads on consecutive bodies, so every load
// and store of the caller is coalesced).  Paired layout (vpb 1): lanes i and
// i ^ 1 (one warp: blocks are whole warps and i is the thread's global
// index) swap their bodies, the even lane stores float4 2q = {x0,x1,y0,y1}
// and the odd lane 2q+1 = {z0,z1,m0,m1}; duplicated layout (vpb 2): each
// lane stores its body's {x,x,y,y}, {z,z,m,m}.  logm: pair q % 4 == 0 holds
// log2 of the masses.  Every lane of the warp calls it (shuffles); lanes with
// in_range false (beyond the padded length) store nothing.
__device__ __forceinline__ void store_jstream_body(float4 *__restrict__ js, int vpb, int logm,
                                                   int i, float4 b, bool in_range) {
    const int q = i >> 1;
    if (logm && jstream_log_slot(q))
        b.w = jstream_log_mass(b.w);
    if (vpb == 2) {
        if (in_range) {
            js[2 * i] = make_float4(b.x, b.x, b.y, b.y);
            js[2 * i + 1] = make_float4(b.z, b.z, b.w, b.w);
        }
        return;
    }
    const float ox = __shfl_xor_sync(0xffffffffu, b.x, 1);
    const float oy = __shfl_xor_sync(0xffffffffu, b.y, 1);
    const float oz = __shfl_xor_sync(0xffffffffu, b.z, 1);
    const float ow = __shfl_xor_sync(0xffffffffu, b.w, 1);
    if (!in_range)
        return;
    if ((i & 1) == 0)
        js[2 * q] = make_float4(b.x, ox, b.y, oy);
    else
        js[2 * q + 1] = make_float4(oz, b.z, ow, b.w);
}

// One interaction, scalar FP32 pipe.
__device__ __forceinline__ void pair_interact1(float sx, float sy, float sz, float sm,
                                               float x, float y, float z, float eps2,
                                               float &ax, float &ay, float &az) {
    float dx = sx - x, dy = sy - y, dz = sz - z;
    float d2 = fmaf(dx, dx, eps2);
    d2 = fmaf(dy, dy, d2);
    d2 = fmaf(dz, dz, d2);
    float inv = rsqrt_mufu(d2);
    float s = (sm * inv) * (inv * inv);
    ax = fmaf(dx, s, ax);
    ay = fmaf(dy, s, ay);
    az = fmaf(dz, s, az);
}

// Knuth TwoSum: s + e == a + b exactly (round-to-nearest, no FTZ hazards for
// the magnitudes involved).  __fadd_rn / __fsub_rn keep the compiler from
// reassociating.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float aa = __fsub_rn(s, bb);
    e = __fadd_rn(__fsub_rn(a, aa), __fsub_rn(b, bb));
}

// Running compensated sum (hi, lo): add t.
__device__ __forceinline__ void comp_add(float &hi, float &lo, float t) {
    float s, e;
    two_sum(hi, t, s, e);
    hi = s;
    lo = __fadd_rn(lo, e);
}

// ---------------------------------------------------------------------------
// Binary32 <-> binary64 conversions on the integer pipe.
//
// GB300 executes FP64 arithmetic at ~1.7 operations per SM per clock, and
// the hardware conversions cvt.f64.f32 / cvt.rn.f32.f64 run on that same
// pipe (measured: a conversion costs as much as a DADD).  The FP64 integrate
// kernels convert every acceleration component in and every position out,
// so the conversions alone doubled their FP64-pipe time.  These versions do
// the common cases with a few 32-bit integer operations and give results
// identical to the hardware instructions; the rare cases (zero and
// subnormal inputs to the widening, results outside the normal binary32
// range for the narrowing, infinities and NaNs) take the hardware path.
// ---------------------------------------------------------------------------

// (double)f, exactly.  A normal binary32 (biased exponent e in 1..254) is
// the binary64 with exponent e + 896 and its 23 mantissa bits on top.
__device__ __forceinline__ double widen_f32(float f) {
    const uint32_t u = __float_as_uint(f);
    if (((u >> 23) & 0xffu) - 1u < 254u) {
        const uint32_t hi = (((u >> 3) & 0x0fffffffu) + 0x38000000u) | (u & 0x80000000u);
        return __hiloint2double((int)hi, (int)(u << 29));
    }
    return (double)f;
}

// (float)d with round-to-nearest-even, exactly.  For a biased binary64
// exponent e in 897..1150 the result is a normal binary32 (or, when the
// rounding carries out of the largest one, infinity, as cvt.rn gives): keep
// the top 23 mantissa bits, round on the 29 dropped ones (ties to even).
__device__ __forceinline__ float narrow_f64(double d) {
    const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
    const uint32_t e = (hi >> 20) & 0x7ffu;
    if (e - 897u < 254u) {
        uint32_t f = (hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
        const uint32_t rest = lo & 0x1fffffffu;
        f += (rest > 0x10000000u) | ((rest == 0x10000000u) & f);
        return __uint_as_float(f);
    }
    return (float)d;
}

// ---------------------------------------------------------------------------
// mbarrier and 1-D bulk copies (cp.async.bulk, the non-tensor TMA path).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

// Global -> shared bulk copy completing on `bar`.  dst, src 16-byte aligned,
// bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, "
        "p; }"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Shared-memory add with acquire-release semantics at CTA scope: a warp that
// finished reading a ring stage releases it; the warp that completes the
// count acquires every other warp's reads before reusing the stage.
__device__ __forceinline__ unsigned atom_add_acqrel_shared(unsigned *p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], %2;"
                 : "=r"(old)
                 : "r"(smem_addr(p)), "r"(v)
                 : "memory");
    return old;
}

// Orders this thread's (acquired) generic-proxy shared-memory accesses before
// its following async-proxy (bulk copy) accesses to shared memory.
__device__ __forceinline__ void fence_proxy_async_shared() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for phase `parity` of `bar`, giving up after `limit_ns` nanoseconds.
// On timeout the status word gets NBGB_STATUS_WAIT_TIMEOUT and false is
// returned; the caller must leave its loop.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint64_t limit_ns = 2000000000ull) {
    if (mbar_try_wait(bar, parity))
        return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        for (int k = 0; k < 64; k++)
            if (mbar_try_wait(bar, parity))
                return true;
        if (global_ns() - t0 > limit_ns) {
            atomicOr(&g_status, NBGB_STATUS_WAIT_TIMEOUT);
            return false;
        }
    }
}

}  // namespace nbgb
