// integrate.cu -- the integration step on the GPU.
//
// Reference mode restates integrateOne (src/nbody.cu:158-182) as applied by
// integrateGravitation_SOA (src/nbody.cu:186-236): semi-implicit Euler with
// the reference's damping and its use of 1/m from velInvMass.w,
//     v += (F * invMass) * dt;  v *= damping;  x += v * dt
// in binary32 with every product and sum rounded separately (no FMA
// contraction), which is bit-identical to the same formula evaluated in IEEE
// single precision on the host.  The fused-drift variant computes
// x = fma(v, dt, x) instead: that is what the reference binary itself
// computes when built with its own flags (meson.build:33-38, -O3 -ffast-math
// -march=native: GCC contracts the position update and leaves the velocity
// update as written), bit for bit.  The reference runs this on one host
// thread after copying forces back; here it is an HBM-bound kernel (80 B per
// body: read posMass, velInvMass, force; write posMass, velInvMass) that can
// also write the paired j-stream for the next force pass (+16 B), so a
// resident step is force -> integrate with no host round trip.
//
// Physics mode (no reference counterpart) is FP64 kick-drift-kick leapfrog:
// positions and velocities live in FP64 (SoA, leading dimension ld, even),
// the force kernel's output is the acceleration (a = F: the sum already
// carries m_j), no damping.  Two kernels:
//   kick_drift  v += a * kick; x += v * dt; writes x, v, the FP32 posMass
//               {x,y,z,m} and the j-stream the next force pass reads
//               (148 B per body: read x, v 48, a 16, m 4; write x, v 48,
//               posMass 16, j-stream 16)
//   half_kick   v += a * dt/2, closing a leapfrog step (64 B per body: read
//               v 24, a 16; write v 24)
// Each thread owns one body pair (2q, 2q+1): FP64 components move as one
// 16-byte double2, FP32 masses as one float2, so every access is a 128-bit
// (or 64-bit) coalesced vector access.  GB300's FP64 pipe is narrow (~1.7
// operations per SM per clock), so the kernels keep FP64 for the updates
// themselves (6 DFMA per body in kick_drift, 3 in half_kick) and do the
// FP32 <-> FP64 conversions on the integer pipe (widen_f32 / narrow_f64,
// identical results): with the hardware conversions these kernels were
// FP64-pipe bound, not HBM bound.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "nbgb_device.cuh"
#include "nbgb_internal.h"
#include "nbody_gb300.h"

namespace nbgb {

constexpr int kIntegrateThreads = 256;

// j-stream store for bodies 2q, 2q+1 in either layout (vpb 1: source pairs,
// vpb 2: each source duplicated); logm: log2 masses in the pairs that carry
// them in log-domain plans.
__device__ __forceinline__ void store_jstream(float4 *__restrict__ js, int vpb, int logm, int q,
                                              float4 b0, float4 b1) {
    if (logm && jstream_log_slot(q)) {
        b0.w = jstream_log_mass(b0.w);
        b1.w = jstream_log_mass(b1.w);
    }
    if (vpb == 2) {
        js[4 * q] = make_float4(b0.x, b0.x, b0.y, b0.y);
        js[4 * q + 1] = make_float4(b0.z, b0.z, b0.w, b0.w);
        js[4 * q + 2] = make_float4(b1.x, b1.x, b1.y, b1.y);
        js[4 * q + 3] = make_float4(b1.z, b1.z, b1.w, b1.w);
    } else {
        js[2 * q] = make_float4(b0.x, b1.x, b0.y, b1.y);
        js[2 * q + 1] = make_float4(b0.z, b1.z, b0.w, b1.w);
    }
}

template <bool FUSED_DRIFT>
__device__ __forceinline__ float drift(float x, float v, float dt) {
    if constexpr (FUSED_DRIFT)
        return __fmaf_rn(v, dt, x);
    else
        return __fadd_rn(x, __fmul_rn(v, dt));
}

// Thread q owns bodies 2q and 2q+1 (one j-stream pair).
template <bool FUSED_DRIFT>
__global__ void __launch_bounds__(kIntegrateThreads)
    integrate_reference_kernel(float4 *__restrict__ pm, float4 *__restrict__ vel,
                               const float4 *__restrict__ force, float dt, float damping, int n,
                               float4 *__restrict__ js, int js_vpb, int js_log, int npad,
                               unsigned *__restrict__ counters, int ncounters) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < ncounters)
        counters[q] = 0u;
    float4 out[2];
    float4 p[2], v[2], f[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {  // all loads first (memory-level parallelism)
        const int i = 2 * q + h;
        if (i < n) {
            p[h] = pm[i];
            v[h] = vel[i];
            f[h] = force[i];
        }
    }
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int i = 2 * q + h;
        if (i < n) {
            float4 pp = p[h], vv = v[h];
            const float4 ff = f[h];
            const float im = vv.w;
            vv.x = __fmul_rn(__fadd_rn(vv.x, __fmul_rn(__fmul_rn(ff.x, im), dt)), damping);
            vv.y = __fmul_rn(__fadd_rn(vv.y, __fmul_rn(__fmul_rn(ff.y, im), dt)), damping);
            vv.z = __fmul_rn(__fadd_rn(vv.z, __fmul_rn(__fmul_rn(ff.z, im), dt)), damping);
            pp.x = drift<FUSED_DRIFT>(pp.x, vv.x, dt);
            pp.y = drift<FUSED_DRIFT>(pp.y, vv.y, dt);
            pp.z = drift<FUSED_DRIFT>(pp.z, vv.z, dt);
            pm[i] = pp;
            vel[i] = vv;
            out[h] = pp;
        } else {
            out[h] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    if (js && 2 * q < npad)
        store_jstream(js, js_vpb, js_log, q, out[0], out[1]);
}

__device__ __forceinline__ double2 ld_d2(const double *p) {
    return *reinterpret_cast<const double2 *>(p);
}
__device__ __forceinline__ void st_d2(double *p, double a, double b) {
    *reinterpret_cast<double2 *>(p) = make_double2(a, b);
}

// FP64 kick then drift of bodies 2q, 2q+1: v += a * kick_dt (skipped when
// kick_dt == 0), x += v * drift_dt; writes x, v, posMass and (js != null)
// the j-stream pair q.  x64: six SoA components of leading dimension ld
// (even; entries n..ld-1 are padding).
__global__ void __launch_bounds__(kIntegrateThreads)
    kick_drift_kernel(double *__restrict__ x64, size_t ld, const float *__restrict__ mass,
                      const float4 *__restrict__ accel, double kick_dt, double drift_dt, int n,
                      float4 *__restrict__ pm, float4 *__restrict__ js, int js_vpb, int js_log,
                      int npad, unsigned *__restrict__ counters, int ncounters) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < ncounters)
        counters[q] = 0u;
    const int i0 = 2 * q;
    float4 out0 = make_float4(0.f, 0.f, 0.f, 0.f), out1 = out0;
    if (i0 < n) {
        const bool two = i0 + 1 < n;
        double2 X = ld_d2(x64 + i0), Y = ld_d2(x64 + ld + i0), Z = ld_d2(x64 + 2 * ld + i0);
        double2 U = ld_d2(x64 + 3 * ld + i0), V = ld_d2(x64 + 4 * ld + i0),
                W = ld_d2(x64 + 5 * ld + i0);
        const float4 a0 = accel[i0];
        const float4 a1 = two ? accel[i0 + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
        float2 m;
        if (two)
            m = *reinterpret_cast<const float2 *>(mass + i0);
        else
            m = make_float2(mass[i0], 0.f);
        if (kick_dt != 0.0) {
            U.x = fma(widen_f32(a0.x), kick_dt, U.x);
            V.x = fma(widen_f32(a0.y), kick_dt, V.x);
            W.x = fma(widen_f32(a0.z), kick_dt, W.x);
            U.y = fma(widen_f32(a1.x), kick_dt, U.y);
            V.y = fma(widen_f32(a1.y), kick_dt, V.y);
            W.y = fma(widen_f32(a1.z), kick_dt, W.y);
        }
        X.x = fma(U.x, drift_dt, X.x);
        Y.x = fma(V.x, drift_dt, Y.x);
        Z.x = fma(W.x, drift_dt, Z.x);
        X.y = fma(U.y, drift_dt, X.y);
        Y.y = fma(V.y, drift_dt, Y.y);
        Z.y = fma(W.y, drift_dt, Z.y);
        // the padding entry of an odd n is written back as read
        st_d2(x64 + i0, X.x, X.y);
        st_d2(x64 + ld + i0, Y.x, Y.y);
        st_d2(x64 + 2 * ld + i0, Z.x, Z.y);
        st_d2(x64 + 3 * ld + i0, U.x, U.y);
        st_d2(x64 + 4 * ld + i0, V.x, V.y);
        st_d2(x64 + 5 * ld + i0, W.x, W.y);
        out0 = make_float4(narrow_f64(X.x), narrow_f64(Y.x), narrow_f64(Z.x), m.x);
        pm[i0] = out0;
        if (two) {
            out1 = make_float4(narrow_f64(X.y), narrow_f64(Y.y), narrow_f64(Z.y), m.y);
            pm[i0 + 1] = out1;
        }
    }
    if (js && i0 < npad)
        store_jstream(js, js_vpb, js_log, q, out0, out1);
}

// FP64 kick of bodies 2q, 2q+1: v += a * kick_dt.
__global__ void __launch_bounds__(kIntegrateThreads)
    half_kick_kernel(double *__restrict__ x64, size_t ld, const float4 *__restrict__ accel,
                     double kick_dt, int n) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int i0 = 2 * q;
    if (i0 >= n)
        return;
    const bool two = i0 + 1 < n;
    double *u = x64 + 3 * ld + i0, *v = x64 + 4 * ld + i0, *w = x64 + 5 * ld + i0;
    double2 U = ld_d2(u), V = ld_d2(v), W = ld_d2(w);
    const float4 a0 = accel[i0];
    const float4 a1 = two ? accel[i0 + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
    U.x = fma(widen_f32(a0.x), kick_dt, U.x);
    V.x = fma(widen_f32(a0.y), kick_dt, V.x);
    W.x = fma(widen_f32(a0.z), kick_dt, W.x);
    U.y = fma(widen_f32(a1.x), kick_dt, U.y);
    V.y = fma(widen_f32(a1.y), kick_dt, V.y);
    W.y = fma(widen_f32(a1.z), kick_dt, W.y);
    st_d2(u, U.x, U.y);
    st_d2(v, V.x, V.y);
    st_d2(w, W.x, W.y);
}

static inline unsigned blocks_for(int work) {
    return (unsigned)((std::max(work, 1) + kIntegrateThreads - 1) / kIntegrateThreads);
}

int launch_integrate_reference(float4 *pm, float4 *vel, const float4 *force, float dt,
                               float damping, size_t n, int fused_drift, float4 *js, int js_vpb,
                               int js_log, int npad, unsigned *counters, int ncounters,
                               cudaStream_t st) {
    const int pairs = (int)((n + 1) / 2);
    const int work = std::max(std::max(pairs, npad / 2), ncounters);
    if (fused_drift)
        integrate_reference_kernel<true><<<blocks_for(work), kIntegrateThreads, 0, st>>>(
            pm, vel, force, dt, damping, (int)n, js, js_vpb, js_log, npad, counters, ncounters);
    else
        integrate_reference_kernel<false><<<blocks_for(work), kIntegrateThreads, 0, st>>>(
            pm, vel, force, dt, damping, (int)n, js, js_vpb, js_log, npad, counters, ncounters);
    return cudaGetLastError() == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

int launch_kick_drift(double *x64, size_t ld, const float *mass, const float4 *accel,
                      double kick_dt, double drift_dt, size_t n, float4 *pm, float4 *js,
                      int js_vpb, int js_log, int npad, unsigned *counters, int ncounters,
                      cudaStream_t st) {
    if ((ld & 1) || ld < n)
        return NBGB_ERR_INVALID_ARGUMENT;
    const int pairs = (int)((n + 1) / 2);
    const int work = std::max(std::max(pairs, npad / 2), ncounters);
    kick_drift_kernel<<<blocks_for(work), kIntegrateThreads, 0, st>>>(
        x64, ld, mass, accel, kick_dt, drift_dt, (int)n, pm, js, js_vpb, js_log, npad, counters,
        ncounters);
    return cudaGetLastError() == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

int launch_half_kick(double *x64, size_t ld, const float4 *accel, double kick_dt, size_t n,
                     cudaStream_t st) {
    if ((ld & 1) || ld < n)
        return NBGB_ERR_INVALID_ARGUMENT;
    const int pairs = (int)((n + 1) / 2);
    half_kick_kernel<<<blocks_for(pairs), kIntegrateThreads, 0, st>>>(x64, ld, accel, kick_dt,
                                                                      (int)n);
    return cudaGetLastError() == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

// Self-test of widen_f32 / narrow_f64 against the hardware conversions on n
// pseudo-random bit patterns of every class (splitmix64 of the index): adds
// the number of mismatches to *bad.
__global__ void conversion_selftest_kernel(unsigned long long seed, long long n,
                                           unsigned long long *bad) {
    unsigned long long local = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        unsigned long long z = seed + (unsigned long long)i * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        // exponent fields drawn across the whole range, and near the
        // boundaries of the fast paths, half of the time
        unsigned long long bits = z;
        if (z & 1ull) {
            const unsigned e = 880u + (unsigned)((z >> 1) % 290u);  // 880..1169
            bits = (z & 0x800fffffffffffffull) | ((unsigned long long)e << 52);
        }
        const double d = __longlong_as_double((long long)bits);
        const float a = narrow_f64(d), b = (float)d;
        if (__float_as_uint(a) != __float_as_uint(b) && !(a != a && b != b))
            local++;
        const float f = __uint_as_float((unsigned)(z >> 32));
        const double wa = widen_f32(f), wb = (double)f;
        if (__double_as_longlong(wa) != __double_as_longlong(wb) && !(wa != wa && wb != wb))
            local++;
    }
    if (local)
        atomicAdd(bad, local);
}

static NBGB_STATUS_READER(read_status_integrate_tu)

int read_status_integrate(unsigned *bits) { return read_status_integrate_tu(bits); }

}  // namespace nbgb

extern "C" {

NBGB_API int nbgb_integrate_reference_ex(float *posMass, float *velInvMass, const float *force,
                                         float dt, float damping, size_t N, int fused_drift,
                                         void *stream) {
    if (N == 0)
        return NBGB_OK;
    if (!posMass || !velInvMass || !force || N > nbgb::kMaxBodies ||
        (fused_drift != 0 && fused_drift != 1))
        return NBGB_ERR_INVALID_ARGUMENT;
    if (((uintptr_t)posMass | (uintptr_t)velInvMass | (uintptr_t)force) & 15u)
        return NBGB_ERR_INVALID_ARGUMENT;
    return nbgb::launch_integrate_reference((float4 *)posMass, (float4 *)velInvMass,
                                            (const float4 *)force, dt, damping, N, fused_drift,
                                            nullptr, 1, 0, 0, nullptr, 0, (cudaStream_t)stream);
}

NBGB_API int nbgb_integrate_reference(float *posMass, float *velInvMass, const float *force,
                                      float dt, float damping, size_t N, void *stream) {
    return nbgb_integrate_reference_ex(posMass, velInvMass, force, dt, damping, N, 0, stream);
}

// Runs the conversion self-test on n patterns; *mismatches gets the count of
// results that differ from the hardware conversions (0 expected).
// Synchronous.
NBGB_API int nbgb_selftest_conversions(long long n, unsigned long long seed,
                                       unsigned long long *mismatches) {
    if (n <= 0 || !mismatches)
        return NBGB_ERR_INVALID_ARGUMENT;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess)
        return NBGB_ERR_CUDA;
    int rc = NBGB_OK;
    if (cudaMemset(d, 0, sizeof(*d)) != cudaSuccess)
        rc = NBGB_ERR_CUDA;
    if (rc == NBGB_OK) {
        nbgb::conversion_selftest_kernel<<<1024, 256>>>(seed, n, d);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpy(mismatches, d, sizeof(*d), cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = NBGB_ERR_CUDA;
    }
    cudaFree(d);
    return rc;
}

}  // extern "C"
