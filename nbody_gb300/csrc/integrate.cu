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
// Each thread owns one body, consecutive threads consecutive bodies, so every
// access of a warp is one contiguous run (float4 AOS: 512 B; FP64 SoA: 256 B;
// a thread owning a body pair instead made every float4 access a 32-byte
// stride, 25 % slower on GB300); the j-stream's source pairs are assembled
// with a lane swap.  GB300's FP64 pipe is narrow (~1.7
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

template <bool FUSED_DRIFT>
__device__ __forceinline__ float drift(float x, float v, float dt) {
    if constexpr (FUSED_DRIFT)
        return __fmaf_rn(v, dt, x);
    else
        return __fadd_rn(x, __fmul_rn(v, dt));
}

// One body per thread (i = global thread index; consecutive threads on
// consecutive bodies, so every float4 access is coalesced); the j-stream
// pairs are assembled with a lane swap (store_jstream_body).
template <bool FUSED_DRIFT>
__global__ void __launch_bounds__(kIntegrateThreads)
    integrate_reference_kernel(float4 *__restrict__ pm, float4 *__restrict__ vel,
                               const float4 *__restrict__ force, float dt, float damping, int n,
                               float4 *__restrict__ js, int js_vpb, int js_log, int npad,
                               unsigned *__restrict__ counters, int ncounters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ncounters)
        counters[i] = 0u;
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < n) {
        float4 pp = pm[i], vv = vel[i];
        const float4 ff = force[i];
        const float im = vv.w;
        vv.x = __fmul_rn(__fadd_rn(vv.x, __fmul_rn(__fmul_rn(ff.x, im), dt)), damping);
        vv.y = __fmul_rn(__fadd_rn(vv.y, __fmul_rn(__fmul_rn(ff.y, im), dt)), damping);
        vv.z = __fmul_rn(__fadd_rn(vv.z, __fmul_rn(__fmul_rn(ff.z, im), dt)), damping);
        pp.x = drift<FUSED_DRIFT>(pp.x, vv.x, dt);
        pp.y = drift<FUSED_DRIFT>(pp.y, vv.y, dt);
        pp.z = drift<FUSED_DRIFT>(pp.z, vv.z, dt);
        pm[i] = pp;
        vel[i] = vv;
        out = pp;
    }
    if (js)
        store_jstream_body(js, js_vpb, js_log, i, out, i < npad);
}

// FP64 kick then drift of body i (one per thread): v += a * kick_dt (skipped
// when kick_dt == 0), x += v * drift_dt; writes x, v, posMass and (js !=
// null) body i's j-stream entry.  x64: six SoA components of leading
// dimension ld (entries n..ld-1 are padding, never touched).
__global__ void __launch_bounds__(kIntegrateThreads)
    kick_drift_kernel(double *__restrict__ x64, size_t ld, const float *__restrict__ mass,
                      const float4 *__restrict__ accel, double kick_dt, double drift_dt, int n,
                      float4 *__restrict__ pm, float4 *__restrict__ js, int js_vpb, int js_log,
                      int npad, unsigned *__restrict__ counters, int ncounters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ncounters)
        counters[i] = 0u;
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < n) {
        double x = x64[i], y = x64[ld + i], z = x64[2 * ld + i];
        double u = x64[3 * ld + i], v = x64[4 * ld + i], w = x64[5 * ld + i];
        const float4 a = accel[i];
        const float m = mass[i];
        if (kick_dt != 0.0) {
            u = fma(widen_f32(a.x), kick_dt, u);
            v = fma(widen_f32(a.y), kick_dt, v);
            w = fma(widen_f32(a.z), kick_dt, w);
        }
        x = fma(u, drift_dt, x);
        y = fma(v, drift_dt, y);
        z = fma(w, drift_dt, z);
        x64[i] = x;
        x64[ld + i] = y;
        x64[2 * ld + i] = z;
        x64[3 * ld + i] = u;
        x64[4 * ld + i] = v;
        x64[5 * ld + i] = w;
        out = make_float4(narrow_f64(x), narrow_f64(y), narrow_f64(z), m);
        pm[i] = out;
    }
    if (js)
        store_jstream_body(js, js_vpb, js_log, i, out, i < npad);
}

// FP64 kick of body i (one per thread): v += a * kick_dt.
__global__ void __launch_bounds__(kIntegrateThreads)
    half_kick_kernel(double *__restrict__ x64, size_t ld, const float4 *__restrict__ accel,
                     double kick_dt, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double *u = x64 + 3 * ld + i, *v = x64 + 4 * ld + i, *w = x64 + 5 * ld + i;
    // every load before the first store (the three components are one
    // array to the compiler, which would otherwise order each load after the
    // previous component's store: three memory round trips instead of one)
    const double u0 = *u, v0 = *v, w0 = *w;
    const float4 a = accel[i];
    *u = fma(widen_f32(a.x), kick_dt, u0);
    *v = fma(widen_f32(a.y), kick_dt, v0);
    *w = fma(widen_f32(a.z), kick_dt, w0);
}

static inline unsigned blocks_for(int work) {
    return (unsigned)((std::max(work, 1) + kIntegrateThreads - 1) / kIntegrateThreads);
}

int launch_integrate_reference(float4 *pm, float4 *vel, const float4 *force, float dt,
                               float damping, size_t n, int fused_drift, float4 *js, int js_vpb,
                               int js_log, int npad, unsigned *counters, int ncounters,
                               cudaStream_t st) {
    const int work = std::max(std::max((int)n, npad), ncounters);
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
    const int work = std::max(std::max((int)n, npad), ncounters);
    kick_drift_kernel<<<blocks_for(work), kIntegrateThreads, 0, st>>>(
        x64, ld, mass, accel, kick_dt, drift_dt, (int)n, pm, js, js_vpb, js_log, npad, counters,
        ncounters);
    return cudaGetLastError() == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

int launch_half_kick(double *x64, size_t ld, const float4 *accel, double kick_dt, size_t n,
                     cudaStream_t st) {
    if ((ld & 1) || ld < n)
        return NBGB_ERR_INVALID_ARGUMENT;
    half_kick_kernel<<<blocks_for((int)n), kIntegrateThreads, 0, st>>>(x64, ld, accel, kick_dt,
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
