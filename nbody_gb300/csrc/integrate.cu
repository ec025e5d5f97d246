// integrate.cu -- the integration step on the GPU.
//
// Reference mode restates integrateOne (src/nbody.cu:158-182) as applied by
// integrateGravitation_SOA (src/nbody.cu:186-236): semi-implicit Euler with
// the reference's damping and its use of 1/m from velInvMass.w,
//     v += (F * invMass) * dt;  v *= damping;  x += v * dt
// in binary32 with every product and sum rounded separately (no FMA
// contraction), which is bit-identical to the same formula evaluated in IEEE
// single precision on the host.  The reference runs this on one host thread
// after copying forces back; here it is an HBM-bound kernel (80 B/body:
// read posMass, velInvMass, force; write posMass, velInvMass) that can also
// write the paired j-stream for the next force pass, so a resident step is
// force -> integrate with no host round trip.
//
// Physics mode (no reference counterpart) is FP64 kick-drift-kick leapfrog:
// positions and velocities live in FP64 (SoA), the force kernel's output is
// the acceleration (a = F: the sum already carries m_j), no damping.  The
// kick/drift kernel writes the FP32 posMass {x,y,z,m} and j-stream the next
// FP32 force pass reads.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "nbgb_device.cuh"
#include "nbgb_internal.h"
#include "nbody_gb300.h"

namespace nbgb {

// Thread q owns bodies 2q and 2q+1 (one j-stream pair).
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

__global__ void integrate_reference_kernel(float4 *__restrict__ pm, float4 *__restrict__ vel,
                                           const float4 *__restrict__ force, float dt,
                                           float damping, int n, float4 *__restrict__ js,
                                           int js_vpb, int js_log, int npad,
                                           unsigned *__restrict__ counters, int ncounters) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < ncounters)
        counters[q] = 0u;
    float4 out[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int i = 2 * q + h;
        if (i < n) {
            float4 p = pm[i];
            float4 v = vel[i];
            const float4 f = force[i];
            const float im = v.w;
            v.x = __fmul_rn(__fadd_rn(v.x, __fmul_rn(__fmul_rn(f.x, im), dt)), damping);
            v.y = __fmul_rn(__fadd_rn(v.y, __fmul_rn(__fmul_rn(f.y, im), dt)), damping);
            v.z = __fmul_rn(__fadd_rn(v.z, __fmul_rn(__fmul_rn(f.z, im), dt)), damping);
            p.x = __fadd_rn(p.x, __fmul_rn(v.x, dt));
            p.y = __fadd_rn(p.y, __fmul_rn(v.y, dt));
            p.z = __fadd_rn(p.z, __fmul_rn(v.z, dt));
            pm[i] = p;
            vel[i] = v;
            out[h] = p;
        } else {
            out[h] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    if (js && 2 * q < npad)
        store_jstream(js, js_vpb, js_log, q, out[0], out[1]);
}

// FP64 kick (v += a * kick_dt) then drift (x += v * drift_dt); either may be
// 0.  Writes posMass (FP32) and, if js != nullptr, the paired j-stream.
__global__ void kdk_kernel(double *__restrict__ px, double *__restrict__ py,
                           double *__restrict__ pz, double *__restrict__ vx,
                           double *__restrict__ vy, double *__restrict__ vz,
                           const float *__restrict__ mass, const float4 *__restrict__ accel,
                           double kick_dt, double drift_dt, int write_pos, int n,
                           float4 *__restrict__ pm, float4 *__restrict__ js, int js_vpb,
                           int js_log, int npad, unsigned *__restrict__ counters, int ncounters) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < ncounters)
        counters[q] = 0u;
    float4 out[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int i = 2 * q + h;
        if (i < n) {
            double x = px[i], y = py[i], z = pz[i];
            double u = vx[i], v = vy[i], w = vz[i];
            if (kick_dt != 0.0) {
                const float4 a = accel[i];
                u = fma((double)a.x, kick_dt, u);
                v = fma((double)a.y, kick_dt, v);
                w = fma((double)a.z, kick_dt, w);
                vx[i] = u;
                vy[i] = v;
                vz[i] = w;
            }
            if (drift_dt != 0.0) {
                x = fma(u, drift_dt, x);
                y = fma(v, drift_dt, y);
                z = fma(w, drift_dt, z);
                px[i] = x;
                py[i] = y;
                pz[i] = z;
            }
            out[h] = make_float4((float)x, (float)y, (float)z, mass[i]);
            if (write_pos)
                pm[i] = out[h];
        } else {
            out[h] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    if (write_pos && js && 2 * q < npad)
        store_jstream(js, js_vpb, js_log, q, out[0], out[1]);
}

int launch_integrate_reference(float4 *pm, float4 *vel, const float4 *force, float dt,
                               float damping, size_t n, float4 *js, int js_vpb, int js_log,
                               int npad, unsigned *counters, int ncounters, cudaStream_t st) {
    const int pairs = (int)((n + 1) / 2);
    const int work = std::max(std::max(pairs, npad / 2), ncounters);
    const int tb = 256;
    integrate_reference_kernel<<<(work + tb - 1) / tb, tb, 0, st>>>(
        pm, vel, force, dt, damping, (int)n, js, js_vpb, js_log, npad, counters, ncounters);
    return cudaGetLastError() == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

int launch_kdk(double *px, double *py, double *pz, double *vx, double *vy, double *vz,
               const float *mass, const float4 *accel, double kick_dt, double drift_dt,
               int write_pos, size_t n, float4 *pm, float4 *js, int js_vpb, int js_log, int npad,
               unsigned *counters, int ncounters, cudaStream_t st) {
    const int pairs = (int)((n + 1) / 2);
    const int work = std::max(std::max(pairs, npad / 2), ncounters);
    const int tb = 256;
    kdk_kernel<<<(work + tb - 1) / tb, tb, 0, st>>>(px, py, pz, vx, vy, vz, mass, accel, kick_dt,
                                                    drift_dt, write_pos, (int)n, pm, js, js_vpb,
                                                    js_log, npad, counters, ncounters);
    return cudaGetLastError() == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

static NBGB_STATUS_READER(read_status_integrate_tu)

int read_status_integrate(unsigned *bits) { return read_status_integrate_tu(bits); }

}  // namespace nbgb

extern "C" {

NBGB_API int nbgb_integrate_reference(float *posMass, float *velInvMass, const float *force,
                                      float dt, float damping, size_t N, void *stream) {
    if (N == 0)
        return NBGB_OK;
    if (!posMass || !velInvMass || !force || N > nbgb::kMaxBodies)
        return NBGB_ERR_INVALID_ARGUMENT;
    if (((uintptr_t)posMass | (uintptr_t)velInvMass | (uintptr_t)force) & 15u)
        return NBGB_ERR_INVALID_ARGUMENT;
    return nbgb::launch_integrate_reference((float4 *)posMass, (float4 *)velInvMass,
                                            (const float4 *)force, dt, damping, N, nullptr, 1, 0,
                                            0, nullptr, 0, (cudaStream_t)stream);
}

}  // extern "C"
