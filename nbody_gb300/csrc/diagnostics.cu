// diagnostics.cu -- conserved quantities of a resident system, in FP64.
//
// Kinetic energy 1/2 sum m v^2, potential energy 1/2 sum m_i phi_i (phi from
// the force kernel's potential mode, FP32 pair terms with compensated sums),
// linear momentum sum m v and angular momentum sum m (x cross v).  Each block
// reduces its bodies in FP64 in a fixed order and writes one partial row; a
// second one-block launch adds the rows in block order, so the result is
// deterministic.  No reference counterpart: the reference reports no energy
// (its integrator damps velocities, src/nbody.cu:151-182); these feed the
// FP64 kick-drift-kick precision study.
#include <cuda_runtime.h>

#include <cstdint>

#include "nbgb_internal.h"
#include "nbody_gb300.h"

namespace nbgb {

constexpr int kDiagThreads = 256;
constexpr int kDiagQ = 8;  // KE, PE, Px, Py, Pz, Lx, Ly, Lz

// Source of positions / velocities / masses: FP64 SoA (KDK; components ld
// doubles apart) when x64 != null, else the FP32 float4 arrays (reference
// integrator).
__global__ void __launch_bounds__(kDiagThreads) diag_partials_kernel(
    int n, const double *__restrict__ x64, size_t ld, const float *__restrict__ mass,
    const float4 *__restrict__ pm, const float4 *__restrict__ vel,
    const float4 *__restrict__ phi, double *__restrict__ part) {
    __shared__ double red[kDiagQ][kDiagThreads];
    double acc[kDiagQ] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * kDiagThreads + threadIdx.x; i < n; i += gridDim.x * kDiagThreads) {
        double m, x, y, z, u, v, w;
        if (x64) {
            m = mass[i];
            x = x64[i];
            y = x64[ld + i];
            z = x64[2 * ld + i];
            u = x64[3 * ld + i];
            v = x64[4 * ld + i];
            w = x64[5 * ld + i];
        } else {
            const float4 p = pm[i], q = vel[i];
            m = p.w;
            x = p.x;
            y = p.y;
            z = p.z;
            u = q.x;
            v = q.y;
            w = q.z;
        }
        acc[0] += 0.5 * m * (u * u + v * v + w * w);
        acc[1] += 0.5 * m * (double)phi[i].w;
        acc[2] += m * u;
        acc[3] += m * v;
        acc[4] += m * w;
        acc[5] += m * (y * w - z * v);
        acc[6] += m * (z * u - x * w);
        acc[7] += m * (x * v - y * u);
    }
#pragma unroll
    for (int q = 0; q < kDiagQ; q++)
        red[q][threadIdx.x] = acc[q];
    __syncthreads();
    for (int s = kDiagThreads / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
#pragma unroll
            for (int q = 0; q < kDiagQ; q++)
                red[q][threadIdx.x] += red[q][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < kDiagQ)
        part[(size_t)blockIdx.x * kDiagQ + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void diag_final_kernel(int nblocks, const double *__restrict__ part,
                                  double *__restrict__ out) {
    if (threadIdx.x < kDiagQ) {
        double s = 0.0;
        for (int b = 0; b < nblocks; b++)
            s += part[(size_t)b * kDiagQ + threadIdx.x];
        out[threadIdx.x] = s;
    }
}

int diag_blocks() { return 512; }
size_t diag_scratch_bytes() { return (size_t)(diag_blocks() + 1) * kDiagQ * sizeof(double); }

// scratch: diag_scratch_bytes() of device memory; out8 (device) receives the
// eight sums.
int launch_diagnostics(int n, const double *x64, size_t ld, const float *mass, const float4 *pm,
                       const float4 *vel, const float4 *phi, double *scratch, double *out8,
                       cudaStream_t st) {
    const int nb = diag_blocks();
    diag_partials_kernel<<<nb, kDiagThreads, 0, st>>>(n, x64, ld, mass, pm, vel, phi, scratch);
    diag_final_kernel<<<1, 32, 0, st>>>(nb, scratch, out8);
    return cudaGetLastError() == cudaSuccess ? NBGB_OK : NBGB_ERR_CUDA;
}

}  // namespace nbgb
