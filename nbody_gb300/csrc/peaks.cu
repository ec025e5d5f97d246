// peaks.cu -- microbenchmarks of the pipes the force kernel is bound by,
// measured on the running GPU so the roofline denominators are this chip's.
//
//   fp32 FFMA      scalar fma.rn.f32, 16 independent chains per thread
//   fp32x2 FFMA2   packed fma.rn.f32x2 (two FMAs per instruction)
//   MUFU rsqrt     rsqrt.approx.ftz.f32, 16 independent chains per thread
//
// FLOP/s counts an FMA as 2 FLOP.  Each kernel runs a full GPU of resident
// warps (SMs x 8 CTAs x 256 threads) and is timed with CUDA events after a
// warm-up launch; the best of `reps` launches is reported.
#include <cuda_runtime.h>

#include <cstdint>
#include <new>

#include "nbgb_device.cuh"
#include "nbody_gb300.h"

namespace nbgb {

constexpr int kChains = 16;

__global__ void __launch_bounds__(256) peak_ffma_kernel(float *out, int iters, float a, float b) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++)
        x[c] = (float)(threadIdx.x + c);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 8; u++)
#pragma unroll
            for (int c = 0; c < kChains; c++)
                asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(x[c]) : "f"(a), "f"(b));
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; c++)
        s += x[c];
    if (s == 1234.5f)
        out[threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) peak_ffma2_kernel(float *out, int iters, float a, float b) {
    f2 x[kChains];
    const f2 aa = f2_pack(a, a), bb = f2_pack(b, b);
#pragma unroll
    for (int c = 0; c < kChains; c++)
        x[c] = f2_pack((float)threadIdx.x, (float)c);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 8; u++)
#pragma unroll
            for (int c = 0; c < kChains; c++)
                asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x[c]) : "l"(aa), "l"(bb));
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; c++) {
        float l, h;
        f2_unpack(x[c], l, h);
        s += l + h;
    }
    if (s == 1234.5f)
        out[threadIdx.x] = s;
}

// Packed add / mul throughput (which = 3 / 4), and FFMA2 with three varying
// operands (which = 5), for comparison with the FFMA2 rate above.
template <int OP>
__global__ void __launch_bounds__(256) peak_f2op_kernel(float *out, int iters, float a, float b) {
    f2 x[kChains], y[kChains], z[kChains];
    f2 aa = f2_pack(a, a), bb = f2_pack(b, b);
#pragma unroll
    for (int c = 0; c < kChains; c++) {
        x[c] = f2_pack((float)threadIdx.x, (float)c);
        y[c] = f2_pack(a - 1e-6f * c, a + 1e-6f * c);
        z[c] = f2_pack(b * c, b + c);
    }
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 8; u++)
#pragma unroll
            for (int c = 0; c < kChains; c++) {
                if (OP == 3)
                    asm volatile("add.rn.ftz.f32x2 %0, %0, %1;" : "+l"(x[c]) : "l"(bb));
                else if (OP == 4)
                    asm volatile("mul.rn.ftz.f32x2 %0, %0, %1;" : "+l"(x[c]) : "l"(aa));
                else
                    asm volatile("fma.rn.ftz.f32x2 %0, %0, %1, %2;"
                                 : "+l"(x[c])
                                 : "l"(y[c]), "l"(z[(c + 3) % kChains]));
            }
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; c++) {
        float l, h;
        f2_unpack(x[c], l, h);
        s += l + h;
    }
    if (s == 1234.5f)
        out[threadIdx.x] = s;
}

// Instruction mixes (which = 6, 7): about the force kernel's ratio of packed
// FMAs to MUFU rsqrt (16 : 3 here, 6 : 1 there; FLOP/s of the FMAs), and
// packed plus scalar FMAs issued together (FLOP/s of both).
template <int MIX>
__global__ void __launch_bounds__(256) peak_mix_kernel(float *out, int iters, float a, float b) {
    f2 x[8], y[8];
    float r[8];
    const f2 aa = f2_pack(a, a), bb = f2_pack(b, b);
#pragma unroll
    for (int c = 0; c < 8; c++) {
        x[c] = f2_pack((float)threadIdx.x, (float)c);
        y[c] = f2_pack((float)c, (float)threadIdx.x);
        r[c] = 1.0f + (float)(threadIdx.x + c);
    }
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 8; u++) {
#pragma unroll
            for (int c = 0; c < 8; c++) {
                asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x[c]) : "l"(aa), "l"(bb));
                if (MIX == 6) {
                    if (c % 3 == 0)
                        asm volatile("rsqrt.approx.ftz.f32 %0, %0;" : "+f"(r[c]));
                } else {
                    asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(r[c]) : "f"(a), "f"(b));
                }
                asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(y[c]) : "l"(bb), "l"(aa));
            }
        }
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        float l, h, l2, h2;
        f2_unpack(x[c], l, h);
        f2_unpack(y[c], l2, h2);
        s += l + h + l2 + h2 + r[c];
    }
    if (s == 1234.5f)
        out[threadIdx.x] = s;
}

// The force kernel's pair interaction with sources in registers instead of
// shared memory (which = 8): 2 targets x 4 source pairs per iteration;
// reported as 20 FLOP per interaction, so it compares with the FP32 peak the
// way the force kernel's figure does.
//
// NLOG > 0: the first NLOG of the NS source pairs use the log-domain form
// (pair_interact2_log), the rest the rsqrt form (which = 11..16).
template <int NS, int NLOG>
__global__ void __launch_bounds__(256, 2) peak_interact_kernel(float *out, int iters, float a,
                                                              float b) {
    constexpr int KT = 2;
    f2 nx[KT], ny[KT], nz[KT], ax[KT], ay[KT], az[KT];
    f2 sx[NS], sy[NS], sz[NS], sm[NS];
    const f2 eps2 = f2_pack(1e-4f, 1e-4f), step = f2_pack(a * 1e-7f, b * 1e-7f);
#pragma unroll
    for (int k = 0; k < KT; k++) {
        const float t = (float)(threadIdx.x * KT + k) * 1e-3f;
        nx[k] = f2_pack(-t, -t);
        ny[k] = f2_pack(t, t);
        nz[k] = f2_pack(0.5f * t, 0.5f * t);
        ax[k] = ay[k] = az[k] = f2_pack(0.f, 0.f);
    }
#pragma unroll
    for (int c = 0; c < NS; c++) {
        sx[c] = f2_pack(0.1f * c, 0.1f * c + 0.05f);
        sy[c] = f2_pack(-0.1f * c, 0.2f);
        sz[c] = f2_pack(0.3f, 0.01f * c);
        sm[c] = c < NLOG ? f2_pack(-9.97f, -8.97f) : f2_pack(1e-3f, 2e-3f);
    }
    const f2 m15 = f2_pack(-1.5f, -1.5f);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < NS; c++) {
#pragma unroll
            for (int k = 0; k < KT; k++) {
                if (c < NLOG)
                    pair_interact2_log(sx[c], sy[c], sz[c], sm[c], nx[k], ny[k], nz[k], eps2,
                                       m15, ax[k], ay[k], az[k]);
                else
                    pair_interact2(sx[c], sy[c], sz[c], sm[c], nx[k], ny[k], nz[k], eps2,
                                   ax[k], ay[k], az[k]);
            }
            sx[c] = f2_add(sx[c], step);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < KT; k++) {
        float l, h;
        f2_unpack(f2_add(f2_add(ax[k], ay[k]), az[k]), l, h);
        s += l + h;
    }
    if (s == 1234.5f)
        out[threadIdx.x] = s;
}

// MUFU throughput: OP 0 = rsqrt (which = 2), 1 = ex2 (which = 9), 2 = lg2
// (which = 10), 16 dependent chains per thread.  The ex2 and lg2 chains add
// a constant after each step to stay at a stable fixed point (2^x - 1.5 at
// x = -1, log2 x + 2 at x = 4); the scalar adds run on the FMA pipe, which
// has 8x the MUFU rate, so the MUFU pipe stays the bound.
template <int OP>
__global__ void __launch_bounds__(256) peak_mufu_kernel(float *out, int iters) {
    float x[kChains], z[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) {
        x[c] = 1.0f + (float)(threadIdx.x + c);
        z[c] = OP == 1 ? -1.0f + 1e-3f * (float)(c + threadIdx.x % 7) : 4.0f + 1e-3f * (float)c;
    }
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 8; u++)
#pragma unroll
            for (int c = 0; c < kChains; c++) {
                if (OP == 0)
                    asm volatile("rsqrt.approx.ftz.f32 %0, %0;" : "+f"(x[c]));
                else if (OP == 1)
                    asm volatile("ex2.approx.ftz.f32 %0, %0;\n\tadd.ftz.f32 %0, %0, 0fBFC00000;"
                                 : "+f"(z[c]));
                else
                    asm volatile("lg2.approx.ftz.f32 %0, %0;\n\tadd.ftz.f32 %0, %0, 0f40000000;"
                                 : "+f"(z[c]));
            }
    }
    if (OP != 0) {
#pragma unroll
        for (int c = 0; c < kChains; c++)
            x[c] = z[c];
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; c++)
        s += x[c];
    if (s == 1234.5f)
        out[threadIdx.x] = s;
}

// FP64 pipe: 16 independent DFMA chains per thread.
__global__ void __launch_bounds__(256) peak_dfma_kernel(float *out, int iters, double a, double b) {
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++)
        x[c] = (double)(threadIdx.x + c);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int u = 0; u < 8; u++)
#pragma unroll
            for (int c = 0; c < kChains; c++)
                asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(x[c]) : "d"(a), "d"(b));
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; c++)
        s += x[c];
    if (s == 1234.5)
        out[threadIdx.x] = (float)s;
}

// Streaming copy (float4 per thread) and the read-only kernel that evicts L2
// between timed copies.
__global__ void __launch_bounds__(256) copy_f4_kernel(const float4 *__restrict__ a,
                                                       float4 *__restrict__ b, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n)
        b[i] = a[i];
}

__global__ void __launch_bounds__(256) read_evict_kernel(const int4 *__restrict__ p, size_t n,
                                                         int *sink) {
    int4 acc = make_int4(0, 0, 0, 0);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int4 v = p[i];
        acc.x ^= v.x;
        acc.y ^= v.y;
        acc.z ^= v.z;
        acc.w ^= v.w;
    }
    if ((acc.x ^ acc.y ^ acc.z ^ acc.w) == 0x7fffffff)
        *sink = 1;
}

}  // namespace nbgb

extern "C" {

// HBM copy rate of one kernel moving `bytes` (half read, half written) with
// L2 evicted before each launch (a 256 MiB read): the median of `reps`
// launches, as bytes / CUDA-event time.  Shows the fixed cost of a short
// streaming kernel on this GPU.  Allocates its buffers; synchronous.
NBGB_API int nbgb_measure_copy(size_t bytes, int reps, double *gb_per_s, float *ms_out) {
    if (bytes < 32 || reps <= 0 || reps > 1000 || !gb_per_s)
        return NBGB_ERR_INVALID_ARGUMENT;
    const size_t n = bytes / 32;  // float4 elements copied
    const size_t flush_bytes = (size_t)256 << 20;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return NBGB_ERR_CUDA;
    float4 *a = nullptr, *b = nullptr;
    int4 *fl = nullptr;
    int *sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = NBGB_ERR_CUDA;
    float *t = new (std::nothrow) float[reps];
    if (!t)
        return NBGB_ERR_NO_MEMORY;
    if (cudaMalloc(&a, n * 16) != cudaSuccess || cudaMalloc(&b, n * 16) != cudaSuccess ||
        cudaMalloc(&fl, flush_bytes) != cudaSuccess || cudaMalloc(&sink, 4) != cudaSuccess ||
        cudaMemset(a, 0, n * 16) != cudaSuccess || cudaMemset(fl, 0, flush_bytes) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        goto done;
    for (int r = -1; r < reps; r++) {  // r = -1: warm-up
        nbgb::read_evict_kernel<<<sms * 8, 256>>>(fl, flush_bytes / 16, sink);
        cudaEventRecord(e0, nullptr);
        nbgb::copy_f4_kernel<<<(unsigned)((n + 255) / 256), 256>>>(a, b, n);
        cudaEventRecord(e1, nullptr);
        if (cudaEventSynchronize(e1) != cudaSuccess)
            goto done;
        if (r >= 0 && cudaEventElapsedTime(&t[r], e0, e1) != cudaSuccess)
            goto done;
    }
    for (int i = 1; i < reps; i++)  // insertion sort for the median
        for (int j = i; j > 0 && t[j] < t[j - 1]; j--) {
            const float x = t[j];
            t[j] = t[j - 1];
            t[j - 1] = x;
        }
    *gb_per_s = (double)n * 32 / (t[reps / 2] * 1e-3) / 1e9;
    if (ms_out)
        *ms_out = t[reps / 2];
    rc = NBGB_OK;
done:
    delete[] t;
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    cudaFree(a);
    cudaFree(b);
    cudaFree(fl);
    cudaFree(sink);
    return rc;
}

// which: 0 = FFMA (FLOP/s), 1 = FFMA2 (FLOP/s), 2 = MUFU rsqrt (ops/s),
//        3 = add.f32x2, 4 = mul.f32x2 (FLOP/s, 2 per instruction), 5 = FFMA2
//        with three varying operands (FLOP/s), 6 = FFMA2 with one MUFU rsqrt
//        per six (FLOP/s of the FFMA2s), 7 = FFMA2 and scalar FFMA
//        interleaved (FLOP/s of both), 8 = the force kernel's pair
//        interaction on register-resident sources (20 FLOP/interaction),
//        9 = MUFU ex2, 10 = MUFU lg2 (ops/s), 11 / 12 = the pair
//        interaction with 1 / 2 of every 4 source pairs in the log-domain
//        form, 13 = 8 source pairs per step, 14..16 = 1..3 of every 8 in the
//        log-domain form, 17 = DFMA (FP64 FLOP/s).
// Result in *rate; *ms = best launch time.  Synchronous.
NBGB_API int nbgb_measure_peak(int which, int iters, int reps, double *rate, float *ms_out) {
    if (which < 0 || which > 17 || iters <= 0 || reps <= 0 || !rate)
        return NBGB_ERR_INVALID_ARGUMENT;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return NBGB_ERR_CUDA;
    float *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = NBGB_ERR_CUDA;
    const dim3 grid(sms * 8), block(256);
    float best = 1e30f;
    if (cudaMalloc(&out, 256 * sizeof(float)) != cudaSuccess)
        return NBGB_ERR_CUDA;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        goto done;
    for (int r = -1; r < reps; r++) {  // r = -1: warm-up
        cudaEventRecord(e0, nullptr);
        if (which == 0)
            nbgb::peak_ffma_kernel<<<grid, block>>>(out, iters, 0.999f, 1e-3f);
        else if (which == 1)
            nbgb::peak_ffma2_kernel<<<grid, block>>>(out, iters, 0.999f, 1e-3f);
        else if (which == 2)
            nbgb::peak_mufu_kernel<0><<<grid, block>>>(out, iters);
        else if (which == 9)
            nbgb::peak_mufu_kernel<1><<<grid, block>>>(out, iters);
        else if (which == 10)
            nbgb::peak_mufu_kernel<2><<<grid, block>>>(out, iters);
        else if (which == 3)
            nbgb::peak_f2op_kernel<3><<<grid, block>>>(out, iters, 0.999f, 1e-3f);
        else if (which == 4)
            nbgb::peak_f2op_kernel<4><<<grid, block>>>(out, iters, 0.999f, 1e-3f);
        else if (which == 5)
            nbgb::peak_f2op_kernel<5><<<grid, block>>>(out, iters, 0.999f, 1e-3f);
        else if (which == 6)
            nbgb::peak_mix_kernel<6><<<grid, block>>>(out, iters, 0.999f, 1e-3f);
        else if (which == 7)
            nbgb::peak_mix_kernel<7><<<grid, block>>>(out, iters, 0.999f, 1e-3f);
        else if (which == 8)
            nbgb::peak_interact_kernel<4, 0><<<dim3(sms * 2), block>>>(out, iters / 8, 0.999f, 1e-3f);
        else if (which == 11)
            nbgb::peak_interact_kernel<4, 1><<<dim3(sms * 2), block>>>(out, iters / 8, 0.999f, 1e-3f);
        else if (which == 12)
            nbgb::peak_interact_kernel<4, 2><<<dim3(sms * 2), block>>>(out, iters / 8, 0.999f, 1e-3f);
        else if (which == 13)
            nbgb::peak_interact_kernel<8, 0><<<dim3(sms * 2), block>>>(out, iters / 16, 0.999f, 1e-3f);
        else if (which == 14)
            nbgb::peak_interact_kernel<8, 1><<<dim3(sms * 2), block>>>(out, iters / 16, 0.999f, 1e-3f);
        else if (which == 15)
            nbgb::peak_interact_kernel<8, 2><<<dim3(sms * 2), block>>>(out, iters / 16, 0.999f, 1e-3f);
        else if (which == 16)
            nbgb::peak_interact_kernel<8, 3><<<dim3(sms * 2), block>>>(out, iters / 16, 0.999f, 1e-3f);
        else
            nbgb::peak_dfma_kernel<<<grid, block>>>(out, iters, 0.999, 1e-3);
        cudaEventRecord(e1, nullptr);
        if (cudaEventSynchronize(e1) != cudaSuccess)
            goto done;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r >= 0 && ms < best)
            best = ms;
    }
    {
        const double threads = (double)grid.x * block.x;
        const double per_thread = (double)iters * 8 * nbgb::kChains;
        double ops = threads * per_thread;
        if (which == 0 || which == 17)
            ops *= 2.0;  // FMA = 2 FLOP
        else if (which == 1 || which == 5)
            ops *= 4.0;  // two FMAs per instruction
        else if (which == 3 || which == 4)
            ops *= 2.0;  // two adds / multiplies per instruction
        else if (which == 6)
            ops = threads * (double)iters * 8 * 8 * 2 * 4;  // FMAs of the FFMA2s only
        else if (which == 7)
            ops = threads * (double)iters * 8 * 8 * (2 * 4 + 2);  // FFMA2s + FFMAs
        else if (which == 8 || which == 11 || which == 12)  // 20 FLOP x interactions:
            ops = (double)sms * 2 * block.x * (double)(iters / 8) * 4 * 2 * 2 * 20;  // NS*KT*2/it
        else if (which >= 13)
            ops = (double)sms * 2 * block.x * (double)(iters / 16) * 8 * 2 * 2 * 20;
        *rate = ops / (best * 1e-3);
        if (ms_out)
            *ms_out = best;
        rc = NBGB_OK;
    }
done:
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    cudaFree(out);
    return rc;
}

}  // extern "C"
