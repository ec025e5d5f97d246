/*
 * refgpu_launch.c -- launches the reference's own GPU force kernels
 * (TEST INFRASTRUCTURE ONLY: the same-box comparison of tests/).
 *
 * oracle/Makefile (target refgpu) compiles the reference's
 * src/nbody_GPU_AOS.cu, src/nbody_GPU_Shared.cu and src/nbody_GPU_Shuffle.cu
 * from the reference sources, unchanged, into sm_103a cubins under
 * oracle/_ref/ with the reference's nvcc flags (-O3 --ftz true,
 * meson.build:82-93).  This file loads such a cubin with the CUDA driver API
 * in the calling process's primary context and launches the kernel exactly
 * as the reference's host wrappers do: <<<300, 256, shared>>> with
 * (float *force, float *posMass, float softeningSquared, size_t N)
 * (src/nbody_GPU_AOS.cu:85, src/nbody_GPU_Shared.cu:91,
 * src/nbody_GPU_Shuffle.cu:99), timing `reps` launches with driver events.
 */
#include <cuda.h>
#include <stddef.h>

#define REF_EXPORT __attribute__((visibility("default")))

/* Returns the mean milliseconds per launch, or a negative CUresult.
   n_before_eps: the kernel takes (force, posMass, N, eps2) instead of
   (force, posMass, eps2, N) (src/nbody_GPU_AOS.cu:44-48). */
REF_EXPORT double refgpu_time(const char *cubin, const char *kernel, unsigned grid,
                              unsigned block, unsigned shmem, unsigned long long force_dev,
                              unsigned long long posmass_dev, float eps2, size_t n,
                              int n_before_eps, int reps)
{
    CUdevice dev;
    CUcontext ctx;
    CUmodule mod;
    CUfunction fn;
    CUevent e0, e1;
    CUresult r;
    float ms = 0.0f;
    if ((r = cuInit(0)) != CUDA_SUCCESS)
        return -(double)r;
    if ((r = cuDeviceGet(&dev, 0)) != CUDA_SUCCESS)
        return -(double)r;
    if ((r = cuDevicePrimaryCtxRetain(&ctx, dev)) != CUDA_SUCCESS)
        return -(double)r;
    if ((r = cuCtxPushCurrent(ctx)) != CUDA_SUCCESS)
        return -(double)r;
    if ((r = cuModuleLoad(&mod, cubin)) != CUDA_SUCCESS)
        goto pop;
    if ((r = cuModuleGetFunction(&fn, mod, kernel)) != CUDA_SUCCESS)
        goto unload;
    {
        CUdeviceptr f = (CUdeviceptr)force_dev, p = (CUdeviceptr)posmass_dev;
        void *args_a[] = {&f, &p, &eps2, &n};
        void *args_b[] = {&f, &p, &n, &eps2};
        void **args = n_before_eps ? args_b : args_a;
        if ((r = cuEventCreate(&e0, CU_EVENT_DEFAULT)) != CUDA_SUCCESS)
            goto unload;
        if ((r = cuEventCreate(&e1, CU_EVENT_DEFAULT)) != CUDA_SUCCESS)
            goto ev0;
        /* one warm-up launch */
        if ((r = cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, shmem, 0, args, 0)) != CUDA_SUCCESS)
            goto ev1;
        if ((r = cuEventRecord(e0, 0)) != CUDA_SUCCESS)
            goto ev1;
        for (int k = 0; k < reps; k++)
            if ((r = cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, shmem, 0, args, 0)) !=
                CUDA_SUCCESS)
                goto ev1;
        if ((r = cuEventRecord(e1, 0)) != CUDA_SUCCESS)
            goto ev1;
        if ((r = cuEventSynchronize(e1)) != CUDA_SUCCESS)
            goto ev1;
        r = cuEventElapsedTime(&ms, e0, e1);
    ev1:
        cuEventDestroy(e1);
    ev0:
        cuEventDestroy(e0);
    }
unload:
    cuModuleUnload(mod);
pop:
    cuCtxPopCurrent(&ctx);
    cuDevicePrimaryCtxRelease(dev);
    if (r != CUDA_SUCCESS)
        return -(double)r;
    return (double)ms / (double)reps;
}
