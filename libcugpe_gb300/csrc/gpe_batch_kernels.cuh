// Batched pass kernels (FP32-mixed form): launch per (axis, kernel class,
// radix plan).  One generated translation unit per (axis, plan) defines
// GPE_BATCH_DEFINITIONS and instantiates launch_bc for it, so they compile in
// parallel; the dispatch over axis and plan (launch_batch) is in
// gpe_batch_dispatch.cu.  A library built without the batched solver defines
// GPE_BATCH_STUBS instead: every batched pass is then refused.
#pragma once
#include "gpe_batch.cuh"
#include "gpe_device_state.h"

namespace gpe {

template <typename R, int AX, int P>
cudaError_t launch_bc(int cls, const BatchItem<R>* items, int nitems, unsigned grid, size_t smem, cudaStream_t st);

#ifdef GPE_BATCH_DEFINITIONS

template <typename R, int AX, int CLS, int P>
static cudaError_t launch_b(const BatchItem<R>* items, int nitems, unsigned grid, size_t smem, cudaStream_t st) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    // kernel attributes belong to the device context: set them once per device
    static DeviceOnce configured;
    const int rc = configured.ensure(dev, [] {
        size_t mx = PassGeom<R, 32, AX, kBatchThreads, P>::SMEM_MAX;
        if (PassGeom<R, 64, AX, kBatchThreads, P>::SMEM_MAX > mx) mx = PassGeom<R, 64, AX, kBatchThreads, P>::SMEM_MAX;
        if (PassGeom<R, 128, AX, kBatchThreads, P>::SMEM_MAX > mx)
            mx = PassGeom<R, 128, AX, kBatchThreads, P>::SMEM_MAX;
        if (PassGeom<R, 256, AX, kBatchThreads, P>::SMEM_MAX > mx)
            mx = PassGeom<R, 256, AX, kBatchThreads, P>::SMEM_MAX;
        cudaError_t e2 = cudaFuncSetAttribute(pass_batch_kernel<R, AX, CLS, P>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mx);
        if (e2 == cudaSuccess)
            e2 = cudaFuncSetAttribute(pass_batch_kernel<R, AX, CLS, P>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                      (int)cudaSharedmemCarveoutMaxShared);
        return (int)e2;
    }, (int)cudaErrorInvalidDevice);
    if (rc) return (cudaError_t)rc;
    pass_batch_kernel<R, AX, CLS, P><<<grid, kBatchThreads, smem, st>>>(items, nitems);
    return cudaGetLastError();
}

template <typename R, int AX, int P>
cudaError_t launch_bc(int cls, const BatchItem<R>* items, int nitems, unsigned grid, size_t smem,
                      cudaStream_t st) {
    switch (cls) {
        case C_KIN: return launch_b<R, AX, C_KIN, P>(items, nitems, grid, smem, st);
        case C_EPI: return launch_b<R, AX, C_EPI, P>(items, nitems, grid, smem, st);
        case C_LAP: return launch_b<R, AX, C_LAP, P>(items, nitems, grid, smem, st);
        default: return launch_b<R, AX, C_EN, P>(items, nitems, grid, smem, st);
    }
}
#elif defined(GPE_BATCH_STUBS)
template <typename R, int AX, int P>
cudaError_t launch_bc(int, const BatchItem<R>*, int, unsigned, size_t, cudaStream_t) {
    return cudaErrorInvalidValue;
}
#endif

}  // namespace gpe

#define GPE_INSTANTIATE_BATCH(AX, P)                                                                          \
    template cudaError_t gpe::launch_bc<float, AX, P>(int, const gpe::BatchItem<float>*, int, unsigned, size_t, \
                                                      cudaStream_t);
