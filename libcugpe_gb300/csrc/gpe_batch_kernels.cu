// Instantiation of the batched pass kernels (FP32-mixed form) and their
// launch dispatch over (axis, kernel class, radix plan).
#include "gpe_batch.cuh"
#include "gpe_device_state.h"

namespace gpe {

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
static cudaError_t launch_bc(int cls, const BatchItem<R>* items, int nitems, unsigned grid, size_t smem,
                             cudaStream_t st) {
    switch (cls) {
        case C_KIN: return launch_b<R, AX, C_KIN, P>(items, nitems, grid, smem, st);
        case C_EPI: return launch_b<R, AX, C_EPI, P>(items, nitems, grid, smem, st);
        case C_LAP: return launch_b<R, AX, C_LAP, P>(items, nitems, grid, smem, st);
        default: return launch_b<R, AX, C_EN, P>(items, nitems, grid, smem, st);
    }
}

template <typename R, int P>
static cudaError_t launch_bp(int axis, int cls, const BatchItem<R>* items, int nitems, unsigned grid, size_t smem,
                             cudaStream_t st) {
    switch (axis) {
        case AX_X: return launch_bc<R, AX_X, P>(cls, items, nitems, grid, smem, st);
        case AX_Y: return launch_bc<R, AX_Y, P>(cls, items, nitems, grid, smem, st);
        default: return launch_bc<R, AX_Z, P>(cls, items, nitems, grid, smem, st);
    }
}

template <>
cudaError_t launch_batch<float>(int axis, int cls, int plan, const BatchItem<float>* items, int nitems,
                                unsigned grid, size_t smem, cudaStream_t st) {
    if (plan == 1) return launch_bp<float, 1>(axis, cls, items, nitems, grid, smem, st);
    if (plan != 0) return cudaErrorInvalidValue;
    return launch_bp<float, 0>(axis, cls, items, nitems, grid, smem, st);
}

}  // namespace gpe
