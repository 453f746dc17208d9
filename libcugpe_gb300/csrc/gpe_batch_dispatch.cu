// Dispatch of the batched passes over axis and radix plan (the launches
// themselves are instantiated per (axis, plan) from gpe_batch_kernels.cuh).
#include "gpe_batch_kernels.cuh"

namespace gpe {

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
