// Batched pass: one launch walks the pencils of one axis of every condensate
// in a batch, whatever its lattice size.  CTA b finds its condensate by a
// binary search over the items' first-CTA offsets and runs the pass body for
// that condensate's pencil length (32, 64, 128 or 256 points, all with
// 128-thread CTAs) under the batch's radix plan P.  Each condensate keeps its own tables, device state and
// reduction slots, so the last-CTA reductions stay per condensate.
#pragma once
#include <cuda_runtime.h>
#include "gpe_launch.cuh"

namespace gpe {

template <typename R>
struct BatchItem {
    PassArgs<R> a;       // the condensate's pass arguments (npencils set)
    uint32_t cta_begin;  // first CTA of this condensate in the launch
    uint32_t nctas;      // CTAs of this condensate
    int n;               // pencil length along the pass axis
    int pad;
};

constexpr int kBatchThreads = 128;
// 7 CTAs per SM: the register budget (72) that the 32- to 128-point bodies of either plan fit
constexpr int kBatchMinBlocks = 7;
constexpr int kBatchLengths[4] = {32, 64, 128, 256};

template <typename R, int AX, int CLS, int P>
__global__ void __launch_bounds__(kBatchThreads, kBatchMinBlocks)
pass_batch_kernel(const BatchItem<R>* __restrict__ items, int nitems) {
    int lo = 0, hi = nitems - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (items[mid].cta_begin <= blockIdx.x) lo = mid;
        else hi = mid - 1;
    }
    const BatchItem<R>& it = items[lo];
    const uint32_t blk = blockIdx.x - it.cta_begin;
    switch (it.n) {
        case 32: pass_body<R, 32, AX, kBatchThreads, CLS, P>(it.a, blk, it.nctas); break;
        case 64: pass_body<R, 64, AX, kBatchThreads, CLS, P>(it.a, blk, it.nctas); break;
        case 128: pass_body<R, 128, AX, kBatchThreads, CLS, P>(it.a, blk, it.nctas); break;
        default: pass_body<R, 256, AX, kBatchThreads, CLS, P>(it.a, blk, it.nctas); break;
    }
}

// CTAs and dynamic shared memory of one condensate's pass in a batch.
template <typename R, int AX, int P>
inline bool batch_shape(int n, size_t pencils, uint32_t ops, uint32_t* nctas, size_t* smem) {
    switch (n) {
#define GPE_BATCH_CASE(NN)                                                                      \
    case NN: {                                                                                  \
        using Geo = PassGeom<R, NN, AX, kBatchThreads, P>;                                      \
        *nctas = (uint32_t)((pencils + Geo::W - 1) / Geo::W);                                   \
        *smem = Geo::SMEM_BASE + slot_bytes<R>(ops, Geo::E * kBatchThreads);                    \
        return true;                                                                            \
    }
        GPE_BATCH_CASE(32)
        GPE_BATCH_CASE(64)
        GPE_BATCH_CASE(128)
        GPE_BATCH_CASE(256)
#undef GPE_BATCH_CASE
        default: return false;
    }
}

template <typename R>
cudaError_t launch_batch(int axis, int cls, int plan, const BatchItem<R>* items, int nitems, unsigned grid,
                         size_t smem, cudaStream_t st);

}  // namespace gpe
