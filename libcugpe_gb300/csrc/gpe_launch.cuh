// Launch dispatch for the fused pencil pass: maps a run-time pencil length
// and axis to the compiled kernel, picks pencils per CTA and the dynamic
// shared memory.  The kernels are instantiated in one generated translation
// unit per (precision, pencil length) so they compile in parallel.
#pragma once
#include <cuda_runtime.h>
#include "gpe_pass.cuh"

namespace gpe {

// Threads per CTA for the fused pass.
constexpr int kPassThreads = 128;

template <int N> constexpr int wide_w() { return kPassThreads / (N / Plan<N>::E); }
template <int N> constexpr int narrow_w() {
    return (32 / (N / Plan<N>::E)) > 0 ? (32 / (N / Plan<N>::E)) : 1;
}

template <typename R, int N, int AX, int W>
size_t pass_smem() {
    return (AX == AX_Z) ? (size_t)W * (N + 1) * sizeof(C2<R>) : (size_t)W * N * sizeof(C2<R>);
}

template <typename R, int N, int AX, int W>
cudaError_t launch_one(const PassArgs<R>& a, size_t pencils, cudaStream_t st) {
    const size_t smem = pass_smem<R, N, AX, W>();
    static bool configured = false;  // per instantiation; attribute is per-device-context
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(pass_kernel<R, N, AX, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    const unsigned grid = (unsigned)(pencils / W);
    pass_kernel<R, N, AX, W><<<grid, W * (N / Plan<N>::E), smem, st>>>(a);
    return cudaGetLastError();
}

template <typename R, int N, int AX>
cudaError_t launch_ax(const PassArgs<R>& a, size_t pencils, cudaStream_t st, unsigned* grid_out) {
    constexpr int WW = wide_w<N>(), WN = narrow_w<N>();
    if (pencils % WW == 0) { *grid_out = (unsigned)(pencils / WW); return launch_one<R, N, AX, WW>(a, pencils, st); }
    if (pencils % WN == 0) { *grid_out = (unsigned)(pencils / WN); return launch_one<R, N, AX, WN>(a, pencils, st); }
    return cudaErrorInvalidValue;
}

template <typename R, int N>
cudaError_t launch_n(const PassArgs<R>& a, int axis, size_t pencils, cudaStream_t st, unsigned* g);

#ifdef GPE_PASS_DEFINITIONS
template <typename R, int N>
cudaError_t launch_n(const PassArgs<R>& a, int axis, size_t pencils, cudaStream_t st, unsigned* g) {
    switch (axis) {
        case AX_X: return launch_ax<R, N, AX_X>(a, pencils, st, g);
        case AX_Y: return launch_ax<R, N, AX_Y>(a, pencils, st, g);
        default: return launch_ax<R, N, AX_Z>(a, pencils, st, g);
    }
}
#endif

// Number of CTAs a pass over `pencils` pencils of length N would use.
inline unsigned pass_grid(int N, size_t pencils) {
    int T = 1;
    switch (N) {
        case 8: T = 8 / Plan<8>::E; break;
        case 16: T = 16 / Plan<16>::E; break;
        case 32: T = 32 / Plan<32>::E; break;
        case 64: T = 64 / Plan<64>::E; break;
        case 128: T = 128 / Plan<128>::E; break;
        case 256: T = 256 / Plan<256>::E; break;
        default: T = 512 / Plan<512>::E; break;
    }
    const int ww = kPassThreads / T, wn = (32 / T) > 0 ? 32 / T : 1;
    if (pencils % ww == 0) return (unsigned)(pencils / ww);
    return (unsigned)(pencils / wn);
}

template <typename R>
cudaError_t launch_pass(const PassArgs<R>& a, int N, int axis, size_t pencils, cudaStream_t st) {
    unsigned g = 0;
    switch (N) {
        case 8: return launch_n<R, 8>(a, axis, pencils, st, &g);
        case 16: return launch_n<R, 16>(a, axis, pencils, st, &g);
        case 32: return launch_n<R, 32>(a, axis, pencils, st, &g);
        case 64: return launch_n<R, 64>(a, axis, pencils, st, &g);
        case 128: return launch_n<R, 128>(a, axis, pencils, st, &g);
        case 256: return launch_n<R, 256>(a, axis, pencils, st, &g);
        case 512: return launch_n<R, 512>(a, axis, pencils, st, &g);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace gpe

// One translation unit per (precision, pencil length) instantiates
// launch_n<R, N>; launch_pass<R> (gpe_engine.cu) switches over them.
#define GPE_INSTANTIATE_N(R, N) \
    template cudaError_t gpe::launch_n<R, N>(const gpe::PassArgs<R>&, int, size_t, cudaStream_t, unsigned*);
