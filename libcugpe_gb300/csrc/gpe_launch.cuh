// Launch dispatch for the fused pencil pass: maps a run-time pencil length
// and axis to the compiled kernel, picks the CTA shape and the dynamic
// shared memory.  The kernels are instantiated in one generated translation
// unit per (precision, pencil length) so they compile in parallel.
#pragma once
#include <cuda_runtime.h>
#include "gpe_device_state.h"
#include "gpe_pass.cuh"

namespace gpe {

// Threads per CTA: 128, or one pencil group of the wanted column width when
// a group is larger (x and y pencils of 256 and 512 points in the FP32 form).
// A lattice with fewer pencils than a CTA holds runs a partial last CTA.
template <typename R, int N, int AX, int P = 0> constexpr int pass_nt() {
    if constexpr (AX == AX_Z) {
        return 128;
    } else {
        constexpr int T = N / Plan<N, P>::E;
        constexpr int want = ((32 / T) > cw_target<R, N, AX>()) ? (32 / T) : cw_target<R, N, AX>();
        return (T * want > 128) ? T * want : 128;
    }
}

template <typename R, int N, int AX, int NT, int CLS, int P>
cudaError_t launch_one(const PassArgs<R>& a, size_t pencils, cudaStream_t st) {
    using Geo = PassGeom<R, N, AX, NT, P>;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    // kernel attributes belong to the device context: set them once per device
    static DeviceOnce configured;
    int rc = configured.ensure(dev, [] {
        cudaError_t e2 = cudaFuncSetAttribute(pass_kernel<R, N, AX, NT, CLS, P>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Geo::SMEM_MAX);
        // the passes use shared memory, not L1, for reuse: ask for the largest carveout
        if (e2 == cudaSuccess)
            e2 = cudaFuncSetAttribute(pass_kernel<R, N, AX, NT, CLS, P>,
                                      cudaFuncAttributePreferredSharedMemoryCarveout,
                                      (int)cudaSharedmemCarveoutMaxShared);
        return (int)e2;
    }, (int)cudaErrorInvalidDevice);
    if (rc) return (cudaError_t)rc;
    unsigned grid = (unsigned)((pencils + Geo::W - 1) / Geo::W);
    size_t smem = Geo::SMEM_BASE + slot_bytes<R>(staged_ops(a.mid, a.post, a.flags), Geo::E * NT);
    if constexpr (CLS == C_KINP) {
        // persistent: one staging buffer per CTA, as many CTAs as fit on the device at once
        smem = Geo::SMEM_BASE + (size_t)Geo::E * NT * sizeof(C2<R>);
        static DeviceValue<unsigned> resident_ctas;
        unsigned resident = 0;
        rc = resident_ctas.ensure(dev, &resident, [dev, smem](unsigned* out) {
            int per_sm = 0, sms = 0;
            cudaError_t e2 = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e2 == cudaSuccess)
                e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pass_kernel<R, N, AX, NT, CLS, P>, NT,
                                                                   smem);
            if (e2 != cudaSuccess) return (int)e2;
            *out = (unsigned)((per_sm > 0 ? per_sm : 1) * sms);
            return 0;
        }, (int)cudaErrorInvalidDevice);
        if (rc) return (cudaError_t)rc;
        if (grid > resident) grid = resident;
    }
    if (smem > Geo::SMEM_MAX) return cudaErrorInvalidConfiguration;  // more staged operands than a CTA holds
    PassArgs<R> b = a;
    b.npencils = (uint32_t)pencils;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    // programmatic dependent launch: +2% steps/s for the FP32 form (128^3-512^3); the FP64 passes
    // ran slower with it (64^3: 4230 against 4679 steps/s), so they launch in plain stream order
    cfg.numAttrs = (sizeof(R) == 4) ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, pass_kernel<R, N, AX, NT, CLS, P>, b);
}

template <typename R, int N, int AX, int P>
cudaError_t launch_ax(const PassArgs<R>& a, size_t pencils, cudaStream_t st, unsigned* grid_out) {
    constexpr int NT = pass_nt<R, N, AX, P>();
    *grid_out = (unsigned)((pencils + PassGeom<R, N, AX, NT, P>::W - 1) / PassGeom<R, N, AX, NT, P>::W);
    switch (op_class(a.pre, a.mid, a.post, a.flags)) {
        case C_KIN:
            // FP32 x pencils of 512 points: the persistent pass overlaps loads and transforms (measured
            // at 512^3 with 16 points per thread: 923 -> 809 us per pass; on y pencils, at either point
            // count, and at 256 points it was slower)
            if constexpr (sizeof(R) == 4 && N >= 512 && AX == AX_X && Plan<N, P>::E <= 16) {
                if ((a.flags & ~(F_VEXTRA | F_DIRECT)) == (F_KIN | F_STORE) && a.pre == PRE_NONE &&
                    a.mid == MID_NONE && a.post == POST_NONE)
                    return launch_one<R, N, AX, NT, C_KINP, P>(a, pencils, st);
            }
            return launch_one<R, N, AX, NT, C_KIN, P>(a, pencils, st);
        case C_EPI: return launch_one<R, N, AX, NT, C_EPI, P>(a, pencils, st);
        case C_LAP: return launch_one<R, N, AX, NT, C_LAP, P>(a, pencils, st);
        case C_DIP: return launch_one<R, N, AX, NT, C_DIP, P>(a, pencils, st);
        case C_EPI_D:
            if constexpr (sizeof(R) == 4 && N <= 128) return launch_one<R, N, AX, NT, C_EPI_D, P>(a, pencils, st);
            else return cudaErrorInvalidValue;
        case C_LAP_D:
            if constexpr (sizeof(R) == 4 && N <= 128) return launch_one<R, N, AX, NT, C_LAP_D, P>(a, pencils, st);
            else return cudaErrorInvalidValue;
        default: return launch_one<R, N, AX, NT, C_EN, P>(a, pencils, st);
    }
}

template <typename R, int N, int P>
cudaError_t launch_n(const PassArgs<R>& a, int axis, size_t pencils, cudaStream_t st, unsigned* g);

#ifdef GPE_PASS_DEFINITIONS
template <typename R, int N, int P>
cudaError_t launch_n(const PassArgs<R>& a, int axis, size_t pencils, cudaStream_t st, unsigned* g) {
    switch (axis) {
        case AX_X: return launch_ax<R, N, AX_X, P>(a, pencils, st, g);
        case AX_Y: return launch_ax<R, N, AX_Y, P>(a, pencils, st, g);
        default: return launch_ax<R, N, AX_Z, P>(a, pencils, st, g);
    }
}
#elif defined(GPE_PASS_STUBS)
// A library built for a subset of pencil lengths (a hook library for tests): the lengths left out
// refuse every pass over them.
template <typename R, int N, int P>
cudaError_t launch_n(const PassArgs<R>&, int, size_t, cudaStream_t, unsigned*) {
    return cudaErrorInvalidValue;
}
#endif

// Radix plan a pass over pencils of n points runs with when `plan` is requested: the alternative
// plans exist for FP32 pencils of 32 to 512 points; everything else runs plan 0.
inline int effective_plan(int plan, int n, bool fp32) { return (plan == 1 && fp32 && has_plan1(n)) ? 1 : 0; }

// Upper bound on the CTAs of a pass over `pencils` pencils (sizes the partials buffer).
inline size_t pass_grid_bound(size_t pencils) { return pencils; }

// Launches one pass with the radix plan `a.plan` (whose twiddles `a.tw` holds).
template <typename R>
cudaError_t launch_pass(const PassArgs<R>& a, int N, int axis, size_t pencils, cudaStream_t st) {
    unsigned g = 0;
    if (a.plan != effective_plan(a.plan, N, sizeof(R) == 4)) return cudaErrorInvalidValue;
    if constexpr (sizeof(R) == 4) {
        if (a.plan == 1) {
            switch (N) {
                case 32: return launch_n<R, 32, 1>(a, axis, pencils, st, &g);
                case 64: return launch_n<R, 64, 1>(a, axis, pencils, st, &g);
                case 128: return launch_n<R, 128, 1>(a, axis, pencils, st, &g);
                case 256: return launch_n<R, 256, 1>(a, axis, pencils, st, &g);
                case 512: return launch_n<R, 512, 1>(a, axis, pencils, st, &g);
                default: return cudaErrorInvalidValue;
            }
        }
    }
    switch (N) {
        case 8: return launch_n<R, 8, 0>(a, axis, pencils, st, &g);
        case 16: return launch_n<R, 16, 0>(a, axis, pencils, st, &g);
        case 32: return launch_n<R, 32, 0>(a, axis, pencils, st, &g);
        case 64: return launch_n<R, 64, 0>(a, axis, pencils, st, &g);
        case 128: return launch_n<R, 128, 0>(a, axis, pencils, st, &g);
        case 256: return launch_n<R, 256, 0>(a, axis, pencils, st, &g);
        case 512: return launch_n<R, 512, 0>(a, axis, pencils, st, &g);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace gpe

// One translation unit per (precision, pencil length, radix plan) instantiates
// launch_n<R, N, P>; launch_pass<R> switches over them.
#define GPE_INSTANTIATE_N(R, N, P) \
    template cudaError_t gpe::launch_n<R, N, P>(const gpe::PassArgs<R>&, int, size_t, cudaStream_t, unsigned*);
