// Launch of the yz-plane pass (gpe_plane.cuh).
#include "gpe_device_state.h"
#include "gpe_plane.cuh"

namespace gpe {

template <int N>
static cudaError_t launch_plane_n(const PlaneArgs& pa, unsigned planes, cudaStream_t st) {
    using Geo = PlaneGeom<N>;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    static DeviceOnce configured;
    const int rc = configured.ensure(dev, [] {
        cudaError_t e2 = cudaFuncSetAttribute(plane_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)Geo::SMEM);
        if (e2 == cudaSuccess)
            e2 = cudaFuncSetAttribute(plane_kernel<N>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                      (int)cudaSharedmemCarveoutMaxShared);
        return (int)e2;
    }, (int)cudaErrorInvalidDevice);
    if (rc) return (cudaError_t)rc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(planes);
    cfg.blockDim = dim3(Geo::NT);
    cfg.dynamicSmemBytes = Geo::SMEM;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, plane_kernel<N>, pa);
}

// The plane pass over `planes` x-planes of n_y = n_z = n points; refuses what it does not support.
cudaError_t launch_plane(const PlaneArgs& pa, int n, unsigned planes, cudaStream_t st) {
    if (!plane_supports(pa.a.pre, pa.a.mid, pa.a.post, pa.a.flags & ~F_DIRECT)) return cudaErrorInvalidValue;
    if (pa.a.plan != 0) return cudaErrorInvalidValue;
    switch (n) {
        case 128: return launch_plane_n<128>(pa, planes, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace gpe
