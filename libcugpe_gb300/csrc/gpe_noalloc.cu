// Allocation-free norm of a caller-owned wavefunction.
//
// Some callers of this library cannot allocate device memory at the moment
// they need a result: code that runs while its stream is being captured into
// a CUDA graph (cudaMalloc/cudaFree are not stream operations and are not
// allowed in every capture mode), applications that hand all device memory
// to their own pool allocator at start-up, and plugins hosted by a process
// that forbids allocations after initialisation.  gpe_gb_norm_noalloc serves
// them: it computes sum Gamma |psi|^2 (the quantity of gpe_get_norm) of a
// wavefunction the caller already holds in device memory, into a device
// double the caller also provides, and allocates nothing.
//
// Its scratch (per-CTA partial sums and the last-CTA ticket) is a file-scope
// __device__ array of fixed size, held by every GPU that loads the library
// until the process exits.  Host code cannot use the array's name as a
// device address; the first call on each device looks the address up with
// cudaGetSymbolAddress while that device is current and keeps it, so that
// first call belongs before any stream capture.  The kept address is valid
// for the life of the device's primary context: after cudaDeviceReset the
// module is loaded again and the array may move, so a process that resets a
// device must not call this entry point on that device again.
#include <cuda_runtime.h>
#include <math.h>

#include "../../include/gpe_gb300.h"
#include "gpe_device_state.h"

namespace {

constexpr int kNaBlocks = 512;
constexpr int kNaThreads = 256;
constexpr long long kNaMaxPoints = 1LL << 27;  // 512^3, the engine's largest lattice

struct NaScratch {
    double partials[kNaBlocks];
    unsigned int ticket;
    unsigned int pad[63];
};

// 4 KiB of partial sums + 256 B for the ticket
static __device__ __align__(256) NaScratch g_na_scratch;

// device address of g_na_scratch per device ordinal (host threads may race to fill an entry: they
// store the same value)
static gpe::DeviceValue<NaScratch*> g_na_addr;

template <typename C>
__global__ void __launch_bounds__(kNaThreads) k_norm_noalloc(const C* __restrict__ psi, long long n, double gamma,
                                                             double* out, NaScratch* s) {
    __shared__ double sw[kNaThreads / 32];
    __shared__ bool last;
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double x = psi[i].x, y = psi[i].y;
        acc += gamma * (x * x + y * y);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < kNaThreads / 32; w++) b += sw[w];
        s->partials[blockIdx.x] = b;
        __threadfence();
        last = (atomicAdd(&s->ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double sum = 0.0, c = 0.0;  // Neumaier, fixed order
        for (unsigned b = 0; b < gridDim.x; b++) {
            const double x = __ldcg(s->partials + b);
            const double t = sum + x;
            c += (fabs(sum) >= fabs(x)) ? (sum - t) + x : (x - t) + sum;
            sum = t;
        }
        *out = sum + c;
        s->ticket = 0;
    }
}

// Device address of the scratch for the current device, looked up once.
int scratch_for_current_device(NaScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    return g_na_addr.ensure(dev, out, [](NaScratch** p) {
        void* a = nullptr;
        const cudaError_t e2 = cudaGetSymbolAddress(&a, g_na_scratch);
        if (e2 != cudaSuccess) return (int)e2;
        *p = static_cast<NaScratch*>(a);
        return 0;
    }, GPE_ERR_ARGUMENT);
}

}  // namespace

extern "C" int gpe_gb_norm_noalloc(const void* psi, int precision, long long n, double gamma, double* norm_out,
                                   void* stream) {
    if (!psi || !norm_out) return GPE_ERR_ARGUMENT;
    if (precision != GPE_PRECISION_FP64 && precision != GPE_PRECISION_FP32) return GPE_ERR_ARGUMENT;
    if (n <= 0 || n > kNaMaxPoints) return GPE_ERR_NOALLOC_SIZE;
    NaScratch* s = nullptr;
    int rc = scratch_for_current_device(&s);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the ticket must start at zero; the partial sums are all rewritten
    cudaError_t e = cudaMemsetAsync(&s->ticket, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return (int)e;
    if (precision == GPE_PRECISION_FP64)
        k_norm_noalloc<double2><<<kNaBlocks, kNaThreads, 0, st>>>(static_cast<const double2*>(psi), n, gamma, norm_out, s);
    else
        k_norm_noalloc<float2><<<kNaBlocks, kNaThreads, 0, st>>>(static_cast<const float2*>(psi), n, gamma, norm_out, s);
    e = cudaGetLastError();
    return e == cudaSuccess ? 0 : (int)e;
}
