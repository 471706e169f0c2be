// k_noalloc.cu -- deterministic FP64 reduction of a caller-owned device array
// that allocates nothing.
//
// Some callers cannot allocate device memory at the moment they need a
// reduction -- for example a host application that hands all device memory
// to its own pool at start-up and forbids cudaMalloc afterwards, or code
// that runs under a fixed device-memory budget.  amps_reduce needs a
// handle, and a handle allocates.  This entry point keeps its per-block
// partial results in a fixed file-scope device array instead; the caller
// passes only the input array and the output slot.
//
// Limits and sharing:
//  * The array holds AMPS_REDUCE_NOALLOC_MAX_BLOCKS partials of
//    AMPS_REDUCE_NOALLOC_CELLS_PER_BLOCK cells each, so n is limited to
//    AMPS_REDUCE_NOALLOC_MAX_CELLS; larger n is rejected with
//    AMPS_ERR_UNSUPPORTED before any device work is queued.
//  * The array is one per device and lives until the process exits.  Every
//    call shares it and overwrites the slots it uses before reading them (the
//    last call's contents stay behind; nothing needs to start at zero).
//  * Calls whose kernels overlap on the GPU (on different streams, or from
//    different threads without ordering) race on the array and give wrong
//    results: order them on one stream.
//  * The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress, with that device current; make that first call
//    before any stream capture on the device.
#include "../../include/amps.h"

#include <cuda_runtime.h>
#include <math.h>

#include <mutex>

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[AMPS_REDUCE_NOALLOC_MAX_BLOCKS];

double *g_partials_addr[kNoAllocMaxDevices] = {nullptr};
std::mutex g_setup_mutex;

__device__ __forceinline__ double fold(double acc, double v, int kind)
{
    if (kind == AMPS_REDUCE_MIN) return fmin(acc, v);
    if (kind == AMPS_REDUCE_MAX) return fmax(acc, v);
    if (kind == AMPS_REDUCE_SUMSQ) return acc + v * v;
    return acc + v;
}

__device__ __forceinline__ double combine(double a, double b, int kind)
{
    if (kind == AMPS_REDUCE_MIN) return fmin(a, b);
    if (kind == AMPS_REDUCE_MAX) return fmax(a, b);
    return a + b;
}

__device__ __forceinline__ double identity(int kind)
{
    return kind == AMPS_REDUCE_MIN ? INFINITY : (kind == AMPS_REDUCE_MAX ? -INFINITY : 0.0);
}

// Block b folds cells [b*C, min(n, (b+1)*C)) in a fixed order and writes one partial.
__global__ void __launch_bounds__(kNoAllocThreads) noalloc_partial_kernel(const double *data, int64_t n, int kind,
                                                                            double *partials)
{
    __shared__ double red[kNoAllocThreads / 32];
    const int64_t lo = (int64_t)blockIdx.x * AMPS_REDUCE_NOALLOC_CELLS_PER_BLOCK;
    const int64_t hi = lo + AMPS_REDUCE_NOALLOC_CELLS_PER_BLOCK < n ? lo + AMPS_REDUCE_NOALLOC_CELLS_PER_BLOCK : n;
    double acc = identity(kind);
    for (int64_t i = lo + threadIdx.x; i < hi; i += kNoAllocThreads) acc = fold(acc, data[i], kind);
    for (int o = 16; o > 0; o >>= 1) acc = combine(acc, __shfl_xor_sync(0xffffffffu, acc, o), kind);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = red[0];
        for (int w = 1; w < kNoAllocThreads / 32; ++w) r = combine(r, red[w], kind);
        partials[blockIdx.x] = r;
    }
}

__global__ void noalloc_final_kernel(const double *partials, int nblocks, int kind, double *out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double r = identity(kind);
    for (int b = 0; b < nblocks; ++b) r = combine(r, partials[b], kind);
    *out = r;
}

// Device address of this device's partials array (looked up once per device).
cudaError_t partials_for_current_device(double **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partials_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) return e;
        g_partials_addr[dev] = static_cast<double *>(p);
    }
    *out = g_partials_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int amps_reduce_noalloc(const double *data, int64_t n, int kind, double *out, void *stream)
{
    if (!data || !out || n < 1 || kind < AMPS_REDUCE_SUM || kind > AMPS_REDUCE_SUMSQ) return AMPS_ERR_INVALID;
    if (n > (int64_t)AMPS_REDUCE_NOALLOC_MAX_CELLS) return AMPS_ERR_UNSUPPORTED;
    double *partials = nullptr;
    if (partials_for_current_device(&partials) != cudaSuccess) return AMPS_ERR_CUDA;
    const int nblocks = (int)((n + AMPS_REDUCE_NOALLOC_CELLS_PER_BLOCK - 1) / AMPS_REDUCE_NOALLOC_CELLS_PER_BLOCK);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // cudaLaunchKernel returns this launch's own status; an error left
    // pending on the calling thread by earlier, unrelated work is neither
    // reported here nor cleared.
    void *pargs[] = {(void *)&data, (void *)&n, (void *)&kind, (void *)&partials};
    if (cudaLaunchKernel((const void *)noalloc_partial_kernel, dim3(nblocks), dim3(kNoAllocThreads), pargs, 0, s) !=
        cudaSuccess)
        return AMPS_ERR_CUDA;
    void *fargs[] = {(void *)&partials, (void *)&nblocks, (void *)&kind, (void *)&out};
    if (cudaLaunchKernel((const void *)noalloc_final_kernel, dim3(1), dim3(32), fargs, 0, s) != cudaSuccess)
        return AMPS_ERR_CUDA;
    return AMPS_OK;
}
