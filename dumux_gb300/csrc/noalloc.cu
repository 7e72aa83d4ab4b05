// noalloc.cu -- Euclidean norm of a device vector without any device allocation.
//
// Some callers cannot allocate device memory while they run: an application whose
// device memory is owned by its own allocator or budget, or a solver loop that must
// not call cudaMalloc because that call can synchronise the device and stall the work
// of other streams.  For them dxg_norm2_noalloc computes ||x||_2 with its reduction
// scratch (per-block partial sums and a completion counter) in a fixed array in the
// library's own device memory, reserved on each device when the library's device code
// is loaded there (at the latest during the first call on that device).
//
// Every call on a device shares that array: calls whose kernels overlap on the GPU
// (different streams, no ordering between them) race on it and give wrong results.
// Order such calls on one stream or with events.
#include <mutex>

#include "common.cuh"

namespace dxg {

// At most kNoAllocMaxBlocks blocks of kNoAllocThreads threads, each thread summing
// kNoAllocPerThread entries: vectors up to 4096 * 256 * 8 = 8,388,608 entries.
constexpr int kNoAllocMaxBlocks = 4096;
constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocPerThread = 8;
constexpr int64_t kNoAllocMaxEntries = (int64_t)kNoAllocMaxBlocks * kNoAllocThreads * kNoAllocPerThread;

// [0, kNoAllocMaxBlocks): partial sums (double bit patterns); [kNoAllocMaxBlocks]:
// completion counter.  33 KB, held by every GPU that loads the library until exit.
static __device__ __align__(256) unsigned long long g_noallocScratch[kNoAllocMaxBlocks + 1];

__global__ void __launch_bounds__(kNoAllocThreads) norm2NoAllocKernel(const double* __restrict__ x, int64_t n,
                                                                      unsigned long long* scratch, double* result)
{
    const int64_t span = (int64_t)kNoAllocThreads * kNoAllocPerThread;
    const int64_t begin = (int64_t)blockIdx.x * span;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kNoAllocPerThread; ++k) {
        const int64_t i = begin + (int64_t)k * kNoAllocThreads + threadIdx.x;
        if (i < n) s += x[i] * x[i];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ double warpSums[kNoAllocThreads / 32];
    __shared__ bool amLast;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) warpSums[wid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < kNoAllocThreads / 32; ++w) b += warpSums[w];
        scratch[blockIdx.x] = (unsigned long long)__double_as_longlong(b);
        __threadfence();
        amLast = atomicAdd(&scratch[kNoAllocMaxBlocks], 1ull) == (unsigned long long)(gridDim.x - 1);
    }
    __syncthreads();
    if (!amLast || threadIdx.x != 0) return;
    __threadfence();
    // the last block adds the partial sums in block order
    double total = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b)
        total += __longlong_as_double((long long)((volatile unsigned long long*)scratch)[b]);
    *result = sqrt(total);
    scratch[kNoAllocMaxBlocks] = 0ull;
}

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noallocMutex;
unsigned long long* g_noallocAddr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once per
// device; the host-side symbol itself is not a device address).
int scratchAddress(unsigned long long** out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DXG_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (!g_noallocAddr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess || !p) return DXG_ERR_CUDA;
        g_noallocAddr[dev] = static_cast<unsigned long long*>(p);
    }
    *out = g_noallocAddr[dev];
    return DXG_OK;
}
}  // namespace

}  // namespace dxg

extern "C" {

int dxg_norm2_noalloc(const double* x, int64_t n, double* result, void* stream)
{
    using namespace dxg;
    if (!result || (n > 0 && !x) || n < 0) return DXG_ERR_ARG;
    // the fixed scratch covers at most kNoAllocMaxEntries entries: refuse longer vectors
    if (n > kNoAllocMaxEntries) return DXG_ERR_SIZE;
    unsigned long long* scratch = nullptr;
    const int st = scratchAddress(&scratch);
    if (st != DXG_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the completion counter must start at zero (an interrupted earlier call may have
    // left it set); the partial sums are all overwritten before they are read
    cudaError_t e = cudaMemsetAsync(scratch + kNoAllocMaxBlocks, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) {
        const int64_t span = (int64_t)kNoAllocThreads * kNoAllocPerThread;
        const int blocks = n == 0 ? 1 : (int)((n + span - 1) / span);
        norm2NoAllocKernel<<<blocks, kNoAllocThreads, 0, s>>>(x, n, scratch, result);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? DXG_OK : DXG_ERR_CUDA;
}

}  // extern "C"
