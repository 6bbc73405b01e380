// Float64 inner product that allocates nothing: a variant of mct_dot_f64 whose
// per-block partial sums live in a fixed, file-scope device array instead of a
// caller-provided scratch buffer.
//
// Who needs it: callers that hand this library only their own input and output
// buffers and cannot (or may not) call cudaMalloc themselves -- for example a host
// application or scripting bridge that manages all GPU memory through its own pool
// or a fixed memory budget, and never gives a library spare device memory.
//
// Limits and sharing rules:
//   * the scratch holds MCT_NOALLOC_MAX_PARTIALS float64 values (512 KiB), one per
//     block of 2048 elements, so n may be at most 134,217,728 elements; larger n is
//     rejected with MCT_E_INVALID;
//   * the array exists once per GPU that loads the library and stays allocated until
//     the process exits;
//   * every call uses the same array: calls that overlap on the GPU (different
//     streams, or different host threads) race and must be serialised by the caller;
//   * each call writes every partial it later reads, so the array's previous contents
//     never leak into a result and nothing needs clearing between calls;
//   * the first call on a device looks up the array's device address (with that
//     device current) and caches it; make that first call before any stream capture.
#include <mutex>

#include "common.cuh"

namespace mct {
namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_PER_THREAD = 8;
constexpr int64_t NA_BLOCK_ELEMS = (int64_t)NA_THREADS * NA_PER_THREAD;  // 2048
constexpr int NA_MAX_PARTIALS = 65536;
constexpr int64_t NA_MAX_N = (int64_t)NA_MAX_PARTIALS * NA_BLOCK_ELEMS;  // 134,217,728
constexpr int NA_MAX_DEVICES = 64;

static_assert(NA_MAX_N == 134217728LL, "documented limit");

// The scratch: one float64 partial sum per block.  In host code this name is only a
// host-side handle; its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_partials[NA_MAX_PARTIALS];

__device__ __forceinline__ double na_block_sum(double v) {
    __shared__ double red[NA_THREADS / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    v = (threadIdx.x < NA_THREADS / 32) ? red[threadIdx.x] : 0.0;
    if (w == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}

// Block b sums elements [b*2048, (b+1)*2048) and writes partials[b].
__global__ void __launch_bounds__(NA_THREADS)
noalloc_dot_partial_kernel(const float* __restrict__ a, const float* __restrict__ b, int64_t n,
                           double* __restrict__ partials) {
    const int64_t base = (int64_t)blockIdx.x * NA_BLOCK_ELEMS + threadIdx.x;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < NA_PER_THREAD; ++k) {
        const int64_t i = base + (int64_t)k * NA_THREADS;
        if (i < n) s += (double)a[i] * (double)b[i];
    }
    s = na_block_sum(s);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(NA_THREADS)
noalloc_dot_finish_kernel(const double* __restrict__ partials, int nparts, double* __restrict__ result) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nparts; i += NA_THREADS) s += partials[i];
    s = na_block_sum(s);
    if (threadIdx.x == 0) *result = s;
}

std::mutex g_na_mutex;
double* g_na_ptr[NA_MAX_DEVICES] = {nullptr};

// Device address of the scratch on the current device, looked up once per device and
// kept: it belongs to the device's primary context and is not refreshed after a
// cudaDeviceReset (the header says so).
int noalloc_scratch(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_error("mct_dot_f64_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
        return MCT_E_CUDA;
    }
    MCT_REQUIRE(dev >= 0 && dev < NA_MAX_DEVICES, "mct_dot_f64_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (g_na_ptr[dev] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess || p == nullptr) {
            set_error("mct_dot_f64_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return MCT_E_CUDA;
        }
        g_na_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_na_ptr[dev];
    return MCT_OK;
}

}  // namespace
}  // namespace mct

using namespace mct;

extern "C" int mct_dot_f64_noalloc(const float* a, const float* b, int64_t n, double* result, void* stream) {
    MCT_REQUIRE(n >= 0, "mct_dot_f64_noalloc: negative length");
    MCT_REQUIRE(n <= NA_MAX_N,
                "mct_dot_f64_noalloc: n = %lld exceeds the maximum of %lld elements of the no-allocation variant "
                "(its fixed scratch holds %d partial sums); use mct_dot_f64 with caller scratch",
                (long long)n, (long long)NA_MAX_N, NA_MAX_PARTIALS);
    MCT_REQUIRE(result && (n == 0 || (a && b)), "mct_dot_f64_noalloc: NULL buffer");
    double* partials = nullptr;
    MCT_TRY(noalloc_scratch(&partials));
    cudaStream_t s = as_stream(stream);
    const int nparts = (int)((n + NA_BLOCK_ELEMS - 1) / NA_BLOCK_ELEMS);
    if (nparts > 0) {
        noalloc_dot_partial_kernel<<<nparts, NA_THREADS, 0, s>>>(a, b, n, partials);
        MCT_TRY(launched("noalloc_dot_partial_kernel"));
    }
    noalloc_dot_finish_kernel<<<1, NA_THREADS, 0, s>>>(partials, nparts, result);
    return launched("noalloc_dot_finish_kernel");
}
