// lfgpu_residual_norm_noalloc: ||f - K u||_2 of a CSR system in caller-owned
// device memory, computed without allocating anything.
//
// Some callers cannot call cudaMalloc: code inside a host framework that owns all
// device memory through its own pool and forbids driver allocations, and
// latency-critical loops where an allocation (which can synchronise the device)
// is not acceptable.  This entry point serves them: it takes device pointers to
// the caller's arrays and keeps its only scratch -- one partial sum per thread
// block, an arrival counter and the result -- in a file-scope static device array
// of fixed size, allocated once when the library's module is loaded in a context
// and held until the process exits.  The call copies the result to host memory
// and synchronises the caller's stream before it returns.
//
// The same residual is what lfgpu_solve reports as true_residual (there through a
// product into a scratch vector and a separate norm); here one kernel computes
// each row's residual with the same per-row arithmetic and accumulates its square,
// and the last block to finish adds the per-block partials in a fixed order, so
// the result is deterministic.
//
// Every call in a context shares the one array, and the array keeps the last
// call's contents.  The arrival counter is cleared on the stream before each
// launch; nothing else needs to start at zero.  Calls whose work overlaps on the
// GPU (two streams, or two host threads) race on the array: issue them on one
// stream, one after the other.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "lfgpu.h"

namespace {

constexpr int kThreads = 256;
constexpr int kRowsPerBlock = kThreads / 4;          // 4 lanes per row
constexpr int kMaxBlocks = 65536;                    // partial sums held in the scratch
static_assert(static_cast<long long>(kMaxBlocks) * kRowsPerBlock == LFGPU_NOALLOC_MAX_ROWS,
              "one partial sum per block of the largest accepted system");
constexpr int kMaxDevices = 64;

// Layout: [0, kMaxBlocks) per-block partial sums, then the result, then the
// arrival counter (as an unsigned int in the next slot).  512 KiB + 256 B.
constexpr int kResultSlot = kMaxBlocks;
constexpr int kCounterSlot = kMaxBlocks + 1;
static __device__ __align__(256) double g_scratch[kMaxBlocks + 32];

// Device address of g_scratch per device, resolved with that device current and
// kept with the unique ID of the context it was resolved in.  A new context on the
// device (after cudaDeviceReset, or a host framework's own driver context) loads
// the module anew, possibly at another address, so its first call resolves again.
struct ScratchAddress {
    unsigned long long context_id = 0;
    void* address = nullptr;
};
ScratchAddress g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mutex;

// The driver's current-context queries, reached through the runtime so that the
// library needs no link against the driver library.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

bool current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (get_current == nullptr || get_id == nullptr) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1{}, q2{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || f1 == nullptr)
            return false;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q2 != cudaDriverEntryPointSuccess || f2 == nullptr)
            return false;
        get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return false;
    return get_id(ctx, id) == CUDA_SUCCESS;
}

__global__ void __launch_bounds__(kThreads) residual_norm_kernel(int n, const int* __restrict__ rowptr,
                                                                  const int* __restrict__ col,
                                                                  const double* __restrict__ val,
                                                                  const double* __restrict__ u,
                                                                  const double* __restrict__ f,
                                                                  double* __restrict__ scratch) {
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 2;
    const int q = threadIdx.x & 3;
    double s = 0.0;
    if (row < n) {
        const int b = rowptr[row], e = rowptr[row + 1];
        for (int k = b + q; k < e; k += 8) {
            const bool two = k + 4 < e;
            const int c0 = col[k], c1 = two ? col[k + 4] : c0;
            const double v0 = val[k], v1 = two ? val[k + 4] : 0.0;
            s += v0 * u[c0];
            s += v1 * u[c1];
        }
    }
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    double sq = 0.0;
    if (row < n && q == 0) {
        const double r = s - f[row];
        sq = r * r;
    }
    // block sum of the squares
    __shared__ double red[kThreads / 32];
    __shared__ int last;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sq;
    __syncthreads();
    unsigned int* counter = reinterpret_cast<unsigned int*>(scratch + kCounterSlot);
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) t += red[w];
        scratch[blockIdx.x] = t;
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double t = 0.0;
    for (int k = threadIdx.x; k < static_cast<int>(gridDim.x); k += kThreads) t += __ldcg(scratch + k);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double total = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) total += red[w];
        scratch[kResultSlot] = sqrt(total);
        *counter = 0u;
    }
}

}  // namespace

extern "C" int lfgpu_residual_norm_noalloc(int64_t n_rows, const int32_t* row_offsets, const int32_t* columns,
                                           const double* values, const double* u, const double* f, void* stream,
                                           double* norm_out) {
    if (n_rows < 0 || norm_out == nullptr) return LFGPU_ERR_ARGUMENT;
    if (n_rows > LFGPU_NOALLOC_MAX_ROWS) return LFGPU_ERR_SCRATCH_LIMIT;
    if (n_rows > 0 && (!row_offsets || !columns || !values || !u || !f)) return LFGPU_ERR_ARGUMENT;
    int device = -1;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) return LFGPU_ERR_CUDA;
    double* scratch = nullptr;
    {
        // First call on this device, or in a new context on it: resolve the array's
        // address with the device current.  This can load the module in the
        // context, so that first call must come before any stream capture.
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        ScratchAddress& slot = g_scratch_addr[device];
        unsigned long long id = 0;
        if (slot.address == nullptr || !current_context_id(&id) || id != slot.context_id) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || p == nullptr) return LFGPU_ERR_CUDA;
            // cudaGetSymbolAddress made the device's primary context current if
            // no context was: record the context the address belongs to.
            if (!current_context_id(&id)) return LFGPU_ERR_CUDA;
            slot.address = p;
            slot.context_id = id;
        }
        scratch = static_cast<double*>(slot.address);
    }
    if (n_rows == 0) {
        *norm_out = 0.0;
        return LFGPU_OK;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The arrival counter must start at zero.  The kernel's last block leaves it at
    // zero, so this only matters after a call that did not finish.
    if (cudaMemsetAsync(scratch + kCounterSlot, 0, sizeof(double), s) != cudaSuccess) return LFGPU_ERR_CUDA;
    const int blocks = static_cast<int>((n_rows + kRowsPerBlock - 1) / kRowsPerBlock);
    residual_norm_kernel<<<blocks, kThreads, 0, s>>>(static_cast<int>(n_rows), row_offsets, columns, values, u, f,
                                                     scratch);
    if (cudaGetLastError() != cudaSuccess) return LFGPU_ERR_CUDA;
    if (cudaMemcpyAsync(norm_out, scratch + kResultSlot, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return LFGPU_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return LFGPU_ERR_CUDA;
    return LFGPU_OK;
}
