// Shared internals of liblfgpu: the handle, device buffers, error plumbing and
// the device-side building blocks (warp reductions, cache-hinted loads, the
// bounded grid barrier) that every kernel file uses.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "lfgpu.h"

namespace lfgpu {

using i64 = long long;

// ------------------------------------------------------------------ host errors
struct Error {
    int code;
    std::string message;
};

#define LF_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t err_ = (call);                                                             \
        if (err_ != cudaSuccess)                                                               \
            throw ::lfgpu::Error{err_ == cudaErrorMemoryAllocation ? LFGPU_ERR_NOMEM : LFGPU_ERR_CUDA, \
                                 std::string(#call) + ": " + cudaGetErrorString(err_)};        \
    } while (0)

#define LF_REQUIRE(cond, code, msg)                     \
    do {                                                \
        if (!(cond)) throw ::lfgpu::Error{(code), (msg)}; \
    } while (0)

// Device buffer that grows on demand and is released with its owner (the handle).
template <typename T>
struct Buf {
    T* p = nullptr;
    size_t count = 0;
    Buf() = default;
    Buf(const Buf&) = delete;
    Buf& operator=(const Buf&) = delete;
    ~Buf() { release(); }  // every buffer of a handle goes with it, whatever lfgpu_destroy lists
    void ensure(size_t n) {
        if (n <= count && p != nullptr) return;
        release();
        if (n == 0) return;
        // Round up to 64 elements so vectorised tails never leave the allocation.
        const size_t padded = (n + 63) / 64 * 64;
        LF_CUDA(cudaMalloc(reinterpret_cast<void**>(&p), padded * sizeof(T)));
        count = n;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        count = 0;
    }
    operator T*() const { return p; }
};

// A wait that gives up after DeviceStatus::wait_limit_ns sets DeviceStatus::abort
// and returns.  The default limit; a handle can set another (lfgpu_set_option).
constexpr unsigned long long kWaitLimitNs = 4000000000ull;  // 4 s

// Device-side status word of one handle.  Kernels record the first failure here;
// the host reads it after the stream synchronises.
struct DeviceStatus {
    int code;            // lfgpu_status of the first failure, 0 if none
    int bad_index;       // element, row or block that caused it (smallest wins)
    unsigned int abort;  // set when any CTA gives up a wait; every wait checks it
    int pad;
    unsigned long long wait_limit_ns;  // how long a bounded wait may spin (the handle's option)
    unsigned long long pad2;
};

// Result record the persistent PCG kernels write (CTA 0) at exit.
struct PcgResult {
    long long iterations;
    long long refinements;
    double initial_residual;
    double final_residual;
    int status;
    int converged;
    int stagnated;
    int pad;
    unsigned long long phase_ns[6];  // CTA 0's time per phase, summed over iterations
};

// Scalars of the grid-wide reductions: one slot per barrier of an iteration,
// each slot holding up to kMaxReduce values per CTA.
constexpr int kMaxReduce = 4;
constexpr int kSlots = 4;

struct Context {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;
    std::string error;
    // The last failure a kernel reported (lfgpu_failure_detail): its status, the
    // index it names and, for a zero pivot carrying load, that DOF's load and
    // diagonal as the sweep left them.
    int fail_code = 0;
    i64 fail_index = -1;
    double fail_values[2] = {0.0, 0.0};

    // mesh
    i64 n_nodes = 0, n_elem = 0, n_mat = 0;
    int plane_mode = 0;
    Buf<double2> xy;
    Buf<int4> elem_nodes;
    Buf<int> elem_mat;
    Buf<double> mat_young, mat_nu, mat_t;
    std::vector<int> h_elem_nodes;  // host copy for setup work
    unsigned long long mesh_version = 0;  // bumps on lfgpu_set_mesh
    Buf<int> ne_ptr, ne_list;             // node -> elements, ascending per node (post-processing)
    unsigned long long ne_version = ~0ull;
    Buf<double> post_fields, post_nodal;

    // pattern
    i64 n = 0, nnz = 0;
    bool have_pattern = false;
    bool paired = false;  // every row has even length and starts at an even offset with (2j, 2j+1) column pairs
    bool pattern_on_device = false;  // lfgpu_build_pattern used the device build
    Buf<int> rowptr, col, map, diag;
    std::vector<int> h_rowptr_cache;
    std::vector<int> h_colors;
    int n_colors = 0;
    std::vector<int> color_offsets;  // host, n_colors + 1
    Buf<int> color_elems;

    // loads
    bool have_nodal = false;
    Buf<double> f_nodal;
    Buf<double> body_bx, body_by;  // per element, or empty
    bool have_body = false;
    Buf<int> edge_ptr;             // per element CSR over edge records (E + 1)
    Buf<int> edge_side, edge_kind;
    Buf<double> edge_a, edge_b;
    bool have_edges = false;

    // constraints
    i64 n_constraints = 0;
    Buf<unsigned char> fixed;
    Buf<double> prescribed;

    // system
    Buf<double> K, K_full, f, f_full;
    bool assembled = false, constrained = false;
    unsigned long long k_version = 0;  // bumps when K changes: invalidates derived matrices

    // derived matrices (built on first use per K version)
    Buf<int> brow, bcol;
    Buf<double> bval64;
    Buf<float> bval32;
    Buf<short> bcol16;      // FP32 BSR columns as offsets from the block row, when all fit in 16 bits
    bool bcol16_ok = false;
    Buf<float> K32;
    Buf<short> col16;       // FP32 CSR columns as offsets from the row, when all fit in 16 bits
    bool col16_ok = false;
    i64 nblocks = 0;
    unsigned long long bsr_version = ~0ull, k32_version = ~0ull, b32_version = ~0ull;
    double last_convert_ms = 0.0;

    // preconditioners
    Buf<double> inv_diag64, blk64;
    Buf<float> inv_diag32, blk32;
    unsigned long long pre_version = ~0ull;
    i64 degenerate_blocks = 0;
    i64 nonfinite_diag = -1;  // first DOF whose diagonal is not finite, -1 if none

    // solve vectors and scratch
    Buf<double> u, R;
    Buf<double> lam, adj_rhs;             // adjoint solution and right-hand side
    Buf<float2> zp[2];                    // mixed graph loop: (z, p) per DOF, two copies
    Buf<float> xhi, xlo;                  // mixed graph loop: FP32 pair of the solution correction
    Buf<double> v64[6];
    Buf<float> v32[6];
    Buf<double> partials;                 // kSlots * kMaxReduce * max CTAs
    Buf<unsigned long long> bar;          // grid barrier counter
    Buf<DeviceStatus> status;
    Buf<PcgResult> pcg_result;
    Buf<char> cg_state;
    Buf<double> scratch64;
    bool solved = false;

    // FP32 inner matrices keep their diagonal as an FP32 (hi, lo) pair that also
    // absorbs each row's off-diagonal rounding error (built with K32 / bval32).
    Buf<float> diag_hi, diag_lo;

    // Tile schedules of the persistent product phase: per matrix format, the row
    // ranges each CTA streams through shared memory (see pcg.cu).
    struct Schedule {
        Buf<int2> tiles;
        Buf<int> cta;
        int grid = 0;
        int units = 0;
        unsigned long long version = ~0ull;
    };
    Schedule sched[4];
    unsigned long long pattern_version = 0;
    std::vector<int> h_brow;

    // IC(0) factor on the pattern of K (ic0.cu): left of the diagonal L(r, c), on
    // it the pivot, right of it L(c, r).  Built per K version; the mirror map (for
    // every upper entry, the index of its lower twin) per pattern version.
    unsigned long long ic0_version = ~0ull, ic0_pattern_version = ~0ull;
    Buf<double> ic0_val, ic0_inv;
    Buf<int> ic0_mirror, ic0_flags, ic0_level;
    Buf<unsigned long long> ic0_misc;  // see kIc0* slots in ic0.cu
    unsigned int ic0_epoch = 0;
    i64 ic0_breakdowns = 0, ic0_levels = 0;

    // Subdomain block-Jacobi (subdomain.cu): the split per (mesh, nodes per
    // subdomain, split kind); the packed lower Cholesky factors per K version.
    i64 sub_nodes = 64;  // the reference's defaults (subdomain_nodes 64, split rcb)
    int sub_split = LFGPU_SPLIT_RCB;
    unsigned long long sub_mesh_version = ~0ull, sub_k_version = ~0ull;
    i64 sub_nodes_built = -1;
    int sub_split_built = -1;
    Buf<int> sub_dofs, sub_begin, sub_owner, sub_local;  // DOFs by subdomain; per DOF: subdomain, slot
    Buf<long long> sub_fac_begin;
    Buf<double> sub_factor;
    Buf<float> sub_inv32;     // mixed loop: each block's inverse, D x D in FP32 (per K version)
    Buf<long long> sub_sq_begin;  // offsets of D x D scratch per subdomain (the inverse's FP64 work)
    unsigned long long sub_inv_version = ~0ull;
    i64 sub_count = 0, sub_degenerate = 0, sub_factor_size = 0, sub_sq_size = 0;
    int sub_max = 0;  // DOFs of the largest subdomain
    double sub_capture = 0.0;

    // IC(0) level schedules of the two sweeps (per pattern version) and the factor
    // in schedule order (per K version; an FP32 copy once a mixed solve asks).
    struct Sweep {
        int levels = 0, entries = 0;
        Buf<int> level_begin;  // 2 per level + 2: first position, first entry
        Buf<int4> pieces;      // per level and cluster CTA, two int4: first and end position, first and
                               // and end entry, then the width of a level ahead (see ic0.cu)
        Buf<int4> desc;        // per position: row, first entry, end entry, output index
        Buf<int> dep;          // per entry: position of the row it depends on
        Buf<double> val, inv;  // factor entries and reciprocal pivots in schedule order
        Buf<float> val32, inv32;
        unsigned long long val_version = ~0ull, val32_version = ~0ull;
    };
    Sweep sweep[2];                   // forward, backward
    unsigned long long sweep_pattern_version = ~0ull;
    int sweep_window = 0;             // ring slots (a power of two); 0: the schedule does not fit
    i64 sweep_max_width = 0, sweep_max_distance = 0;
    int sweep_maxp = 0, sweep_maxe = 0;  // the largest piece a CTA takes of a level: rows, entries
    Buf<double> sweep_y, sweep_rhs;   // forward result in backward positions; r in forward positions
    Buf<float> sweep_y32, sweep_rhs32, sweep_rr32;  // the same in FP32; r32 in backward positions

    // Options (lfgpu_set_option).
    unsigned long long wait_limit_ns = kWaitLimitNs;
    int ic0_sweep = LFGPU_IC0_SWEEP_AUTO;

    lfgpu_timings timings{};
    i64 launches = 0;                 // kernels launched by this handle (graph nodes included)
    cudaEvent_t user_ev[8] = {};      // lfgpu_event_record slots
};

void check_status(Context& c);   // syncs the stream, raises the first device failure
void reset_status(Context& c);
float elapsed_ms(Context& c);    // between ev_a and ev_b (synchronises ev_b)

// ------------------------------------------------------------------ device side
__device__ __forceinline__ void record_failure(DeviceStatus* s, int code, int index) {
    if (atomicCAS(&s->code, 0, code) == 0 || s->code == code) atomicMin(&s->bad_index, index);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Streaming loads for matrix data that is read once per product: evict-first in
// L2 so the iteration vectors stay resident.
__device__ __forceinline__ double ld_stream(const double* p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float* p) { return __ldcs(p); }
__device__ __forceinline__ int ld_stream(const int* p) { return __ldcs(p); }
__device__ __forceinline__ short ld_stream(const short* p) { return __ldcs(p); }
__device__ __forceinline__ double2 ld_stream(const double2* p) { return __ldcs(p); }
__device__ __forceinline__ float4 ld_stream(const float4* p) { return __ldcs(p); }
__device__ __forceinline__ int2 ld_stream(const int2* p) { return __ldcs(p); }

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}


// GPU-scope accesses for values and flags that other CTAs poll while a kernel runs.
__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_gpu(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_gpu(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_relaxed_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// True when a bounded wait started at t0 must stop: another CTA aborted, or the
// limit ran out (then this wait records LFGPU_ERR_TIMEOUT and sets the abort flag).
__device__ __forceinline__ bool wait_expired(DeviceStatus* status, unsigned long long t0, int index) {
    if (ld_relaxed_gpu(&status->abort) != 0u) return true;
    if (global_ns() - t0 > status->wait_limit_ns) {
        atomicExch(&status->abort, 1u);
        record_failure(status, LFGPU_ERR_TIMEOUT, index);
        return true;
    }
    return false;
}

// Grid-wide barrier for cooperative launches, bounded in time.  Every CTA arrives
// with a release add on a monotonically increasing counter and waits (acquire)
// until all CTAs of this episode arrived.  Returns false if the wait ran out or
// another CTA aborted; the caller then leaves its loop.
__device__ __forceinline__ bool grid_barrier(unsigned long long* counter, unsigned long long target,
                                             DeviceStatus* status, int* s_flag) {
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(counter), "l"(1ull) : "memory");
        const unsigned long long start = global_ns();
        int ok = 1;
        while (true) {
            unsigned long long seen;
            asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(seen) : "l"(counter) : "memory");
            if (seen >= target) break;
            unsigned int ab;
            asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(ab) : "l"(&status->abort) : "memory");
            if (ab != 0u) {
                ok = 0;
                break;
            }
            if (global_ns() - start > status->wait_limit_ns) {
                atomicExch(&status->abort, 1u);
                record_failure(status, LFGPU_ERR_TIMEOUT, static_cast<int>(blockIdx.x));
                ok = 0;
                break;
            }
        }
        *s_flag = ok;
    }
    __syncthreads();
    return *s_flag != 0;
}

// Sum K per-thread values over the CTA; thread 0 gets the totals.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* s_red /* [32 * K] */) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) s_red[warp * K + k] = v[k];
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double t = lane < nw ? s_red[lane * K + k] : 0.0;
            v[k] = warp_sum(t);
        }
    }
    __syncthreads();
}

// Grid-wide sum of K values with a fixed reduction order (deterministic): each CTA
// publishes its block sum in its slot, passes the barrier, then every CTA adds the
// published values in CTA order.  Returns false when the barrier gave up.
template <int K>
__device__ __forceinline__ bool grid_sum(double (&v)[K], double* partials, int slot, unsigned long long* counter,
                                         unsigned long long target, DeviceStatus* status, double* s_red,
                                         int* s_flag) {
    block_sum<K>(v, s_red);
    double* mine = partials + (static_cast<size_t>(slot) * gridDim.x + blockIdx.x) * kMaxReduce;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) mine[k] = v[k];
    }
    if (!grid_barrier(counter, target, status, s_flag)) return false;
    if (threadIdx.x < 32) {
        const double* all = partials + static_cast<size_t>(slot) * gridDim.x * kMaxReduce;
        double acc[K];
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] = 0.0;
        for (int b = threadIdx.x; b < static_cast<int>(gridDim.x); b += 32) {
#pragma unroll
            for (int k = 0; k < K; ++k) acc[k] += all[static_cast<size_t>(b) * kMaxReduce + k];
        }
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] = warp_sum(acc[k]);
        if (threadIdx.x == 0) {
#pragma unroll
            for (int k = 0; k < K; ++k) s_red[k] = acc[k];
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = s_red[k];
    __syncthreads();
    return true;
}

// ------------------------------------------------------------------ bulk async copies
// cp.async.bulk (1-D TMA) into shared memory, completion tracked by an mbarrier.
__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ unsigned long long l2_evict_first_policy() {
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

// Global -> shared bulk copy; dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, unsigned bytes, unsigned long long* bar,
                                          unsigned long long policy) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

// The same without an L2 policy (data the next kernels read again).
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Order this CTA's earlier generic-proxy shared-memory accesses before later bulk copies.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for an mbarrier phase, bounded in time; records LFGPU_ERR_TIMEOUT on expiry.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, DeviceStatus* status,
                                          unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long start = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (global_ns() - start > limit_ns) {
            atomicExch(&status->abort, 1u);
            record_failure(status, LFGPU_ERR_TIMEOUT, static_cast<int>(blockIdx.x));
            return false;
        }
    }
    return true;
}

// Wait for copies this CTA already issued into a stage to land before it releases
// its shared memory, after another wait ran out: a bounded spin on the stage's
// phase that neither the abort flag nor the handle's wait limit cuts short (a copy
// lands within microseconds).  False if even this bound ran out.
constexpr unsigned long long kDrainNs = 10000000ull;
__device__ __forceinline__ bool mbar_drain(unsigned long long* bar, unsigned parity) {
    const unsigned long long start = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - start > kDrainNs) return false;
    return true;
}

inline int grid_for(i64 work, int block, int cap = 1 << 20) {
    i64 g = (work + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return static_cast<int>(g);
}

}  // namespace lfgpu
