// Incomplete Cholesky IC(0) of the constrained K on the GPU: the factorisation
// (IncompleteCholesky0, src/precond.cpp:298-384).  The triangular sweeps that
// apply the factor run inside the PCG graph (cg_graph.cu).
//
// Storage.  The factor lives on the pattern of K.  In row r the entries left of
// the diagonal hold L(r, c), the diagonal holds the pivot L(r, r), and the entries
// right of it hold L(c, r) -- the transpose -- so the forward sweep reads the left
// part of each row and the backward sweep the right part, both as contiguous row
// segments of one array.  This needs a structurally symmetric pattern, which Q4
// assembly always produces; the setup checks that every entry right of a diagonal
// has its twin left of the other row's diagonal.
//
// Factorisation.  Row r needs the finished rows c < r it references.  Warps take
// 32-row chunks from a counter in increasing row order; each thread factorises one
// row and waits (bounded) on a per-row flag for every row it references, so a row
// proceeds as soon as its dependencies are done -- no level schedule.  Each row is
// computed by one thread in the reference's operation order without contraction,
// so the factor equals the reference's bit for bit.
//
// Level schedules.  The triangular sweeps (cg_graph.cu) can also run level by
// level: sweep_schedule (host_setup.cpp) lists the rows of each sweep level by
// level, and ensure_ic0_sweep_values copies the factor into that order, so the
// entries a level needs are contiguous.  The forward sweep writes its result in
// the backward sweep's order, so the backward sweep reads it contiguously.
#include "common.cuh"
#include "host_setup.hpp"
#include "kernels.hpp"

#include <climits>
#include <cmath>
#include <thread>

namespace lfgpu {
namespace {

constexpr int kThreads = 256;

// For every entry right of the diagonal of row c (column r > c): the index of the
// entry (r, c) left of the diagonal of row r.  A missing twin records
// LFGPU_ERR_ARGUMENT with the row.
__global__ void ic0_mirror_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                  const int* __restrict__ diag, int* __restrict__ mirror, DeviceStatus* status) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const int d = diag[c], e = rowptr[c + 1];
        for (int k = d + 1; k < e; ++k) {
            const int r = col[k];
            int lo = rowptr[r], hi = diag[r];
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (col[mid] < c) lo = mid + 1;
                else hi = mid;
            }
            const bool found = lo < diag[r] && col[lo] == c;
            mirror[k] = found ? lo : -1;
            if (!found) record_failure(status, LFGPU_ERR_ARGUMENT, c);
        }
    }
}

// max_r |K(r, r)| (the pivot floor's scale, src/precond.cpp:334-338).
__global__ void ic0_scale_kernel(int n, const int* __restrict__ diag, const double* __restrict__ K,
                                 unsigned long long* misc) {
    double m = 0.0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
        m = fmax(m, fabs(K[diag[r]]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&misc[kIc0Scale], static_cast<unsigned long long>(__double_as_longlong(m)));
}

// Bounded wait until row c's flag shows this factorisation's epoch.
__device__ __forceinline__ bool wait_row(const int* flag, int epoch, DeviceStatus* status, int row) {
    if (ld_acquire_gpu(flag) == epoch) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned it = 1;; ++it) {
        if (ld_acquire_gpu(flag) == epoch) return true;
        if ((it & 63u) == 0u && wait_expired(status, t0, row)) return false;
    }
}

// Row r of the factor (src/precond.cpp:344-382): for each c < r in the row,
// L(r,c) = (K(r,c) - sum_j L(r,j) L(c,j)) / L(c,c) over the common columns j < c,
// then L(r,r) = sqrt(K(r,r) - sum_c L(r,c)^2), with a non-positive or non-finite
// value replaced by the floor.
__device__ __forceinline__ void factor_row(int r, const int* __restrict__ rowptr, const int* __restrict__ col,
                                           const int* __restrict__ diag, const double* __restrict__ K, double* F,
                                           double* inv, int* flags, int* level, int epoch, double floor_value,
                                           unsigned long long* misc, DeviceStatus* status) {
    const int b = rowptr[r], d = diag[r];
    int lev = 0;
    for (int k = b; k < d; ++k) {
        const int c = col[k];
        wait_row(flags + c, epoch, status, r);  // on expiry the row is finished with whatever is there
        lev = max(lev, __ldcg(level + c) + 1);
        double sum = K[k];
        int p = b, q = rowptr[c];
        const int qe = diag[c];
        while (p < k && q < qe) {
            const int cp = col[p], cq = col[q];
            if (cp < cq) {
                ++p;
            } else if (cp > cq) {
                ++q;
            } else {
                sum = __dsub_rn(sum, __dmul_rn(F[p], __ldcg(F + q)));
                ++p;
                ++q;
            }
        }
        F[k] = __dmul_rn(sum, __ldcg(inv + c));
    }
    double sum = K[d];
    for (int k = b; k < d; ++k) sum = __dsub_rn(sum, __dmul_rn(F[k], F[k]));
    if (!(sum > 0.0) || !isfinite(sum)) {
        atomicAdd(&misc[kIc0Breakdowns], 1ull);
        sum = floor_value;
    }
    const double pivot = __dsqrt_rn(sum);
    F[d] = pivot;
    inv[r] = __ddiv_rn(1.0, pivot);
    level[r] = lev;
    atomicMax(&misc[kIc0MaxLevel], static_cast<unsigned long long>(lev));
    __threadfence();
    st_release_gpu(flags + r, epoch);
}

__global__ void __launch_bounds__(kThreads) ic0_factor_kernel(int n, const int* __restrict__ rowptr,
                                                              const int* __restrict__ col,
                                                              const int* __restrict__ diag,
                                                              const double* __restrict__ K, double* F, double* inv,
                                                              int* flags, int* level, int epoch,
                                                              unsigned long long* misc, DeviceStatus* status) {
    const int lane = threadIdx.x & 31;
    const double scale = __longlong_as_double(static_cast<long long>(misc[kIc0Scale]));
    const double floor_value = fmax(1.0e-30, 1.0e-14 * scale);
    while (true) {
        int base = 0;
        if (lane == 0) base = static_cast<int>(atomicAdd(&misc[kIc0FactorChunk], 32ull));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const int r = base + lane;
        if (r < n) factor_row(r, rowptr, col, diag, K, F, inv, flags, level, epoch, floor_value, misc, status);
        __syncwarp();
    }
}

// Right of each diagonal: copy L(c, r) from its twin.
__global__ void ic0_transpose_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ diag,
                                     const int* __restrict__ mirror, double* F) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const int e = rowptr[c + 1];
        for (int k = diag[c] + 1; k < e; ++k) F[k] = F[mirror[k]];
    }
}

}  // namespace

void ensure_ic0(Context& c) {
    if (c.ic0_version == c.k_version) return;
    LF_REQUIRE(c.n > 0 && c.n < INT_MAX / 2, LFGPU_ERR_ARGUMENT, "ic0: system size out of range");
    const int n = static_cast<int>(c.n);
    const int grid = grid_for(n, kThreads, 16 * c.num_sms);
    c.ic0_misc.ensure(kIc0Slots);
    if (c.ic0_pattern_version != c.pattern_version) {
        c.ic0_mirror.ensure(c.nnz);
        c.ic0_flags.ensure(n);
        c.ic0_level.ensure(n);
        LF_CUDA(cudaMemsetAsync(c.ic0_flags.p, 0, sizeof(int) * n, c.stream));
        c.ic0_epoch = 0;
        ic0_mirror_kernel<<<grid, kThreads, 0, c.stream>>>(n, c.rowptr, c.col, c.diag, c.ic0_mirror, c.status);
        c.launches += 1;
        LF_CUDA(cudaGetLastError());
        try {
            check_status(c);
        } catch (const Error& e) {
            if (e.code != LFGPU_ERR_ARGUMENT) throw;
            throw Error{LFGPU_ERR_ARGUMENT, "ic0 needs a structurally symmetric pattern"};
        }
        c.ic0_pattern_version = c.pattern_version;
    }
    c.ic0_val.ensure(c.nnz);
    c.ic0_inv.ensure(n);
    if (c.ic0_epoch >= static_cast<unsigned>(INT_MAX)) {
        LF_CUDA(cudaMemsetAsync(c.ic0_flags.p, 0, sizeof(int) * n, c.stream));
        c.ic0_epoch = 0;
    }
    const int epoch = static_cast<int>(++c.ic0_epoch);
    LF_CUDA(cudaMemsetAsync(c.ic0_misc.p, 0, sizeof(unsigned long long) * kIc0Slots, c.stream));
    ic0_scale_kernel<<<grid, kThreads, 0, c.stream>>>(n, c.diag, c.K, c.ic0_misc);
    // Every thread may wait on rows other warps hold, so the grid stays within one
    // resident wave; warps take further chunks from the counter.
    const int resident = c.num_sms * (2048 / kThreads);
    ic0_factor_kernel<<<std::min(resident, grid_for(n, kThreads)), kThreads, 0, c.stream>>>(
        n, c.rowptr, c.col, c.diag, c.K, c.ic0_val, c.ic0_inv, c.ic0_flags, c.ic0_level, epoch, c.ic0_misc, c.status);
    ic0_transpose_kernel<<<grid, kThreads, 0, c.stream>>>(n, c.rowptr, c.diag, c.ic0_mirror, c.ic0_val);
    c.launches += 3;
    LF_CUDA(cudaGetLastError());
    unsigned long long misc[kIc0Slots];
    LF_CUDA(cudaMemcpyAsync(misc, c.ic0_misc.p, sizeof(misc), cudaMemcpyDeviceToHost, c.stream));
    check_status(c);
    c.ic0_breakdowns = static_cast<i64>(misc[kIc0Breakdowns]);
    // The forward and the backward sweep each have (longest chain + 1) levels.
    c.ic0_levels = 2 * (static_cast<i64>(misc[kIc0MaxLevel]) + 1);
    c.ic0_version = c.k_version;
}

// ------------------------------------------------------------------ level schedules
namespace {

// Factor entries and reciprocal pivots in schedule order: forward entries are
// row r's columns left of its diagonal, ascending; backward entries row c's
// columns right of its diagonal, descending (the L(c, r) the transpose stored there).
template <typename T>
__global__ void ic0_schedule_values_kernel(int n, bool forward, const int4* __restrict__ desc,
                                           const int* __restrict__ rowptr, const int* __restrict__ diag,
                                           const double* __restrict__ F, const double* __restrict__ inv,
                                           T* __restrict__ val, T* __restrict__ pinv) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int4 d = desc[p];
        const int row = d.x;
        if (forward) {
            const int b = rowptr[row];
            for (int j = d.y; j < d.z; ++j) val[j] = static_cast<T>(F[b + (j - d.y)]);
        } else {
            const int top = rowptr[row + 1] - 1;
            for (int j = d.y; j < d.z; ++j) val[j] = static_cast<T>(F[top - (j - d.y)]);
        }
        pinv[p] = static_cast<T>(inv[row]);
    }
}

}  // namespace

void ensure_ic0_schedule(Context& c) {
    if (c.sweep_pattern_version == c.pattern_version) return;
    const int n = static_cast<int>(c.n);
    std::vector<int> rowptr(static_cast<size_t>(n) + 1), col(static_cast<size_t>(c.nnz)), diag(static_cast<size_t>(n));
    LF_CUDA(cudaMemcpyAsync(rowptr.data(), c.rowptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, c.stream));
    LF_CUDA(cudaMemcpyAsync(col.data(), c.col.p, sizeof(int) * c.nnz, cudaMemcpyDeviceToHost, c.stream));
    LF_CUDA(cudaMemcpyAsync(diag.data(), c.diag.p, sizeof(int) * n, cudaMemcpyDeviceToHost, c.stream));
    LF_CUDA(cudaStreamSynchronize(c.stream));
    SweepSchedule fw, bw;
    std::thread other([&] { sweep_schedule(n, rowptr.data(), col.data(), diag.data(), false, bw); });
    sweep_schedule(n, rowptr.data(), col.data(), diag.data(), true, fw);
    other.join();
    // The forward sweep writes y(r) where the backward sweep reads it: r's backward position.
    for (int p = 0; p < n; ++p) fw.desc[4 * static_cast<size_t>(p) + 3] = bw.position[static_cast<size_t>(fw.desc[4 * static_cast<size_t>(p)])];
    const SweepSchedule* both[2] = {&fw, &bw};
    long long need = 0;
    c.sweep_max_width = 0;
    c.sweep_max_distance = 0;
    c.sweep_maxp = 0;
    c.sweep_maxe = 0;
    std::vector<int> pieces;
    for (int d = 0; d < 2; ++d) {
        const SweepSchedule& s = *both[d];
        // Slots a level overwrites must hold no row a CTA still reads; CTAs run at
        // most one level apart, so the ring spans the longest dependency distance
        // plus two levels.
        need = std::max(need, s.max_distance + 2LL * s.max_width);
        c.sweep_max_width = std::max<i64>(c.sweep_max_width, s.max_width);
        c.sweep_max_distance = std::max<i64>(c.sweep_max_distance, s.max_distance);
        Context::Sweep& dst = c.sweep[d];
        dst.levels = s.levels;
        dst.entries = static_cast<int>(s.dep.size());
        dst.level_begin.ensure(s.level_begin.size());
        dst.desc.ensure(static_cast<size_t>(n));
        dst.dep.ensure(s.dep.size() + kSweepSlack);
        LF_CUDA(cudaMemcpyAsync(dst.level_begin.p, s.level_begin.data(), sizeof(int) * s.level_begin.size(),
                                cudaMemcpyHostToDevice, c.stream));
        LF_CUDA(cudaMemcpyAsync(dst.desc.p, s.desc.data(), sizeof(int) * s.desc.size(), cudaMemcpyHostToDevice,
                                c.stream));
        if (!s.dep.empty())
            LF_CUDA(cudaMemcpyAsync(dst.dep.p, s.dep.data(), sizeof(int) * s.dep.size(), cudaMemcpyHostToDevice,
                                    c.stream));
        // Each level's rows split into kSweepCluster contiguous pieces, one per
        // cluster CTA: first and end position, first and end entry; then the width
        // of level L - 1 + kSweepRingBars, whose ring mbarrier is armed at the end
        // of level L (-1: none).
        pieces.assign(8 * static_cast<size_t>(s.levels) * kSweepCluster, 0);
        for (int L = 0; L < s.levels; ++L) {
            const int p0 = s.level_begin[2 * static_cast<size_t>(L)], p1 = s.level_begin[2 * static_cast<size_t>(L) + 2];
            const int chunk = (p1 - p0 + kSweepCluster - 1) / kSweepCluster;
            for (int k = 0; k < kSweepCluster; ++k) {
                const int first = std::min(p1, p0 + k * chunk), end = std::min(p1, first + chunk);
                int* pc = &pieces[8 * (static_cast<size_t>(L) * kSweepCluster + k)];
                pc[0] = first;
                pc[1] = end;
                pc[2] = first < end ? s.desc[4 * static_cast<size_t>(first) + 1] : 0;
                pc[3] = first < end ? s.desc[4 * static_cast<size_t>(end - 1) + 2] : 0;
                const int ahead = L - 1 + kSweepRingBars;
                pc[4] = L > 0 && ahead < s.levels
                            ? s.level_begin[2 * static_cast<size_t>(ahead) + 2] - s.level_begin[2 * static_cast<size_t>(ahead)]
                            : -1;
                c.sweep_maxp = std::max(c.sweep_maxp, end - first);
                c.sweep_maxe = std::max(c.sweep_maxe, pc[3] - pc[2]);
            }
        }
        dst.pieces.ensure(std::max<size_t>(2, pieces.size() / 4));
        if (!pieces.empty())
            LF_CUDA(cudaMemcpyAsync(dst.pieces.p, pieces.data(), sizeof(int) * pieces.size(), cudaMemcpyHostToDevice,
                                    c.stream));
        LF_CUDA(cudaStreamSynchronize(c.stream));  // `pieces` is refilled for the other sweep
        dst.val_version = dst.val32_version = ~0ull;
    }
    int window = 256;
    while (window < need && window <= kSweepRingMax) window *= 2;
    c.sweep_window = window <= kSweepRingMax ? window : 0;
    // Both precisions' rings and stages must fit one CTA's shared memory.
    int optin = 0;
    LF_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c.device));
    if (c.sweep_window > 0 &&
        sweep_smem_bytes(static_cast<int>(sizeof(double)), c.sweep_window, c.sweep_maxp, c.sweep_maxe) +
                kSweepStaticSmem >
            optin)
        c.sweep_window = 0;
    LF_CUDA(cudaStreamSynchronize(c.stream));  // the host schedules are released on return
    c.sweep_pattern_version = c.pattern_version;
}

void ensure_ic0_sweep_values(Context& c, bool fp32) {
    const int n = static_cast<int>(c.n);
    const int grid = grid_for(n, kThreads, 16 * c.num_sms);
    for (int d = 0; d < 2; ++d) {
        Context::Sweep& s = c.sweep[d];
        const int total = s.entries;
        if (s.val_version != c.ic0_version) {
            s.val.ensure(static_cast<size_t>(total) + kSweepSlack);
            s.inv.ensure(static_cast<size_t>(n) + kSweepSlack);
            ic0_schedule_values_kernel<double><<<grid, kThreads, 0, c.stream>>>(
                n, d == 0, s.desc, c.rowptr, c.diag, c.ic0_val, c.ic0_inv, s.val, s.inv);
            c.launches += 1;
            s.val_version = c.ic0_version;
        }
        if (fp32 && s.val32_version != c.ic0_version) {
            s.val32.ensure(static_cast<size_t>(total) + kSweepSlack);
            s.inv32.ensure(static_cast<size_t>(n) + kSweepSlack);
            ic0_schedule_values_kernel<float><<<grid, kThreads, 0, c.stream>>>(
                n, d == 0, s.desc, c.rowptr, c.diag, c.ic0_val, c.ic0_inv, s.val32, s.inv32);
            c.launches += 1;
            s.val32_version = c.ic0_version;
        }
    }
    LF_CUDA(cudaGetLastError());
}

// LFGPU_IC0_SWEEP_AUTO takes the FP64 level sweeps where the forward schedule's
// levels hold kLevelsMinWidth rows on average or more.  A level costs them about
// 1.8 us whatever its width (one row's FP64 chain plus the exchange); the polled
// sweeps' cost per level grows with it.  Per forward + backward application on
// GB300 (cantilever workloads, RCM): 200x200, 50 rows a level: polled 3.9 ms,
// levels 5.6 ms; 500x500, 125 rows: 13.3-13.6 ms, 14.1 ms; 1000x1000, 250 rows:
// 30.5-30.9 ms, 28.4 ms.
constexpr i64 kLevelsMinWidth = 192;

bool ic0_levels_chosen(const Context& c, bool required) {
    if (c.sweep_window <= 0 || c.sweep_pattern_version != c.pattern_version) return false;
    if (required || c.ic0_sweep == LFGPU_IC0_SWEEP_LEVELS) return true;
    return c.ic0_sweep == LFGPU_IC0_SWEEP_AUTO && c.n >= kLevelsMinWidth * c.sweep[0].levels;
}

bool ic0_use_levels(Context& c, bool required) {
    if (c.ic0_sweep == LFGPU_IC0_SWEEP_POLLED && !required) return false;
    LF_REQUIRE(c.ic0_sweep != LFGPU_IC0_SWEEP_POLLED, LFGPU_ERR_UNSUPPORTED,
               "mixed-precision ic0 needs the level-scheduled sweeps");
    ensure_ic0_schedule(c);
    if (c.sweep_window > 0) return ic0_levels_chosen(c, required);
    LF_REQUIRE(!required && c.ic0_sweep == LFGPU_IC0_SWEEP_AUTO, LFGPU_ERR_UNSUPPORTED,
               "the ic0 level schedule does not fit the sweep's shared-memory ring");
    return false;
}

}  // namespace lfgpu
