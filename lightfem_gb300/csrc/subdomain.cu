// Subdomain block-Jacobi setup: the reference's SubdomainBlockJacobi
// (src/precond.cpp:121-238) for any subdomain size.
//
// The split (build_dof_subdomain, src/solver.cpp:631-653) runs on the host:
// chunks of consecutive nodes or recursive coordinate bisection, the two DOFs of a
// node in its node's subdomain.  A subdomain lists its DOFs in ascending order,
// and its dense block takes K's entries whose row and column both belong to it.
//
// The factor runs on the device, one CTA per subdomain, in place in the packed
// lower factor (only the lower triangle of the dense block is ever read).  It is
// a right-looking Cholesky: after pivot j, every entry (i, m) with j < m <= i
// subtracts L(i, j) L(m, j).  Each entry therefore subtracts its products in the
// same order (j ascending) as the reference's row-by-row loop, and each product, difference, square root and quotient is
// rounded on its own.  So the factor equals the reference's bit for bit.  A block
// whose pivot is not positive and finite becomes the identity, as there.  The
// packed lower factor stores reciprocal pivots on its diagonal, as the
// reference's does.
//
// For the mixed loop the setup also builds each block's inverse from the FP64
// factor and stores it in FP32 as a full square (ensure_subdomain_inverse).
#include "common.cuh"
#include "kernels.hpp"
#include "host_setup.hpp"

#include <algorithm>
#include <vector>

namespace lfgpu {
namespace {

constexpr int kCaptureThreads = 256;

__global__ void __launch_bounds__(LFGPU_SUBDOMAIN_MAX_DOFS) subdomain_factor_kernel(
    const int* __restrict__ rowptr, const int* __restrict__ col, const double* __restrict__ K,
    const int* __restrict__ sub_dofs, const int* __restrict__ sub_begin, const int* __restrict__ owner,
    const int* __restrict__ local, const long long* __restrict__ fac_begin, double* factor,
    unsigned long long* __restrict__ degenerate) {
    __shared__ double colj[LFGPU_SUBDOMAIN_MAX_DOFS];  // column j of L below the pivot
    __shared__ int s_fail;
    const int s = blockIdx.x;
    const int begin = sub_begin[s], D = sub_begin[s + 1] - begin;
    const int t = threadIdx.x, T = blockDim.x, lane = t & 31, warp = t >> 5, W = T >> 5;
    double* L = factor + fac_begin[s];  // packed lower triangle, row i at i (i + 1) / 2
    auto row = [&](int i) { return L + static_cast<long long>(i) * (i + 1) / 2; };
    const long long size = static_cast<long long>(D) * (D + 1) / 2;
    for (long long k = t; k < size; k += T) L[k] = 0.0;
    if (t == 0) s_fail = 0;
    __syncthreads();
    // The lower triangle of the dense block (the only part the factorisation reads).
    for (int i = t; i < D; i += T) {
        const int dof = sub_dofs[begin + i];
        double* ri = row(i);
        for (int k = rowptr[dof]; k < rowptr[dof + 1]; ++k) {
            const int c = col[k];
            if (owner[c] != s) continue;
            const int m = local[c];
            if (m <= i) ri[m] = K[k];
        }
    }
    __syncthreads();
    for (int j = 0; j < D; ++j) {
        double* rj = row(j);
        if (t == 0) {
            const double d = rj[j];
            if (!(d > 0.0) || !isfinite(d)) s_fail = 1;
            else rj[j] = __dsqrt_rn(d);
        }
        __syncthreads();
        if (s_fail) break;
        const double pivot = rj[j];
        for (int i = j + 1 + t; i < D; i += T) {
            const double v = __ddiv_rn(row(i)[j], pivot);
            row(i)[j] = v;
            colj[i] = v;
        }
        __syncthreads();
        // Trailing update, a warp per row (rows interleaved over warps), lanes over
        // the row's entries j < m <= i; each entry is updated once per step.
        for (int i = j + 1 + warp; i < D; i += W) {
            double* ri = row(i);
            const double lij = colj[i];
            for (int m = j + 1 + lane; m <= i; m += 32) ri[m] = __dsub_rn(ri[m], __dmul_rn(lij, colj[m]));
        }
        __syncthreads();
    }
    const bool fail = s_fail != 0;
    for (int i = t; i < D; i += T) {
        double* ri = row(i);
        if (fail) {
            for (int m = 0; m < i; ++m) ri[m] = 0.0;
            ri[i] = 1.0;
        } else {
            ri[i] = __ddiv_rn(1.0, ri[i]);  // reciprocal pivot
        }
    }
    if (fail && t == 0) atomicAdd(degenerate, 1ull);
}

// subdomain_capture_ratio (src/precond.cpp:107-119): entries whose row and column
// share a subdomain.
__global__ void __launch_bounds__(kCaptureThreads) subdomain_capture_kernel(int n, const int* __restrict__ rowptr,
                                                                            const int* __restrict__ col,
                                                                            const int* __restrict__ owner,
                                                                            unsigned long long* __restrict__ inside) {
    unsigned long long count = 0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const int o = owner[r];
        for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) count += owner[col[k]] == o;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) count += __shfl_xor_sync(0xffffffffu, count, d);
    if ((threadIdx.x & 31) == 0 && count) atomicAdd(inside, count);
}

// Each block's inverse M^-1 = (L L^T)^-1 for the mixed loop: thread j solves
// L L^T x = e_j in FP64 with the packed factor (forward, then backward in place,
// x in the FP64 scratch `work`, laid out k-major so that the threads' accesses
// coalesce), and stores the whole inverse in FP32 as a D x D square (one
// subdomain after another at the scratch's offsets).  Forward, the lanes of a warp
// read neighbouring entries of one factor row; backward, every thread reads the
// same entry (a broadcast).
__global__ void __launch_bounds__(LFGPU_SUBDOMAIN_MAX_DOFS) subdomain_inverse_kernel(
    const int* __restrict__ sub_begin, const long long* __restrict__ fac_begin,
    const long long* __restrict__ sq_begin, const double* __restrict__ factor, double* __restrict__ work,
    float* __restrict__ inv) {
    const int s = blockIdx.x, j = threadIdx.x;
    const int D = sub_begin[s + 1] - sub_begin[s];
    const double* L = factor + fac_begin[s];
    double* x = work + sq_begin[s];  // x[k * D + j]: entry k of thread j's column
    const bool mine = j < D;
    for (int i = 0; i < D; ++i) {  // forward: L y = e_j (y_k = 0 for k < j)
        const double* li = L + static_cast<long long>(i) * (i + 1) / 2;
        double acc = (i == j) ? 1.0 : 0.0;
        if (i > j)
            for (int k = j; k < i; ++k) acc = fma(-li[k], x[static_cast<long long>(k) * D + j], acc);
        if (mine) x[static_cast<long long>(i) * D + j] = i < j ? 0.0 : acc * li[i];  // li[i]: reciprocal pivot
    }
    for (int i = D - 1; i >= 0; --i) {  // backward: L^T x = y, in place
        double acc = mine ? x[static_cast<long long>(i) * D + j] : 0.0;
        for (int k = i + 1; k < D; ++k)
            acc = fma(-L[static_cast<long long>(k) * (k + 1) / 2 + i], mine ? x[static_cast<long long>(k) * D + j] : 0.0,
                      acc);
        if (mine) x[static_cast<long long>(i) * D + j] = acc * L[static_cast<long long>(i) * (i + 1) / 2 + i];
    }
    // The whole square in FP32, in the scratch's layout: entry (k, j) at k D + j,
    // which by symmetry is also entry (j, k).
    float* out = inv + sq_begin[s];
    for (int k = 0; k < D; ++k)
        if (mine) out[static_cast<long long>(k) * D + j] = static_cast<float>(x[static_cast<long long>(k) * D + j]);
}

// The split and the per-subdomain DOF lists, rebuilt when the mesh or the
// requested split changes.
void build_split(Context& c) {
    LF_REQUIRE(c.n == 2 * c.n_nodes, LFGPU_ERR_STATE, "the subdomain split needs the pattern of the current mesh");
    std::vector<double2> xy2(static_cast<size_t>(c.n_nodes));
    LF_CUDA(cudaMemcpyAsync(xy2.data(), c.xy.p, sizeof(double2) * xy2.size(), cudaMemcpyDeviceToHost, c.stream));
    LF_CUDA(cudaStreamSynchronize(c.stream));
    std::vector<double> xy(2 * xy2.size());
    for (size_t k = 0; k < xy2.size(); ++k) {
        xy[2 * k] = xy2[k].x;
        xy[2 * k + 1] = xy2[k].y;
    }
    std::vector<uint32_t> node_owner;
    const i64 S = subdomain_split(c.n_nodes, xy.data(), c.sub_nodes, c.sub_split == LFGPU_SPLIT_RCB, node_owner);
    const i64 n = c.n;
    // DOFs of each subdomain in ascending order, and each DOF's slot in its list.
    std::vector<int> begin(static_cast<size_t>(S) + 1, 0), dofs(static_cast<size_t>(n)), owner(static_cast<size_t>(n)),
        local(static_cast<size_t>(n));
    for (i64 d = 0; d < n; ++d) {
        owner[static_cast<size_t>(d)] = static_cast<int>(node_owner[static_cast<size_t>(d / 2)]);
        ++begin[static_cast<size_t>(owner[static_cast<size_t>(d)]) + 1];
    }
    int largest = 0;
    for (i64 k = 0; k < S; ++k) {
        largest = std::max(largest, begin[static_cast<size_t>(k) + 1]);
        begin[static_cast<size_t>(k) + 1] += begin[static_cast<size_t>(k)];
    }
    LF_REQUIRE(largest <= LFGPU_SUBDOMAIN_MAX_DOFS, LFGPU_ERR_UNSUPPORTED,
               "a subdomain holds " + std::to_string(largest) + " DOFs; the GPU block factor takes at most " +
                   std::to_string(LFGPU_SUBDOMAIN_MAX_DOFS));
    std::vector<int> cursor(begin.begin(), begin.end() - 1);
    for (i64 d = 0; d < n; ++d) {
        const int o = owner[static_cast<size_t>(d)];
        const int slot = cursor[static_cast<size_t>(o)]++;
        dofs[static_cast<size_t>(slot)] = static_cast<int>(d);
        local[static_cast<size_t>(d)] = slot - begin[static_cast<size_t>(o)];
    }
    std::vector<long long> fac(static_cast<size_t>(S) + 1, 0), sq(static_cast<size_t>(S) + 1, 0);
    for (i64 k = 0; k < S; ++k) {
        const long long size = begin[static_cast<size_t>(k) + 1] - begin[static_cast<size_t>(k)];
        fac[static_cast<size_t>(k) + 1] = fac[static_cast<size_t>(k)] + size * (size + 1) / 2;
        sq[static_cast<size_t>(k) + 1] = sq[static_cast<size_t>(k)] + size * size;
    }
    c.sub_dofs.ensure(static_cast<size_t>(n));
    c.sub_owner.ensure(static_cast<size_t>(n));
    c.sub_local.ensure(static_cast<size_t>(n));
    c.sub_begin.ensure(static_cast<size_t>(S) + 1);
    c.sub_fac_begin.ensure(static_cast<size_t>(S) + 1);
    c.sub_sq_begin.ensure(static_cast<size_t>(S) + 1);
    LF_CUDA(cudaMemcpyAsync(c.sub_dofs.p, dofs.data(), sizeof(int) * dofs.size(), cudaMemcpyHostToDevice, c.stream));
    LF_CUDA(cudaMemcpyAsync(c.sub_owner.p, owner.data(), sizeof(int) * owner.size(), cudaMemcpyHostToDevice,
                            c.stream));
    LF_CUDA(cudaMemcpyAsync(c.sub_local.p, local.data(), sizeof(int) * local.size(), cudaMemcpyHostToDevice,
                            c.stream));
    LF_CUDA(cudaMemcpyAsync(c.sub_begin.p, begin.data(), sizeof(int) * begin.size(), cudaMemcpyHostToDevice,
                            c.stream));
    LF_CUDA(cudaMemcpyAsync(c.sub_fac_begin.p, fac.data(), sizeof(long long) * fac.size(), cudaMemcpyHostToDevice,
                            c.stream));
    LF_CUDA(cudaMemcpyAsync(c.sub_sq_begin.p, sq.data(), sizeof(long long) * sq.size(), cudaMemcpyHostToDevice,
                            c.stream));
    c.sub_sq_size = sq.back();
    LF_CUDA(cudaStreamSynchronize(c.stream));  // the host vectors end with this function
    c.sub_count = S;
    c.sub_max = largest;
    c.sub_factor_size = fac.back();
    c.sub_mesh_version = c.mesh_version;
    c.sub_nodes_built = c.sub_nodes;
    c.sub_split_built = c.sub_split;
    c.sub_k_version = ~0ull;    // the factors and the mixed loop's inverses follow the new split
    c.sub_inv_version = ~0ull;
}

}  // namespace

void ensure_subdomains(Context& c) {
    if (c.sub_mesh_version != c.mesh_version || c.sub_nodes_built != c.sub_nodes || c.sub_split_built != c.sub_split)
        build_split(c);
    if (c.sub_k_version == c.k_version) return;
    c.sub_factor.ensure(static_cast<size_t>(std::max<long long>(1, c.sub_factor_size)));
    c.scratch64.ensure(64);
    unsigned long long* counters = reinterpret_cast<unsigned long long*>(c.scratch64.p + 24);  // degenerate, inside
    LF_CUDA(cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned long long), c.stream));
    const int threads = std::max(32, (c.sub_max + 31) / 32 * 32);
    if (c.sub_count > 0)
        subdomain_factor_kernel<<<static_cast<unsigned>(c.sub_count), threads, 0, c.stream>>>(
            c.rowptr, c.col, c.K, c.sub_dofs, c.sub_begin, c.sub_owner, c.sub_local, c.sub_fac_begin, c.sub_factor,
            counters);
    subdomain_capture_kernel<<<grid_for(c.n, kCaptureThreads, 16 * c.num_sms), kCaptureThreads, 0, c.stream>>>(
        static_cast<int>(c.n), c.rowptr, c.col, c.sub_owner, counters + 1);
    c.launches += c.sub_count > 0 ? 2 : 1;
    LF_CUDA(cudaGetLastError());
    unsigned long long h[2] = {0, 0};
    LF_CUDA(cudaMemcpyAsync(h, counters, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
    check_status(c);
    c.sub_degenerate = static_cast<i64>(h[0]);
    c.sub_capture = c.nnz > 0 ? static_cast<double>(h[1]) / static_cast<double>(c.nnz) : 0.0;
    c.sub_k_version = c.k_version;
}

void ensure_subdomain_inverse(Context& c) {
    ensure_subdomains(c);
    if (c.sub_inv_version == c.k_version) return;
    c.sub_inv32.ensure(static_cast<size_t>(std::max<long long>(1, c.sub_sq_size)));
    if (c.sub_count > 0) {
        // FP64 scratch for the columns, released again: it is twice the factor's size.
        Buf<double> work;
        work.ensure(static_cast<size_t>(std::max<long long>(1, c.sub_sq_size)));
        const int threads = std::max(32, (c.sub_max + 31) / 32 * 32);
        subdomain_inverse_kernel<<<static_cast<unsigned>(c.sub_count), threads, 0, c.stream>>>(
            c.sub_begin, c.sub_fac_begin, c.sub_sq_begin, c.sub_factor, work, c.sub_inv32);
        c.launches += 1;
        LF_CUDA(cudaGetLastError());
        LF_CUDA(cudaStreamSynchronize(c.stream));
        work.release();
    }
    c.sub_inv_version = c.k_version;
}

}  // namespace lfgpu
