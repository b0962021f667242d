// CSR pattern and element->value map built on the device (build_csr_assembly_pattern
// + CsrMatrix::value_index, src/sparse.cpp:15-74), bit-identical to the reference's
// and to the host build in host_setup.cpp.
//
// A Q4 element couples both DOFs of each of its nodes, so rows 2i and 2i+1 share
// the column list {2j, 2j+1 : j in S(i)}, S(i) being the nodes that share an
// element with node i (i included); a node in no element keeps only its diagonal.
//
//   1. node -> element incidence (counts, exclusive scan, fill)
//   2. |S(i)| per node: gather the nodes of i's elements, sort, drop duplicates
//   3. row lengths -> row offsets (exclusive scan, 64-bit total checked)
//   4. columns: S(i) again, written to rows 2i and 2i+1
//   5. map: for each element entry (a, b), the position of column dof_b in row
//      dof_a (binary search in the sorted row)
//
// A node with more than kMaxNodeElems elements does not fit the per-thread
// candidate list; the build reports it and the caller uses the host build.
#include "common.cuh"
#include "kernels.hpp"

#include <vector>

namespace lfgpu {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxNodeElems = 16;
constexpr int kMaxCand = 4 * kMaxNodeElems;
constexpr int kScanBlock = 1024;

__global__ void count_node_elems(int ne, const int4* __restrict__ en, int* cnt) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        const int4 q = en[e];
        atomicAdd(cnt + q.x, 1);
        atomicAdd(cnt + q.y, 1);
        atomicAdd(cnt + q.z, 1);
        atomicAdd(cnt + q.w, 1);
    }
}

// Exclusive scan of `in` (n values) into `out`, in three passes: per-block scans
// with block totals, a scan of the totals, then the block offsets.
__global__ void __launch_bounds__(kScanBlock) scan_blocks(int n, const int* __restrict__ in, int* out,
                                                          long long* block_total) {
    __shared__ long long s_warp[kScanBlock / 32];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long v = i < n ? in[i] : 0;
    long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        long long w = lane < kScanBlock / 32 ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kScanBlock / 32) s_warp[lane] = w;
    }
    __syncthreads();
    const long long before = (warp > 0 ? s_warp[warp - 1] : 0) + x - v;
    if (i < n) out[i] = static_cast<int>(before);  // block-local; offsets added later
    if (threadIdx.x == kScanBlock - 1) block_total[blockIdx.x] = s_warp[kScanBlock / 32 - 1];
}

// One block: exclusive scan of the block totals in place, grand total at [nb].
__global__ void __launch_bounds__(kScanBlock) scan_totals(int nb, long long* total) {
    __shared__ long long s_carry;
    __shared__ long long s_v[kScanBlock];
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += kScanBlock) {  // nb is small: a plain shared-memory scan
        const int i = base + threadIdx.x;
        const long long v = i < nb ? total[i] : 0;
        s_v[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kScanBlock; o <<= 1) {
            const long long y = threadIdx.x >= o ? s_v[threadIdx.x - o] : 0;
            __syncthreads();
            s_v[threadIdx.x] += y;
            __syncthreads();
        }
        const long long carry = s_carry;
        if (i < nb) total[i] = carry + s_v[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) s_carry = carry + s_v[kScanBlock - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) total[nb] = s_carry;
}

__global__ void add_offsets(int n, int* out, const long long* __restrict__ offsets) {
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] = static_cast<int>(out[i] + offsets[blockIdx.x]);
}

__global__ void fill_node_elems(int ne, const int4* __restrict__ en, const int* __restrict__ nptr, int* fill,
                                int* list) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        const int4 q = en[e];
        list[nptr[q.x] + atomicAdd(fill + q.x, 1)] = e;
        list[nptr[q.y] + atomicAdd(fill + q.y, 1)] = e;
        list[nptr[q.z] + atomicAdd(fill + q.z, 1)] = e;
        list[nptr[q.w] + atomicAdd(fill + q.w, 1)] = e;
    }
}

// S(i) sorted and without duplicates in s[]; returns |S(i)|, or -1 if node i has
// more than kMaxNodeElems elements.
__device__ __forceinline__ int node_set(int i, const int* __restrict__ nptr, const int* __restrict__ list,
                                        const int4* __restrict__ en, int* s) {
    const int b = nptr[i], e = nptr[i + 1];
    if (e - b > kMaxNodeElems) return -1;
    int m = 0;
    for (int k = b; k < e; ++k) {
        const int4 q = en[list[k]];
        const int nd[4] = {q.x, q.y, q.z, q.w};
        for (int a = 0; a < 4; ++a) {  // insertion into the sorted prefix, skipping duplicates
            const int v = nd[a];
            int p = m;
            while (p > 0 && s[p - 1] > v) --p;
            if (p > 0 && s[p - 1] == v) continue;
            for (int t = m; t > p; --t) s[t] = s[t - 1];
            s[p] = v;
            ++m;
        }
    }
    return m;
}

__global__ void set_sizes(int nn, const int* __restrict__ nptr, const int* __restrict__ list,
                          const int4* __restrict__ en, int* rowlen, int* flags) {
    int s[kMaxCand];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const int m = node_set(i, nptr, list, en, s);
        if (m < 0) {
            atomicOr(flags, 1);  // too many elements at a node
            rowlen[2 * i] = rowlen[2 * i + 1] = 1;
            continue;
        }
        if (m == 0) atomicOr(flags, 2);  // isolated node: rows of length 1, pattern not paired
        const int len = m > 0 ? 2 * m : 1;
        rowlen[2 * i] = len;
        rowlen[2 * i + 1] = len;
    }
}

__global__ void fill_columns(int nn, const int* __restrict__ nptr, const int* __restrict__ list,
                             const int4* __restrict__ en, const int* __restrict__ rowptr, int* col) {
    int s[kMaxCand];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const int m = node_set(i, nptr, list, en, s);
        for (int half = 0; half < 2; ++half) {
            int* out = col + rowptr[2 * i + half];
            if (m <= 0) {
                out[0] = 2 * i + half;
                continue;
            }
            for (int k = 0; k < m; ++k) {
                out[2 * k] = 2 * s[k];
                out[2 * k + 1] = 2 * s[k] + 1;
            }
        }
    }
}

__global__ void fill_map(int ne, const int4* __restrict__ en, const int* __restrict__ rowptr,
                         const int* __restrict__ col, int* map) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        const int4 q = en[e];
        const int nd[4] = {q.x, q.y, q.z, q.w};
        int* out = map + 64LL * e;
        for (int a = 0; a < 4; ++a) {
            const int r0 = rowptr[2 * nd[a]], r1 = rowptr[2 * nd[a] + 1];
            const int len = r1 - r0;
            for (int b = 0; b < 4; ++b) {
                const int want = 2 * nd[b];
                int lo = 0, hi = len;  // first position with col >= want
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (col[r0 + mid] < want) lo = mid + 1;
                    else hi = mid;
                }
                for (int i = 0; i < 2; ++i) {
                    const int base = rowptr[2 * nd[a] + i] + lo;
                    out[(2 * a + i) * 8 + 2 * b] = base;
                    out[(2 * a + i) * 8 + 2 * b + 1] = base + 1;
                }
            }
        }
    }
}

// Each node's element list in ascending element order (insertion sort: a node has
// a handful of elements).
__global__ void sort_node_elems(int nn, const int* __restrict__ nptr, int* list) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const int b = nptr[i], e = nptr[i + 1];
        for (int k = b + 1; k < e; ++k) {
            const int v = list[k];
            int p = k;
            while (p > b && list[p - 1] > v) {
                list[p] = list[p - 1];
                --p;
            }
            list[p] = v;
        }
    }
}

// Exclusive scan of n ints on the stream; returns the total (synchronises).
long long exclusive_scan(Context& c, const int* in, int* out, int n, Buf<long long>& tmp) {
    const int nb = (n + kScanBlock - 1) / kScanBlock;
    tmp.ensure(static_cast<size_t>(nb) + 1);
    scan_blocks<<<nb, kScanBlock, 0, c.stream>>>(n, in, out, tmp);
    scan_totals<<<1, kScanBlock, 0, c.stream>>>(nb, tmp);
    add_offsets<<<nb, kScanBlock, 0, c.stream>>>(n, out, tmp);
    c.launches += 3;
    LF_CUDA(cudaGetLastError());
    long long total = 0;
    LF_CUDA(cudaMemcpyAsync(&total, tmp.p + nb, sizeof(total), cudaMemcpyDeviceToHost, c.stream));
    LF_CUDA(cudaStreamSynchronize(c.stream));
    return total;
}

}  // namespace

void ensure_node_elements(Context& c) {
    if (c.ne_version == c.mesh_version) return;
    const int nn = static_cast<int>(c.n_nodes), ne = static_cast<int>(c.n_elem);
    const int grid_e = grid_for(ne, kThreads, 16 * c.num_sms), grid_n = grid_for(nn, kThreads, 16 * c.num_sms);
    Buf<int> cnt, fill;
    Buf<long long> tmp;
    cnt.ensure(static_cast<size_t>(nn) + 1);
    fill.ensure(static_cast<size_t>(nn) + 1);
    c.ne_ptr.ensure(static_cast<size_t>(nn) + 1);
    c.ne_list.ensure(4 * static_cast<size_t>(ne) + 1);
    LF_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * (nn + 1), c.stream));
    LF_CUDA(cudaMemsetAsync(fill.p, 0, sizeof(int) * (nn + 1), c.stream));
    if (ne > 0) count_node_elems<<<grid_e, kThreads, 0, c.stream>>>(ne, c.elem_nodes, cnt);
    exclusive_scan(c, cnt, c.ne_ptr, nn + 1, tmp);
    if (ne > 0) fill_node_elems<<<grid_e, kThreads, 0, c.stream>>>(ne, c.elem_nodes, c.ne_ptr, fill, c.ne_list);
    sort_node_elems<<<grid_n, kThreads, 0, c.stream>>>(nn, c.ne_ptr, c.ne_list);
    c.launches += 3;
    LF_CUDA(cudaGetLastError());
    c.ne_version = c.mesh_version;
}

bool build_pattern_device(Context& c, std::vector<int>& rowptr_host) {
    const int nn = static_cast<int>(c.n_nodes), ne = static_cast<int>(c.n_elem);
    LF_REQUIRE(c.n_nodes < (1LL << 29) && c.n_elem < (1LL << 29), LFGPU_ERR_ARGUMENT, "mesh too large");
    const int n = 2 * nn;
    const int grid_e = grid_for(ne, kThreads, 16 * c.num_sms), grid_n = grid_for(nn, kThreads, 16 * c.num_sms);
    Buf<int> cnt, nptr, fill, list, rowlen, flags;
    Buf<long long> tmp;
    cnt.ensure(static_cast<size_t>(nn) + 1);
    nptr.ensure(static_cast<size_t>(nn) + 1);
    fill.ensure(static_cast<size_t>(nn) + 1);
    list.ensure(4 * static_cast<size_t>(ne) + 1);
    rowlen.ensure(static_cast<size_t>(n) + 1);
    flags.ensure(1);
    LF_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * (nn + 1), c.stream));
    LF_CUDA(cudaMemsetAsync(fill.p, 0, sizeof(int) * (nn + 1), c.stream));
    LF_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(int), c.stream));
    LF_CUDA(cudaMemsetAsync(rowlen.p + n, 0, sizeof(int), c.stream));  // the scan's last input
    if (ne > 0) count_node_elems<<<grid_e, kThreads, 0, c.stream>>>(ne, c.elem_nodes, cnt);
    exclusive_scan(c, cnt, nptr, nn + 1, tmp);  // nptr[nn] = 4 E
    if (ne > 0) fill_node_elems<<<grid_e, kThreads, 0, c.stream>>>(ne, c.elem_nodes, nptr, fill, list);
    set_sizes<<<grid_n, kThreads, 0, c.stream>>>(nn, nptr, list, c.elem_nodes, rowlen, flags);
    c.launches += 3;
    LF_CUDA(cudaGetLastError());
    int h_flags = 0;
    LF_CUDA(cudaMemcpyAsync(&h_flags, flags.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    LF_CUDA(cudaStreamSynchronize(c.stream));
    if (h_flags & 1) return false;  // a node with too many elements: host build
    c.rowptr.ensure(static_cast<size_t>(n) + 1);
    const long long nnz = exclusive_scan(c, rowlen, c.rowptr, n + 1, tmp);  // rowptr[n] = nnz
    LF_REQUIRE(nnz < (1LL << 31), LFGPU_ERR_ARGUMENT, "pattern must have fewer than 2^31 nonzeros");
    c.col.ensure(static_cast<size_t>(nnz));
    c.map.ensure(64 * static_cast<size_t>(ne) + 1);
    fill_columns<<<grid_n, kThreads, 0, c.stream>>>(nn, nptr, list, c.elem_nodes, c.rowptr, c.col);
    if (ne > 0) fill_map<<<grid_e, kThreads, 0, c.stream>>>(ne, c.elem_nodes, c.rowptr, c.col, c.map);
    c.launches += 2;
    LF_CUDA(cudaGetLastError());
    rowptr_host.resize(static_cast<size_t>(n) + 1);
    LF_CUDA(cudaMemcpyAsync(rowptr_host.data(), c.rowptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, c.stream));
    LF_CUDA(cudaStreamSynchronize(c.stream));
    c.n = n;
    c.nnz = nnz;
    c.paired = (h_flags & 2) == 0;
    return true;
}

}  // namespace lfgpu
