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

#include <algorithm>
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

// ------------------------------------------------------------------ RCM
// Reverse Cuthill-McKee (reverse_cuthill_mckee, src/reordering.cpp:11-62) on the
// device, equal to the reference's order.  The adjacency of node i is S(i) minus i
// (nodes sharing an element), each list sorted by (degree, index); seeds are taken
// in (degree, index) order.  The breadth-first search runs level by level in one
// CTA: every frontier node u (rank r in its level) offers each unvisited neighbour
// v at adjacency position p the key (r, p), v keeps the smallest key, and sorting
// the level by key reproduces the sequential queue order exactly (v is appended by
// the first frontier node that sees it, at its position in that node's list).
constexpr int kRcmThreads = 1024;
constexpr int kRcmMaxLevel = 4096;  // widest level the in-CTA sort takes

__global__ void rcm_degrees(int nn, const int* __restrict__ nptr, const int* __restrict__ list,
                            const int4* __restrict__ en, int* deg, int* flags) {
    int s[kMaxCand];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const int m = node_set(i, nptr, list, en, s);
        if (m < 0) atomicOr(flags, 1);  // too many elements at a node: the caller orders on the host
        deg[i] = m > 0 ? m - 1 : 0;
    }
}

__global__ void rcm_adjacency(int nn, const int* __restrict__ nptr, const int* __restrict__ list,
                              const int4* __restrict__ en, const int* __restrict__ deg,
                              const int* __restrict__ adj_ptr, int* adj) {
    int s[kMaxCand];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const int m = node_set(i, nptr, list, en, s);
        int* out = adj + adj_ptr[i];
        int k = 0;
        for (int t = 0; t < m; ++t) {  // insertion by (degree, index)
            const int v = s[t];
            if (v == i) continue;
            const int dv = deg[v];
            int p = k;
            while (p > 0 && (deg[out[p - 1]] > dv || (deg[out[p - 1]] == dv && out[p - 1] > v))) {
                out[p] = out[p - 1];
                --p;
            }
            out[p] = v;
            ++k;
        }
    }
}

__global__ void __launch_bounds__(kRcmThreads) rcm_bfs(int nn, const int* __restrict__ adj_ptr,
                                                       const int* __restrict__ adj, const int* __restrict__ deg,
                                                       unsigned long long* key, unsigned char* seen, int* front_a,
                                                       int* front_b, int* out, int* overflow) {
    extern __shared__ unsigned long long s_key[];  // kRcmMaxLevel keys, then kRcmMaxLevel node indices
    int* s_val = reinterpret_cast<int*>(s_key + kRcmMaxLevel);
    __shared__ unsigned long long s_best;
    __shared__ int s_count;
    const int tid = threadIdx.x;
    constexpr unsigned long long kNone = ~0ull;
    int total = 0;  // nodes placed so far (the same in every thread)
    int* front = front_a;
    int* next = front_b;
    while (true) {
        // next seed: the unvisited node of smallest (degree, index)
        if (tid == 0) s_best = kNone;
        __syncthreads();
        unsigned long long best = kNone;
        for (int i = tid; i < nn; i += kRcmThreads)
            if (!seen[i]) best = min(best, (static_cast<unsigned long long>(deg[i]) << 32) | static_cast<unsigned>(i));
        for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, o));
        if ((tid & 31) == 0) atomicMin(&s_best, best);
        __syncthreads();
        if (s_best == kNone) return;
        const int seed = static_cast<int>(s_best & 0xffffffffull);
        if (tid == 0) {
            seen[seed] = 1;
            front[0] = seed;
            out[total] = seed;
        }
        int width = 1;
        total += 1;
        __syncthreads();
        while (true) {
            if (tid == 0) s_count = 0;
            __syncthreads();
            for (int r = tid; r < width; r += kRcmThreads) {
                const int u = front[r];
                const int b = adj_ptr[u], e = adj_ptr[u + 1];
                for (int p = b; p < e; ++p) {
                    const int v = adj[p];
                    if (seen[v]) continue;
                    const unsigned long long k = (static_cast<unsigned long long>(r) << 32) | static_cast<unsigned>(p - b);
                    if (atomicMin(key + v, k) == kNone) {
                        const int slot = atomicAdd(&s_count, 1);
                        if (slot < kRcmMaxLevel) s_val[slot] = v;
                    }
                }
            }
            __syncthreads();
            const int m = s_count;
            if (m == 0) break;  // this component is done
            if (m > kRcmMaxLevel) {
                if (tid == 0) *overflow = 1;
                return;
            }
            int pw = 1;
            while (pw < m) pw <<= 1;
            for (int i = tid; i < pw; i += kRcmThreads) {
                if (i < m) {
                    s_key[i] = key[s_val[i]];
                } else {
                    s_key[i] = kNone;
                    s_val[i] = -1;
                }
            }
            __syncthreads();
            for (int k2 = 2; k2 <= pw; k2 <<= 1) {  // bitonic sort by key, ascending
                for (int j = k2 >> 1; j > 0; j >>= 1) {
                    for (int i = tid; i < pw; i += kRcmThreads) {
                        const int ixj = i ^ j;
                        if (ixj > i) {
                            const bool up = (i & k2) == 0;
                            if ((s_key[i] > s_key[ixj]) == up) {
                                const unsigned long long tk = s_key[i];
                                s_key[i] = s_key[ixj];
                                s_key[ixj] = tk;
                                const int tv = s_val[i];
                                s_val[i] = s_val[ixj];
                                s_val[ixj] = tv;
                            }
                        }
                    }
                    __syncthreads();
                }
            }
            for (int i = tid; i < m; i += kRcmThreads) {
                const int v = s_val[i];
                next[i] = v;
                out[total + i] = v;
                seen[v] = 1;
                key[v] = kNone;
            }
            __syncthreads();
            total += m;
            width = m;
            int* t = front;
            front = next;
            next = t;
        }
    }
}

// csr_profile (src/sparse.cpp:227-242) of the pattern this mesh produces, from the
// node sets alone: rows 2i and 2i+1 span columns 2 min S(i) .. 2 max S(i) + 1, a
// node in no element keeps only its diagonal.  out: [0] nonzeros, [1] bandwidth,
// [2] profile (64-bit sums), [3] nodes with too many elements (not counted).
__global__ void mesh_profile(int nn, const int* __restrict__ nptr, const int* __restrict__ list,
                             const int4* __restrict__ en, unsigned long long* out) {
    int s[kMaxCand];
    unsigned long long nz = 0, band = 0, prof = 0, bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        const int m = node_set(i, nptr, list, en, s);
        if (m < 0) {
            ++bad;
            continue;
        }
        if (m == 0) {
            nz += 2;
            continue;
        }
        const long long lo = 2LL * s[0], hi = 2LL * s[m - 1] + 1;
        for (int h = 0; h < 2; ++h) {
            const long long r = 2LL * i + h;
            nz += 2ULL * m;
            band = max(band, static_cast<unsigned long long>(max(r - lo, hi - r)));
            prof += static_cast<unsigned long long>(r - lo);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        nz += __shfl_xor_sync(0xffffffffu, nz, o);
        prof += __shfl_xor_sync(0xffffffffu, prof, o);
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
        band = max(band, __shfl_xor_sync(0xffffffffu, band, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out + 0, nz);
        atomicMax(out + 1, band);
        atomicAdd(out + 2, prof);
        atomicAdd(out + 3, bad);
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

bool mesh_profile_device(Context& c, long long out[3]) {
    const int nn = static_cast<int>(c.n_nodes);
    ensure_node_elements(c);
    Buf<unsigned long long> acc;
    acc.ensure(4);
    LF_CUDA(cudaMemsetAsync(acc.p, 0, 4 * sizeof(unsigned long long), c.stream));
    mesh_profile<<<grid_for(nn, kThreads, 16 * c.num_sms), kThreads, 0, c.stream>>>(nn, c.ne_ptr, c.ne_list,
                                                                                      c.elem_nodes, acc);
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
    unsigned long long h[4];
    LF_CUDA(cudaMemcpyAsync(h, acc.p, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
    LF_CUDA(cudaStreamSynchronize(c.stream));
    if (h[3] != 0) return false;
    out[0] = static_cast<long long>(h[0]);
    out[1] = static_cast<long long>(h[1]);
    out[2] = static_cast<long long>(h[2]);
    return true;
}

bool rcm_device(Context& c, std::vector<int>& order) {
    const int nn = static_cast<int>(c.n_nodes);
    ensure_node_elements(c);
    const int grid_n = grid_for(nn, kThreads, 16 * c.num_sms);
    Buf<int> deg, adj_ptr, adj, fa, fb, out, flags;
    Buf<unsigned long long> key;
    Buf<unsigned char> seen;
    Buf<long long> tmp;
    deg.ensure(static_cast<size_t>(nn) + 1);
    adj_ptr.ensure(static_cast<size_t>(nn) + 1);
    flags.ensure(1);
    LF_CUDA(cudaMemsetAsync(deg.p + nn, 0, sizeof(int), c.stream));
    LF_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(int), c.stream));
    rcm_degrees<<<grid_n, kThreads, 0, c.stream>>>(nn, c.ne_ptr, c.ne_list, c.elem_nodes, deg, flags);
    const long long total = exclusive_scan(c, deg, adj_ptr, nn + 1, tmp);  // synchronises
    int too_many = 0;
    LF_CUDA(cudaMemcpy(&too_many, flags.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (too_many) return false;
    adj.ensure(static_cast<size_t>(total) + 1);
    rcm_adjacency<<<grid_n, kThreads, 0, c.stream>>>(nn, c.ne_ptr, c.ne_list, c.elem_nodes, deg, adj_ptr, adj);
    key.ensure(static_cast<size_t>(nn));
    seen.ensure(static_cast<size_t>(nn));
    fa.ensure(kRcmMaxLevel);
    fb.ensure(kRcmMaxLevel);
    out.ensure(static_cast<size_t>(nn));
    LF_CUDA(cudaMemsetAsync(key.p, 0xFF, sizeof(unsigned long long) * nn, c.stream));
    LF_CUDA(cudaMemsetAsync(seen.p, 0, nn, c.stream));
    LF_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(int), c.stream));
    const int smem = kRcmMaxLevel * (8 + 4);
    LF_CUDA(cudaFuncSetAttribute(rcm_bfs, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    rcm_bfs<<<1, kRcmThreads, smem, c.stream>>>(nn, adj_ptr, adj, deg, key, seen, fa, fb, out, flags);
    c.launches += 3;
    LF_CUDA(cudaGetLastError());
    int overflow = 0;
    LF_CUDA(cudaMemcpyAsync(&overflow, flags.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    order.resize(static_cast<size_t>(nn));
    LF_CUDA(cudaMemcpyAsync(order.data(), out.p, sizeof(int) * nn, cudaMemcpyDeviceToHost, c.stream));
    LF_CUDA(cudaStreamSynchronize(c.stream));
    if (overflow) return false;
    std::reverse(order.begin(), order.end());
    return true;
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
