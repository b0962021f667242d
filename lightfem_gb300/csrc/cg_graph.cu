// Preconditioned CG as a device-driven CUDA graph.
//
// Same recurrences as the persistent kernel in pcg.cu (pcg_solve,
// src/solver.cpp:532-627, in FP64; the FP32-inner / FP64-refinement scheme in
// mixed precision), but every phase is its own kernel at full occupancy and the
// loop runs inside one CUDA graph without host round trips:
//
//   init -> WHILE(loop) { product ; update ; [FP64: p update]
//                         [mixed: IF(refine) { FP64 residual ; re-precondition }] }
//
// The WHILE and IF bodies are graph conditional nodes; their conditions are set
// from the device (cudaGraphSetConditional) by the block that finishes each
// reduction.  Scalars (rho, alpha, beta, norms, counters) live in a device
// CgState.  Dot products are reduced deterministically: every block publishes
// its partial, and the last block to arrive adds them in a fixed order.  The
// mixed loop's direct form has no last block in its product: every CTA of the
// update that follows adds the product's partials itself, in that same order.
//
// Products: a quarter warp per CSR row or per BSR block row, several entries or
// blocks in flight per lane (FP64 BSR: a whole 2x2 block per lane as two 16-byte
// loads, fused multiply-adds only; FP32 BSR: one 16-byte block per lane).  The
// FP32 products stream 16-bit column offsets from the row when they fit.  Matrix
// loads carry the evict-first hint so the vectors stay in L2.
//
// The subdomain block-Jacobi preconditioner is applied by its own kernels: the
// FP64 loop runs its block solves between the update and the r.z reduction (as
// IC(0) runs its sweeps), the mixed loop applies FP32 block inverses after each
// iteration's IF node.
#include "common.cuh"
#include "kernels.hpp"

#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

namespace lfgpu {
namespace {

constexpr int kThreads = 256;
constexpr int kTimedPasses = 5000;  // profiling runs up to this long time every launch

struct CgState {
    double rho, alpha, beta, r0, rnorm, rmax, rtrue, rtrue_prev;
    long long it, refs;
    int status, converged, stagnated, done, no_progress, refine;
    unsigned int count[4];
    // FP32 copies for the mixed loop, set where alpha and beta are, so that no
    // thread of the loop kernels converts them (GB300's FP64 pipe is narrow):
    // alpha = alpha32 + alpha32_lo to about 44 bits (pair_quotient).
    float alpha32, alpha32_lo, beta32, pad32;
    // Raised by the last CTA of mx_update_staged once beta is set; the other CTAs
    // wait for it before they form the next direction (only equality with the
    // value a CTA saw at its start matters, so it may wrap).
    unsigned int go, pad_go;
    // The values last written to the graph's conditional handles (the WHILE loop's
    // and each body iteration's IF), so that a kernel writes one only when it
    // changes: cudaGraphSetConditional costs a noticeable part of a microsecond.
    // 0: not written yet in this solve, 1: false, 2: true.
    int loop_val, branch_val[8];
};

struct CgArgs {
    int n, nb;
    const int* rowptr;
    const int* col;
    const double* K;
    const float* K32;
    const int* brow;
    const int* bcol;
    const short* bcol16;           // FP32 BSR: columns as offsets from the block row, or nullptr
    const short* col16;            // FP32 CSR: columns as offsets from the row, or nullptr
    const double2* bval64;
    const float4* bval32;
    const float* dhi;
    const float* dlo;
    const double* invd64;
    const double* blk64;
    const float* invd32;
    const float* blk32;
    const double* f;
    const double* x0;
    double* x;
    double* r;
    double* z;
    double* p;
    double* q;
    double* r64;
    float* r32;
    float* p32;
    float* q32;
    float2* zp0;                   // (z, p) per DOF, two alternating copies
    float2* zp1;
    float* xhi;                    // FP32 pair of the solution correction
    float* xlo;
    double* partials;  // 4 slots x blocks x 4
    const int* diag;               // IC(0): diagonal position of every row
    const double* icf;             // IC(0) factor on the pattern of K (ic0.cu)
    const double* icinv;           // IC(0) reciprocal pivots
    double* y;                     // IC(0) forward-sweep result
    unsigned long long* ic_chunks; // IC(0) row-chunk counters (forward, backward)
    const int* sub_dofs;           // subdomain block-Jacobi: DOFs by subdomain
    const int* sub_begin;
    const long long* sub_fac;      // packed lower factor offset of each subdomain
    const double* sub_factor;
    const float* sub_inv32;        // mixed loop: block inverses, FP32 D x D squares
    const long long* sub_sq;       // offset of each subdomain's square
    // IC(0) level-scheduled sweeps (ic0.cu builds the schedules): [0] forward, [1] backward
    struct SweepPlan {
        const int* level_begin;    // 2 per level + 2: first position, first entry
        const int4* pieces;        // per level and CTA, two int4: first and end position, first and end
                                   // entry; the width of level L - 1 + kSweepRingBars (-1: none)
        const int4* desc;          // per position: row, first entry, end entry, output index
        const int* dep;            // per entry: position of the row it depends on
        const void* val;           // factor entries in schedule order (double or float)
        const void* inv;           // reciprocal pivots in schedule order
        int levels;
    } sw[2];
    int staged_stash;              // mx_update_staged: nodes per CTA whose (z, p) stay in shared memory
    int product_grid;              // CTAs of mx_product (the direct form's update adds their p.q pairs)
    int sw_window;                 // ring slots per CTA (a power of two)
    int sw_maxp, sw_maxe;          // the largest piece: positions, entries (the stage size)
    void* sw_y;                    // forward result in backward positions (double or float)
    void* sw_rhs;                  // r in forward positions (double or float)
    float* sw_rr;                  // mixed: r32 in backward positions (the backward sweep's r.z)
    int blocks;
    CgState* st;
    DeviceStatus* status;
    double target, reduction;
    long long maxit, max_ref;
    int restart;
    int paired;    // CSR storage with a paired pattern: the mixed loop's FP32 copy is the BSR blocks
    int use_cond;  // 0 in the unrolled profiling graph, which has no conditional nodes
    int half;      // the body iteration (0 .. 7) whose IF handle `branch` is
    cudaGraphConditionalHandle loop, branch;
};

// A handle keeps its value from one evaluation to the next.  Every solve starts
// from a zeroed CgState, so the first call of each solve writes the handle.
__device__ __forceinline__ void set_loop(const CgArgs& a, bool go) {
    const int want = go ? 2 : 1;
    if (a.use_cond && a.st->loop_val != want) {
        cudaGraphSetConditional(a.loop, go ? 1u : 0u);
        a.st->loop_val = want;
    }
}
__device__ __forceinline__ void set_branch(const CgArgs& a, bool go) {
    const int want = go ? 2 : 1;
    if (a.use_cond && a.st->branch_val[a.half] != want) {
        cudaGraphSetConditional(a.branch, go ? 1u : 0u);
        a.st->branch_val[a.half] = want;
    }
}

// Block sums of K values, then the last block to finish adds every block's sums in
// block order and runs fin(totals) on thread 0.  Returns true in the last block.
template <int K, typename Final>
__device__ __forceinline__ bool reduce_tail(const CgArgs& a, int slot, double (&v)[K], double* s_red, Final&& fin) {
    __shared__ int s_last;
    double* part = a.partials + static_cast<size_t>(slot) * a.blocks * kMaxReduce;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) part[blockIdx.x * kMaxReduce + k] = v[k];
        unsigned t;  // arrive with release semantics: the partials above are visible first
        asm volatile("atom.add.release.gpu.global.u32 %0, [%1], 1;" : "=r"(t) : "l"(&a.st->count[slot]) : "memory");
        s_last = t == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
    for (int b = threadIdx.x; b < static_cast<int>(gridDim.x); b += blockDim.x) {
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] += __ldcg(part + b * kMaxReduce + k);
    }
    block_sum<K>(acc, s_red);
    if (threadIdx.x == 0) {
        a.st->count[slot] = 0;
        fin(acc);
    }
    return true;
}

// FP64 per-thread values: FP64 warp and block sums.
template <int K, typename Final>
__device__ __forceinline__ bool reduce_last(const CgArgs& a, int slot, double (&v)[K], Final&& fin) {
    __shared__ double s_red[32 * kMaxReduce];
    block_sum<K>(v, s_red);
    return reduce_tail<K>(a, slot, v, s_red, fin);
}

// An unevaluated FP32 pair (hi + lo) for the dot products of the FP32 loop: each
// addition is Knuth's two-sum, so the pair carries about 48 bits.  This keeps
// the dot products near FP64 accuracy with FP32 arithmetic only -- FP64 shuffles
// and adds in every thread would keep GB300's narrow FP64 pipe busy for several
// microseconds per reduction.
struct FloatPair {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float s = __fadd_rn(hi, x);
        const float bp = __fsub_rn(s, hi);
        const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
        lo = __fadd_rn(lo, e);
        hi = s;
    }
    __device__ __forceinline__ void add(const FloatPair& o) {
        add(o.hi);
        lo = __fadd_rn(lo, o.lo);
    }
};

// FP32-pair per-thread values summed over the CTA (the mixed inner loop): warp
// sums as pairs, then the warps' pairs in warp 0, whose threads all get the CTA's
// totals as pairs in w (the other threads' w is zero).  FP32 arithmetic only: on
// GB300 a dependent FP64 add takes about as long as a dozen FP32 ones.
// NT > 0: only the CTA's first NT threads take part, synchronised on named barrier 1.
template <int NT>
__device__ __forceinline__ void pair_reduce_sync() {
    if constexpr (NT == 0)
        __syncthreads();
    else
        asm volatile("bar.sync 1, %0;" ::"n"(NT) : "memory");
}

template <int K, int NT = 0>
__device__ __forceinline__ void block_pair_reduce(FloatPair (&v)[K], FloatPair (&w)[K]) {
    __shared__ float2 s_warp[32 * kMaxReduce];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            FloatPair other;
            other.hi = __shfl_xor_sync(0xffffffffu, v[k].hi, o);
            other.lo = __shfl_xor_sync(0xffffffffu, v[k].lo, o);
            v[k].add(other);
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) s_warp[warp * K + k] = make_float2(v[k].hi, v[k].lo);
    }
    pair_reduce_sync<NT>();
#pragma unroll
    for (int k = 0; k < K; ++k) w[k] = FloatPair{};
    if (warp == 0) {
        const int nw = (NT == 0 ? static_cast<int>(blockDim.x) : NT) >> 5;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (lane < nw) {
                const float2 t = s_warp[lane * K + k];
                w[k].hi = t.x;
                w[k].lo = t.y;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                FloatPair other;
                other.hi = __shfl_xor_sync(0xffffffffu, w[k].hi, o);
                other.lo = __shfl_xor_sync(0xffffffffu, w[k].lo, o);
                w[k].add(other);
            }
        }
    }
    pair_reduce_sync<NT>();  // s_warp is free again
}

// The grid-wide step for FP32-pair values: each CTA leaves its pair totals, and
// the last CTA to arrive adds all CTAs' pairs, in a fixed assignment to its threads
// and a fixed shuffle tree (deterministic), then runs fin on the FP64 values
// hi + lo.  Pairs instead of FP64 partials keep the last CTA's tail, which the
// rest of the iteration waits for, off GB300's slow FP64 adds.  Returns true in
// the last CTA.
template <int K, typename Final>
__device__ __forceinline__ bool reduce_tail_pair(const CgArgs& a, int slot, const FloatPair (&w)[K], Final&& fin) {
    __shared__ int s_last;
    float2* part = reinterpret_cast<float2*>(a.partials + static_cast<size_t>(slot) * a.blocks * kMaxReduce);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) part[blockIdx.x * kMaxReduce + k] = make_float2(w[k].hi, w[k].lo);
        unsigned t;  // arrive with release semantics: the partials above are visible first
        asm volatile("atom.add.release.gpu.global.u32 %0, [%1], 1;" : "=r"(t) : "l"(&a.st->count[slot]) : "memory");
        s_last = t == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    FloatPair acc[K];
    for (int b = threadIdx.x; b < static_cast<int>(gridDim.x); b += blockDim.x) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float2 t = __ldcg(part + b * kMaxReduce + k);
            acc[k].add(FloatPair{t.x, t.y});
        }
    }
    FloatPair tot[K];
    block_pair_reduce<K>(acc, tot);
    if (threadIdx.x == 0) {
        double d[K];
#pragma unroll
        for (int k = 0; k < K; ++k) d[k] = static_cast<double>(tot[k].hi) + static_cast<double>(tot[k].lo);
        a.st->count[slot] = 0;
        fin(d);
    }
    return true;
}

// FP32-pair per-thread values: pair sums within the CTA, then across the grid.
template <int K, typename Final>
__device__ __forceinline__ bool reduce_last(const CgArgs& a, int slot, FloatPair (&v)[K], Final&& fin) {
    FloatPair w[K];
    block_pair_reduce<K>(v, w);
    return reduce_tail_pair<K>(a, slot, w, fin);
}

// Warp-uniform loop over row groups of 8 (quarter warp per row) across the grid.
template <typename F>
__device__ __forceinline__ void rows_by_quad(int rows, F&& f) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int base = warp * 8; base < rows; base += nwarps * 8) {
        const int row = base + (lane >> 2);
        f(row < rows, row, lane & 3);
    }
}

__device__ __forceinline__ double quad_sum(double v) {
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    return v + __shfl_xor_sync(0xffffffffu, v, 2);
}
__device__ __forceinline__ float quad_sum(float v) {
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    return v + __shfl_xor_sync(0xffffffffu, v, 2);
}

// y = K x in FP64 for CSR rows; out(row, y) on the quad leader.
template <typename G, typename Out>
__device__ __forceinline__ void csr64_rows(const CgArgs& a, const G& g, Out&& out) {
    rows_by_quad(a.n, [&](bool act, int row, int sub) {
        double s = 0.0;
        if (act) {
            const int b = __ldg(a.rowptr + row), e = __ldg(a.rowptr + row + 1);
            for (int k = b + sub; k < e; k += 8) {  // two independent units in flight per lane
                const bool two = k + 4 < e;
                const int c0 = ld_stream(a.col + k), c1 = two ? ld_stream(a.col + k + 4) : c0;
                const double v0 = ld_stream(a.K + k), v1 = two ? ld_stream(a.K + k + 4) : 0.0;
                const double x0 = g(c0), x1 = g(c1);
                s += v0 * x0;
                s += v1 * x1;
            }
        }
        s = quad_sum(s);
        if (act && sub == 0) out(row, s);
    });
}

// y = K x in FP64 for BSR block rows: lane pairs read the two 16-byte halves of a
// block; even lanes sum the top row, odd lanes the bottom row.
template <typename G, typename Out>
__device__ __forceinline__ void bsr64_rows(const CgArgs& a, const G& g, Out&& out) {
    // A quarter warp per block row, whole 2x2 blocks per lane (two 16-byte
    // loads), three blocks in flight per lane: the nine blocks of an interior
    // node in one round.  Fused multiply-adds only: GB300's FP64 pipe is the bound.
    rows_by_quad(a.nb, [&](bool act, int node, int sub) {
        double s0 = 0.0, s1 = 0.0;
        if (act) {
            const int b = __ldg(a.brow + node), e = __ldg(a.brow + node + 1);
            for (int k = b + sub; k < e; k += 12) {
                const bool t1 = k + 4 < e, t2 = k + 8 < e;
                const double2 zero = make_double2(0.0, 0.0);
                const int c0 = ld_stream(a.bcol + k);
                const int c1 = t1 ? ld_stream(a.bcol + k + 4) : c0;
                const int c2 = t2 ? ld_stream(a.bcol + k + 8) : c0;
                const double2 u0 = ld_stream(a.bval64 + 2 * static_cast<size_t>(k));
                const double2 w0 = ld_stream(a.bval64 + 2 * static_cast<size_t>(k) + 1);
                const double2 u1 = t1 ? ld_stream(a.bval64 + 2 * static_cast<size_t>(k + 4)) : zero;
                const double2 w1 = t1 ? ld_stream(a.bval64 + 2 * static_cast<size_t>(k + 4) + 1) : zero;
                const double2 u2 = t2 ? ld_stream(a.bval64 + 2 * static_cast<size_t>(k + 8)) : zero;
                const double2 w2 = t2 ? ld_stream(a.bval64 + 2 * static_cast<size_t>(k + 8) + 1) : zero;
                const double2 x0 = g(c0), x1 = g(c1), x2 = g(c2);
                s0 = fma(u0.x, x0.x, s0);
                s0 = fma(u0.y, x0.y, s0);
                s1 = fma(w0.x, x0.x, s1);
                s1 = fma(w0.y, x0.y, s1);
                s0 = fma(u1.x, x1.x, s0);
                s0 = fma(u1.y, x1.y, s0);
                s1 = fma(w1.x, x1.x, s1);
                s1 = fma(w1.y, x1.y, s1);
                s0 = fma(u2.x, x2.x, s0);
                s0 = fma(u2.y, x2.y, s0);
                s1 = fma(w2.x, x2.x, s1);
                s1 = fma(w2.y, x2.y, s1);
            }
        }
        s0 = quad_sum(s0);
        s1 = quad_sum(s1);
        if (act && sub == 0) out(node, make_double2(s0, s1));
    });
}

// FP32 BSR block rows, quarter warp per block row (one 16-byte block per lane).
// Each lane keeps three blocks in flight (k, k+4, k+8), so the nine blocks of an
// interior node's row cost one round of gather latency instead of three.  The
// grid-stride loop loads the next row's block offsets while this row's blocks
// stream, which takes one dependent load off each row's chain.
template <typename G, typename Out>
__device__ __forceinline__ void bsr32_rows(const CgArgs& a, const G& g, Out&& out) {
    const int lane = threadIdx.x & 31, sub = lane & 3;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int stride = ((gridDim.x * blockDim.x) >> 5) * 8;
    int node = warp * 8 + (lane >> 2);
    int nb_b = 0, nb_e = 0;
    if (node < a.nb) {
        nb_b = __ldg(a.brow + node);
        nb_e = __ldg(a.brow + node + 1);
    }
    for (int base = warp * 8; base < a.nb; base += stride, node += stride) {  // warp-uniform
        const bool act = node < a.nb;
        const int b = nb_b, e = nb_e;
        if (node + stride < a.nb) {
            nb_b = __ldg(a.brow + node + stride);
            nb_e = __ldg(a.brow + node + stride + 1);
        }
        float s0 = 0.f, s1 = 0.f;
        if (act) {
            // Columns as 16-bit offsets from the block row when they fit (half the bytes).
            auto col = [&](int k) { return a.bcol16 ? node + ld_stream(a.bcol16 + k) : ld_stream(a.bcol + k); };
            for (int k = b + sub; k < e; k += 12) {
                const bool t1 = k + 4 < e, t2 = k + 8 < e;
                const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
                const int c0 = col(k);
                const int c1 = t1 ? col(k + 4) : c0;
                const int c2 = t2 ? col(k + 8) : c0;
                const float4 v0 = ld_stream(a.bval32 + k);
                const float4 v1 = t1 ? ld_stream(a.bval32 + k + 4) : zero;
                const float4 v2 = t2 ? ld_stream(a.bval32 + k + 8) : zero;
                const float2 x0 = g(c0), x1 = g(c1), x2 = g(c2);
                s0 += v0.x * x0.x + v0.y * x0.y;
                s1 += v0.z * x0.x + v0.w * x0.y;
                s0 += v1.x * x1.x + v1.y * x1.y;
                s1 += v1.z * x1.x + v1.w * x1.y;
                s0 += v2.x * x2.x + v2.y * x2.y;
                s1 += v2.z * x2.x + v2.w * x2.y;
            }
        }
        s0 = quad_sum(s0);
        s1 = quad_sum(s1);
        if (act && sub == 0) out(node, make_float2(s0, s1));
    }
}

// FP32 CSR rows, quarter warp per row; five entries in flight per lane cover the
// eighteen entries of an interior row in one round.
template <typename G, typename Out>
__device__ __forceinline__ void csr32_rows(const CgArgs& a, const G& g, Out&& out) {
    rows_by_quad(a.n, [&](bool act, int row, int sub) {
        float s = 0.f;
        if (act) {
            const int b = __ldg(a.rowptr + row), e = __ldg(a.rowptr + row + 1);
            for (int k = b + sub; k < e; k += 20) {
                int c[5];
                float v[5];
#pragma unroll
                for (int j = 0; j < 5; ++j) {
                    const bool on = k + 4 * j < e;
                    const int kk = on ? k + 4 * j : k;
                    // Columns as 16-bit offsets from the row when they fit (half the bytes).
                    c[j] = a.col16 ? row + ld_stream(a.col16 + kk) : ld_stream(a.col + kk);
                    v[j] = on ? ld_stream(a.K32 + k + 4 * j) : 0.f;
                }
                float x[5];
#pragma unroll
                for (int j = 0; j < 5; ++j) x[j] = g(c[j]);
#pragma unroll
                for (int j = 0; j < 5; ++j) s += v[j] * x[j];
            }
        }
        s = quad_sum(s);
        if (act && sub == 0) out(row, s);
    });
}

__device__ __forceinline__ double2 block2_apply(const double* __restrict__ blk, int i, double r0, double r1) {
    const double f0 = blk[3 * i], f1 = blk[3 * i + 1], f2 = blk[3 * i + 2];
    double s0 = __dmul_rn(r0, f0);
    double s1 = __dmul_rn(__dsub_rn(r1, __dmul_rn(f1, s0)), f2);
    s1 = __dmul_rn(s1, f2);
    s0 = __dmul_rn(__dsub_rn(s0, __dmul_rn(f1, s1)), f0);
    return make_double2(s0, s1);
}

__device__ __forceinline__ float2 block2_apply32(const float* __restrict__ blk, int i, float r0, float r1) {
    const float f0 = blk[3 * i], f1 = blk[3 * i + 1], f2 = blk[3 * i + 2];
    float s0 = r0 * f0;
    float s1 = (r1 - f1 * s0) * f2;
    s1 = s1 * f2;
    s0 = (s0 - f1 * s1) * f0;
    return make_float2(s0, s1);
}

template <int PRECOND>
__device__ __forceinline__ double2 precond64(const CgArgs& a, int i, double2 rv) {
    if (PRECOND == LFGPU_PRECOND_JACOBI) {
        const double2 d = reinterpret_cast<const double2*>(a.invd64)[i];
        return make_double2(d.x * rv.x, d.y * rv.y);
    }
    return block2_apply(a.blk64, i, rv.x, rv.y);
}

// z of node i from the preconditioner's values pc (Jacobi: the inverse diagonal,
// two floats a node; 2x2 blocks: the factor, three floats a node), wherever they are.
template <int PRECOND>
__device__ __forceinline__ float2 precond32_at(const float* pc, int i, float2 rv) {
    if (PRECOND == LFGPU_PRECOND_JACOBI) {
        const float2 d = reinterpret_cast<const float2*>(pc)[i];
        return make_float2(d.x * rv.x, d.y * rv.y);
    }
    return block2_apply32(pc, i, rv.x, rv.y);
}

template <int PRECOND>
__device__ __forceinline__ float2 precond32(const CgArgs& a, int i, float2 rv) {
    return precond32_at<PRECOND>(PRECOND == LFGPU_PRECOND_JACOBI ? a.invd32 : a.blk32, i, rv);
}

#define GRID_NODES(i) for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nb; i += gridDim.x * blockDim.x)

// ------------------------------------------------------------------ FP64 kernels
// r = f - K x0 for a warm start.
template <int STORAGE>
__global__ void __launch_bounds__(kThreads) cg64_residual(CgArgs a) {
    if (STORAGE == LFGPU_STORAGE_CSR) {
        csr64_rows(a, [&](int c) { return a.x0[c]; }, [&](int row, double y) { a.r[row] = a.f[row] - y; });
    } else {
        const double2* x02 = reinterpret_cast<const double2*>(a.x0);
        bsr64_rows(a, [&](int c) { return x02[c]; }, [&](int node, double2 y) {
            a.r[2 * node] = a.f[2 * node] - y.x;
            a.r[2 * node + 1] = a.f[2 * node + 1] - y.y;
        });
    }
}

template <int PRECOND>
__global__ void __launch_bounds__(kThreads) cg64_init(CgArgs a) {
    double v[2] = {0.0, 0.0};
    double2* x2 = reinterpret_cast<double2*>(a.x);
    double2* r2 = reinterpret_cast<double2*>(a.r);
    double2* z2 = reinterpret_cast<double2*>(a.z);
    double2* p2 = reinterpret_cast<double2*>(a.p);
    const double2* f2 = reinterpret_cast<const double2*>(a.f);
    GRID_NODES(i) {
        const double2 rv = a.x0 ? r2[i] : f2[i];
        const double2 zv = precond64<PRECOND>(a, i, rv);
        r2[i] = rv;
        z2[i] = zv;
        p2[i] = zv;
        x2[i] = a.x0 ? reinterpret_cast<const double2*>(a.x0)[i] : make_double2(0.0, 0.0);
        v[0] += rv.x * rv.x + rv.y * rv.y;
        v[1] += rv.x * zv.x + rv.y * zv.y;
    }
    reduce_last<2>(a, 0, v, [&](const double* t) {
        CgState* s = a.st;
        s->r0 = s->rnorm = sqrt(fmax(0.0, t[0]));
        s->rho = t[1];
        s->it = 0;
        if (s->r0 <= a.target) {
            s->converged = 1;
            s->done = 1;
        } else if (!(t[1] > 0.0) || !isfinite(t[1])) {
            s->status = LFGPU_ERR_RHO_INITIAL;
            s->done = 1;
        }
        set_loop(a, !s->done);
    });
}

template <int STORAGE>
__global__ void __launch_bounds__(kThreads) cg64_product(CgArgs a) {
    if (a.st->done) return;
    double v[1] = {0.0};
    if (STORAGE == LFGPU_STORAGE_CSR) {
        csr64_rows(a, [&](int c) { return a.p[c]; }, [&](int row, double y) {
            a.q[row] = y;
            v[0] += a.p[row] * y;
        });
    } else {
        const double2* p2 = reinterpret_cast<const double2*>(a.p);
        bsr64_rows(a, [&](int c) { return p2[c]; }, [&](int node, double2 y) {
            reinterpret_cast<double2*>(a.q)[node] = y;
            const double2 pv = p2[node];
            v[0] += pv.x * y.x + pv.y * y.y;
        });
    }
    reduce_last<1>(a, 1, v, [&](const double* t) {
        CgState* s = a.st;
        if (!(t[0] > 0.0) || !isfinite(t[0])) {
            s->status = LFGPU_ERR_NOT_SPD;
            s->done = 1;
            set_loop(a, false);
        } else {
            s->alpha = s->rho / t[0];
        }
    });
}

template <int PRECOND>
__global__ void __launch_bounds__(kThreads) cg64_update(CgArgs a) {
    if (a.st->done) return;
    const double alpha = a.st->alpha;
    double v[2] = {0.0, 0.0};
    double2* x2 = reinterpret_cast<double2*>(a.x);
    double2* r2 = reinterpret_cast<double2*>(a.r);
    double2* z2 = reinterpret_cast<double2*>(a.z);
    const double2* p2 = reinterpret_cast<const double2*>(a.p);
    const double2* q2 = reinterpret_cast<const double2*>(a.q);
    GRID_NODES(i) {
        const double2 pv = p2[i], qv = q2[i];
        double2 xv = x2[i], rv = r2[i];
        xv.x += alpha * pv.x;
        xv.y += alpha * pv.y;
        rv.x -= alpha * qv.x;
        rv.y -= alpha * qv.y;
        const double2 zv = precond64<PRECOND>(a, i, rv);
        x2[i] = xv;
        r2[i] = rv;
        z2[i] = zv;
        v[0] += rv.x * rv.x + rv.y * rv.y;
        v[1] += rv.x * zv.x + rv.y * zv.y;
    }
    reduce_last<2>(a, 2, v, [&](const double* t) {
        CgState* s = a.st;
        s->it += 1;
        s->rnorm = sqrt(fmax(0.0, t[0]));
        if (s->rnorm <= a.target) {
            s->converged = 1;
            s->done = 1;
        } else if (!(t[1] > 0.0) || !isfinite(t[1])) {
            s->status = LFGPU_ERR_RHO;
            s->done = 1;
        } else {
            s->beta = t[1] / s->rho;
            s->rho = t[1];
            if (s->it >= a.maxit) s->done = 1;
        }
        set_loop(a, !s->done);
    });
}

__global__ void __launch_bounds__(kThreads) cg64_direction(CgArgs a) {
    if (a.st->done) return;
    const double beta = a.st->beta;
    double2* p2 = reinterpret_cast<double2*>(a.p);
    const double2* z2 = reinterpret_cast<const double2*>(a.z);
    GRID_NODES(i) {
        const double2 zv = z2[i];
        double2 pv = p2[i];
        pv.x = zv.x + beta * pv.x;
        pv.y = zv.y + beta * pv.y;
        p2[i] = pv;
    }
}

// ------------------------------------------------------------------ mixed kernels
// FP32 vectors of the inner solve.  In the direct form (see kDirectMinNodes) p is
// a plain vector that mx_update_staged rewrites.  Otherwise z and p are
// interleaved per DOF, (z_c, p_c), so the product gathers both with one 16-byte
// load per node and forms p; two copies alternate between iterations (the product
// reads one, the update writes the other).  The solution correction since the
// last residual replacement is kept as an unevaluated FP32 pair (hi + lo, about
// 48 significant bits) and added to the FP64 solution when a replacement is due,
// so no FP64 arithmetic runs per iteration.
__device__ __forceinline__ float pnew(float z, float p, float beta) { return __fmaf_rn(beta, p, z); }
__device__ __forceinline__ float with_diag(float off, float hi, float lo, float x) { return fmaf(hi, x, off) + lo * x; }

__device__ __forceinline__ float4* zp_buffer(const CgArgs& a, long long it) {
    return reinterpret_cast<float4*>((it & 1) ? a.zp1 : a.zp0);
}

// (hi, lo) += (ah + al) * p with error-free transformations (Knuth's two-sum,
// the fma two-product), then renormalised so |lo| <= ulp(hi) / 2.  The _rn
// intrinsics keep the compiler from fusing the steps the error terms rely on.
__device__ __forceinline__ void pair_axpy(float& hi, float& lo, float ah, float al, float p) {
    const float prod = __fmul_rn(ah, p);
    const float perr = __fmaf_rn(al, p, __fmaf_rn(ah, p, -prod));
    const float s = __fadd_rn(hi, prod);
    const float bp = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(prod, bp));
    const float l = __fadd_rn(lo, __fadd_rn(err, perr));
    hi = __fadd_rn(s, l);
    lo = __fsub_rn(l, __fsub_rn(hi, s));
}

// num / den as an unevaluated FP32 pair (hi + lo, about 44 bits; Dekker's
// division): one FP32 quotient, its remainder from an error-free product, and a
// correction.  The loop's scalars (alpha, beta) come from this instead of an FP64
// division, whose dependent steps take a large part of a microsecond on GB300
// and hold up every CTA waiting for them.
__device__ __forceinline__ void pair_quotient(double num, double den, float& hi, float& lo) {
    const float nh = static_cast<float>(num), nl = static_cast<float>(num - static_cast<double>(nh));
    const float dh = static_cast<float>(den), dl = static_cast<float>(den - static_cast<double>(dh));
    const float q1 = __fdiv_rn(nh, dh);
    const float p = __fmul_rn(q1, dh);
    const float pe = __fmaf_rn(q1, dh, -p);  // q1 * dh = p + pe exactly
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(nh, p), pe), __fsub_rn(nl, __fmul_rn(q1, dl)));
    const float q2 = __fdiv_rn(r, dh);
    hi = __fadd_rn(q1, q2);
    lo = __fsub_rn(q2, __fsub_rn(hi, q1));
}

// Preconditioners applied by their own kernels (the subdomain block solves,
// mx_sub_apply; the IC(0) sweeps, ic0_level_sweep) run after mx_init and after
// every mx_update: those two leave z and r.z to them.
template <int PRECOND>
constexpr bool applied_separately() {
    return PRECOND == LFGPU_PRECOND_SUBDOMAIN || PRECOND == LFGPU_PRECOND_IC0;
}

// DIRECT form, with the pointwise preconditioners (Jacobi, 2x2 nodal blocks) on
// meshes of kDirectMinNodes nodes or more: the update (mx_update_staged) also
// forms the next direction.  Its CTAs, all resident (a cooperative launch), wait
// for the last one to set beta and then rewrite p = z + beta p for their own
// nodes.  The product then gathers p alone, 8 bytes a node instead of the
// (z, p_old) pair's 16, and writes no p.  p is the same fma of the same values as
// when the product forms it, once per node instead of once per gather.  The wait
// costs a few microseconds whatever the size, the saving grows with it, and the
// direct form's update also forms alpha, so its product has no last-CTA tail.
// Per iteration of the mixed BSR/Jacobi solve on GB300 (n x n plane-strain
// cantilevers, RCM), direct against (z, p_old) form, one box: 400x400 (160,801
// nodes) 22.92 against 25.23 us; 500x500 (251,001) 26.20 against 29.17.  (Before
// the update formed alpha: 27.05 against 26.93 at 400x400, 47.69 against 50.66
// at 800x800.)  Smaller meshes keep the (z, p_old) form until measured.  The
// separately applied preconditioners keep it too: their z arrives after mx_update.
constexpr long long kDirectMinNodes = 150000;

bool direct_form(int precond, long long nodes) {
    return (precond == LFGPU_PRECOND_JACOBI || precond == LFGPU_PRECOND_BLOCK2) && nodes >= kDirectMinNodes;
}

template <int PRECOND, bool DIRECT>
__global__ void __launch_bounds__(kThreads) mx_init(CgArgs a) {
    constexpr bool kSub = applied_separately<PRECOND>();
    static_assert(!(DIRECT && kSub), "the direct form needs a pointwise preconditioner");
    double v[2] = {0.0, 0.0};
    const double2* f2 = reinterpret_cast<const double2*>(a.f);
    float4* zp = reinterpret_cast<float4*>(a.zp0);
    float2* p2 = reinterpret_cast<float2*>(a.p32);
    GRID_NODES(i) {
        const double2 fv = f2[i];
        const float2 rv = make_float2(static_cast<float>(fv.x), static_cast<float>(fv.y));
        float2 zv = make_float2(0.f, 0.f);
        if constexpr (!kSub) zv = precond32<PRECOND>(a, i, rv);
        reinterpret_cast<double2*>(a.x)[i] = make_double2(0.0, 0.0);
        reinterpret_cast<float2*>(a.xhi)[i] = make_float2(0.f, 0.f);
        reinterpret_cast<float2*>(a.xlo)[i] = make_float2(0.f, 0.f);
        reinterpret_cast<double2*>(a.r64)[i] = fv;
        reinterpret_cast<float2*>(a.r32)[i] = rv;
        if constexpr (DIRECT)
            p2[i] = make_float2(pnew(zv.x, 0.f, 0.f), pnew(zv.y, 0.f, 0.f));  // beta = 0, p_old = 0
        else
            zp[i] = make_float4(zv.x, 0.f, zv.y, 0.f);
        v[0] += fv.x * fv.x + fv.y * fv.y;
        v[1] += static_cast<double>(rv.x * zv.x + rv.y * zv.y);
    }
    reduce_last<2>(a, 0, v, [&](const double* t) {
        CgState* s = a.st;
        s->r0 = s->rnorm = s->rmax = s->rtrue = s->rtrue_prev = sqrt(fmax(0.0, t[0]));
        s->rho = t[1];
        s->beta = 0.0;
        s->beta32 = 0.f;
        s->it = 0;
        s->refs = 0;
        if (s->r0 <= a.target) {
            s->converged = 1;
            s->done = 1;
        } else if (!kSub && (!(t[1] > 0.0) || !isfinite(t[1]))) {
            s->status = LFGPU_ERR_RHO_INITIAL;
            s->done = 1;
        }
        set_loop(a, !s->done);
    });
}

// q = K32 p and p.q.  DIRECT: p as mx_update_staged left it, gathered alone, and
// each CTA only leaves its p.q pair: the update's CTAs form alpha from them, so no
// CTA of the product waits at the end for a last one's sum and division.
// Otherwise p = z + beta p_old is formed on the fly from the (z, p_old) pairs, each
// row writes its p, and the last CTA sets alpha.  The FP32 copy of K is the BSR
// blocks for BSR storage and for a paired CSR pattern (a.paired), FP32 CSR rows
// otherwise.
template <int STORAGE, bool DIRECT>
__global__ void __launch_bounds__(kThreads, 8) mx_product(CgArgs a) {  // 8 CTAs an SM: the grid in one wave
    if (a.st->done) return;
    const float beta = a.st->beta32;
    const float4* zp4 = zp_buffer(a, a.st->it);
    FloatPair acc;
    // Gathers and row results per node (a 2x2 block row).
    const float2* hi2 = reinterpret_cast<const float2*>(a.dhi);
    const float2* lo2 = reinterpret_cast<const float2*>(a.dlo);
    const float2* p2 = reinterpret_cast<const float2*>(a.p32);
    auto gather_node = [&](int c) {
        if constexpr (DIRECT) {
            return p2[c];
        } else {
            const float4 v = zp4[c];
            return make_float2(pnew(v.x, v.y, beta), pnew(v.z, v.w, beta));
        }
    };
    auto finish_node = [&](int node, float2 off) {
        float2 pn;
        if constexpr (DIRECT) {
            pn = p2[node];
        } else {
            const float4 v = zp4[node];
            pn = make_float2(pnew(v.x, v.y, beta), pnew(v.z, v.w, beta));
            reinterpret_cast<float2*>(a.p32)[node] = pn;
        }
        const float2 h = hi2[node], l = lo2[node];
        const float2 y = make_float2(with_diag(off.x, h.x, l.x, pn.x), with_diag(off.y, h.y, l.y, pn.y));
        reinterpret_cast<float2*>(a.q32)[node] = y;
        acc.add(pn.x * y.x + pn.y * y.y);
    };
    if (STORAGE == LFGPU_STORAGE_CSR && !a.paired) {
        const float2* zp2 = reinterpret_cast<const float2*>(zp4);
        const float* p = a.p32;
        csr32_rows(a,
                   [&](int c) {
                       if constexpr (DIRECT) {
                           return p[c];
                       } else {
                           const float2 v = zp2[c];
                           return pnew(v.x, v.y, beta);
                       }
                   },
                   [&](int row, float off) {
                       float pn;
                       if constexpr (DIRECT) {
                           pn = p[row];
                       } else {
                           const float2 v = zp2[row];
                           pn = pnew(v.x, v.y, beta);
                           a.p32[row] = pn;
                       }
                       const float y = with_diag(off, a.dhi[row], a.dlo[row], pn);
                       a.q32[row] = y;
                       acc.add(pn * y);
                   });
    } else {
        bsr32_rows(a, gather_node, finish_node);
    }
    FloatPair v[1] = {acc};
    if constexpr (DIRECT) {
        // Each CTA leaves its p.q pair; every CTA of mx_update_staged adds them for alpha.
        FloatPair w[1];
        block_pair_reduce<1>(v, w);
        if (threadIdx.x == 0)
            reinterpret_cast<float2*>(a.partials + static_cast<size_t>(a.blocks) * kMaxReduce)[blockIdx.x * kMaxReduce] =
                make_float2(w[0].hi, w[0].lo);
        return;
    }
    reduce_last<1>(a, 1, v, [&](const double* t) {
        CgState* s = a.st;
        if (!(t[0] > 0.0) || !isfinite(t[0])) {
            s->status = LFGPU_ERR_NOT_SPD;
            s->done = 1;
            set_loop(a, false);
        } else {
            pair_quotient(s->rho, t[0], s->alpha32, s->alpha32_lo);
            s->alpha = static_cast<double>(s->alpha32) + static_cast<double>(s->alpha32_lo);
        }
    });
}

__device__ __forceinline__ unsigned ld_acquire_gpu_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// The last CTA's step of the mixed update: iteration count, inner residual, the
// replacement test, and (unless the preconditioner is applied separately) beta.
template <bool SUB>
__device__ __forceinline__ void update_totals(const CgArgs& a, const double* t) {
    CgState* s = a.st;
    s->it += 1;
    // The inner residual norm only decides when to replace the residual: FP32 is
    // enough, and an FP64 square root would hold up the grid.
    const double rn = static_cast<double>(__fsqrt_rn(static_cast<float>(fmax(0.0, t[0]))));
    s->rnorm = rn;
    s->rmax = fmax(s->rmax, rn);
    const bool refine = rn <= a.reduction * s->rmax || rn <= a.target || s->it >= a.maxit;
    s->refine = refine;
    if (!refine && !SUB) {
        if (!(t[1] > 0.0) || !isfinite(t[1])) {
            s->status = LFGPU_ERR_RHO;
            s->done = 1;
        } else {
            float lo;
            pair_quotient(t[1], s->rho, s->beta32, lo);
            s->beta = static_cast<double>(s->beta32) + static_cast<double>(lo);
            s->rho = t[1];
        }
    }
    set_branch(a, refine && !s->done);
    set_loop(a, !s->done);
}

// The direct form's grid-wide wait for beta (bounded), after update_totals ran in
// the last CTA: true when the CTA goes on to form the direction.  A CTA whose wait
// runs out ends the solve.  go0: CgState::go as the CTA found it at its start.
__device__ __forceinline__ bool wait_for_beta(const CgArgs& a, bool last, unsigned go0) {
    __shared__ int s_go;
    if (threadIdx.x == 0) {
        int ok = 1;
        if (last) {
            asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&a.st->go) : "memory");
        } else {
            // The wait lasts about one pass of the update; each poll is an L2
            // round trip, so the limit is checked on every one.
            const unsigned long long t0 = global_ns();
            while (ld_acquire_gpu_u32(&a.st->go) == go0) {
                if (wait_expired(a.status, t0, static_cast<int>(blockIdx.x))) {
                    ok = 0;
                    break;
                }
            }
        }
        if (!ok) {
            a.st->done = 1;
            set_branch(a, false);
            set_loop(a, false);
        }
        s_go = ok && !__ldcg(&a.st->done) && !__ldcg(&a.st->refine);
    }
    __syncthreads();
    return s_go != 0;
}

// x += alpha p (into the FP32 pair), r -= alpha q, z = M^-1 r; r.r and r.z.  The
// (z, p_old) form: z goes into the pair copy the next product reads (the direct
// form's update is mx_update_staged).
template <int PRECOND>
__global__ void __launch_bounds__(kThreads) mx_update(CgArgs a) {
    constexpr bool kSub = applied_separately<PRECOND>();
    if (a.st->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0) set_branch(a, false);
        return;
    }
    const float alpha = a.st->alpha32, alpha_lo = a.st->alpha32_lo;
    const float2* p2 = reinterpret_cast<const float2*>(a.p32);
    const float2* q2 = reinterpret_cast<const float2*>(a.q32);
    float2* r2 = reinterpret_cast<float2*>(a.r32);
    float2* hi2 = reinterpret_cast<float2*>(a.xhi);
    float2* lo2 = reinterpret_cast<float2*>(a.xlo);
    float4* zp_next = zp_buffer(a, a.st->it + 1);
    FloatPair rr, rz;
    GRID_NODES(i) {
        const float2 pv = p2[i], qv = q2[i];
        float2 hv = hi2[i], lv = lo2[i];
        float2 rv = r2[i];
        pair_axpy(hv.x, lv.x, alpha, alpha_lo, pv.x);
        pair_axpy(hv.y, lv.y, alpha, alpha_lo, pv.y);
        rv.x -= alpha * qv.x;
        rv.y -= alpha * qv.y;
        float2 zv = make_float2(0.f, 0.f);
        if constexpr (!kSub) zv = precond32<PRECOND>(a, i, rv);
        hi2[i] = hv;
        lo2[i] = lv;
        r2[i] = rv;
        zp_next[i] = make_float4(zv.x, pv.x, zv.y, pv.y);
        rr.add(rv.x * rv.x + rv.y * rv.y);
        if constexpr (!kSub) rz.add(rv.x * zv.x + rv.y * zv.y);
    }
    FloatPair v[2] = {rr, rz};
    reduce_last<2>(a, 2, v, [&](const double* t) { update_totals<kSub>(a, t); });
}

// After a residual replacement with a pointwise preconditioner: p = z + beta p, with
// the z and beta of mx_reprecondition.
__global__ void __launch_bounds__(kThreads) mx_direction(CgArgs a) {
    if (a.st->done || !a.st->refine) return;
    const float beta = a.st->beta32;
    const float2* z2 = reinterpret_cast<const float2*>(a.zp0);
    float2* pw = reinterpret_cast<float2*>(a.p32);
    GRID_NODES(i) {
        const float2 zv = z2[i], pv = pw[i];
        pw[i] = make_float2(pnew(zv.x, pv.x, beta), pnew(zv.y, pv.y, beta));
    }
}

// x64 += hi + lo, then hi = lo = 0 (hi + lo is exact in FP64).  Inside the loop it
// runs only when a replacement is due; after the loop, always.
template <bool ALWAYS>
__global__ void __launch_bounds__(kThreads) mx_flush(CgArgs a) {
    if (!ALWAYS && (a.st->done || !a.st->refine)) return;
    double2* x2 = reinterpret_cast<double2*>(a.x);
    float2* hi2 = reinterpret_cast<float2*>(a.xhi);
    float2* lo2 = reinterpret_cast<float2*>(a.xlo);
    GRID_NODES(i) {
        const float2 hv = hi2[i], lv = lo2[i];
        double2 xv = x2[i];
        xv.x += static_cast<double>(hv.x) + static_cast<double>(lv.x);
        xv.y += static_cast<double>(hv.y) + static_cast<double>(lv.y);
        x2[i] = xv;
        hi2[i] = make_float2(0.f, 0.f);
        lo2[i] = make_float2(0.f, 0.f);
    }
}

// FP64 residual replacement: r64 = f - K64 x, r32 = r64.
template <int STORAGE>
__global__ void __launch_bounds__(kThreads) mx_residual(CgArgs a) {
    if (a.st->done || !a.st->refine) return;  // only reachable this way in the unrolled graph
    double v[1] = {0.0};
    if (STORAGE == LFGPU_STORAGE_CSR) {
        csr64_rows(a, [&](int c) { return a.x[c]; }, [&](int row, double y) {
            const double rv = a.f[row] - y;
            a.r64[row] = rv;
            a.r32[row] = static_cast<float>(rv);
            v[0] += rv * rv;
        });
    } else {
        const double2* x2 = reinterpret_cast<const double2*>(a.x);
        bsr64_rows(a, [&](int c) { return x2[c]; }, [&](int node, double2 y) {
            const double2 fv = reinterpret_cast<const double2*>(a.f)[node];
            const double2 rv = make_double2(fv.x - y.x, fv.y - y.y);
            reinterpret_cast<double2*>(a.r64)[node] = rv;
            reinterpret_cast<float2*>(a.r32)[node] = make_float2(static_cast<float>(rv.x), static_cast<float>(rv.y));
            v[0] += rv.x * rv.x + rv.y * rv.y;
        });
    }
    reduce_last<1>(a, 3, v, [&](const double* t) {
        CgState* s = a.st;
        s->refs += 1;
        const double rt = sqrt(fmax(0.0, t[0]));
        s->rtrue = rt;
        if (rt <= a.target) {
            s->converged = 1;
            s->done = 1;
        } else if (s->refs >= a.max_ref || s->it >= a.maxit) {
            s->done = 1;
        } else {
            s->no_progress = rt >= s->rtrue_prev ? s->no_progress + 1 : 0;
            if (s->no_progress >= 3) {
                s->stagnated = 1;
                s->done = 1;
            }
            s->rtrue_prev = fmin(s->rtrue_prev, rt);
            s->rmax = rt;
        }
        set_loop(a, !s->done);
    });
}

// z = M^-1 r32 after a residual replacement, and beta.  The next direction is
// formed by the product from the (z, p_old) pairs, or (DIRECT) by mx_direction
// from z, kept in the first half of zp0.
template <int PRECOND, bool DIRECT>
__global__ void __launch_bounds__(kThreads) mx_reprecondition(CgArgs a) {
    if (a.st->done || !a.st->refine) return;
    const float2* r2 = reinterpret_cast<const float2*>(a.r32);
    float4* zp = zp_buffer(a, a.st->it);  // the copy the next product reads
    FloatPair rz;
    GRID_NODES(i) {
        const float2 rv = r2[i];
        const float2 zv = precond32<PRECOND>(a, i, rv);
        if constexpr (DIRECT) {
            reinterpret_cast<float2*>(a.zp0)[i] = zv;
        } else {
            float4 t = zp[i];
            t.x = zv.x;
            t.z = zv.y;
            zp[i] = t;
        }
        rz.add(rv.x * zv.x + rv.y * zv.y);
    }
    FloatPair v[1] = {rz};
    reduce_last<1>(a, 2, v, [&](const double* t) {
        CgState* s = a.st;
        if (!(t[0] > 0.0) || !isfinite(t[0])) {
            s->status = LFGPU_ERR_RHO;
            s->done = 1;
        } else {
            s->beta = a.restart ? 0.0 : t[0] / s->rho;
            s->beta32 = static_cast<float>(s->beta);
            s->rho = t[0];
        }
        set_loop(a, !s->done);
    });
}

// ------------------------------------------------------------------ IC(0) sweeps
// z = (L L^T)^-1 r with the factor of ic0.cu (IncompleteCholesky0::apply,
// src/precond.cpp:386-412):
//   forward   y(r) = (r(r) - sum_{c<r} L(r,c) y(c)) / L(r,r), rows ascending;
//   backward  z(c) = (y(c) - sum_{r>c} L(r,c) z(r)) / L(c,c), rows descending.
// Each term is subtracted in the reference's order -- columns ascending forward;
// rows descending backward, the order in which the reference's column scatter
// reaches z(c) -- without contraction, so z equals the reference's bit for bit.
//
// No level schedule: CTAs take 256-row chunks in sweep order from a counter, one
// thread per row.  A value not yet written holds the kPending pattern, and a
// thread polls (bounded) until its operand appears: in shared memory when the
// operand's row is in the same chunk, else in global memory at GPU scope.  Chunks
// are taken in dependency order, so the oldest unfinished row can always proceed.
constexpr int kSweepRows = 1024;  // rows per chunk, one CTA thread per row
constexpr unsigned long long kPending = ~0ull;  // a NaN pattern marking "not written yet"

// A result that happens to carry the kPending pattern is stored as the default NaN.
__device__ __forceinline__ unsigned long long publishable(double v) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    return b == kPending ? 0x7FF8000000000000ull : b;
}

// Bounded polls; on abort or expiry they return the kPending NaN, which poisons
// the sweep, and the next dot product stops the solve (the status records why).
__device__ __forceinline__ double poll_global(const double* p, DeviceStatus* status, int row) {
    const unsigned long long* q = reinterpret_cast<const unsigned long long*>(p);
    unsigned long long v = ld_relaxed_gpu(q);
    if (v == kPending) {
        const unsigned long long t0 = global_ns();
        for (unsigned it = 1; (v = ld_relaxed_gpu(q)) == kPending; ++it)
            if ((it & 63u) == 0u && wait_expired(status, t0, row)) break;
    }
    return __longlong_as_double(static_cast<long long>(v));
}

__device__ __forceinline__ double poll_shared(const volatile unsigned long long* p, DeviceStatus* status, int row) {
    unsigned long long v = *p;
    if (v == kPending) {
        const unsigned long long t0 = global_ns();
        for (unsigned it = 1; (v = *p) == kPending; ++it) {
            // Back off: the producer of the operand is often a lane of this same
            // warp, which only runs while this lane's path yields.
            __nanosleep(32);
            if ((it & 1023u) == 0u && wait_expired(status, t0, row)) break;
        }
    }
    return __longlong_as_double(static_cast<long long>(v));
}

// One CTA per chunk of kSweepRows consecutive rows.  The critical path of a sweep
// crosses chunks only at some of its levels: inside a chunk an operand is a
// shared-memory poll away, across chunks an L2 round trip, so larger chunks
// shorten the path (1024 rows: 14 % faster than 256 on the 200x200 workload).
// Giving a thread several rows of a chunk, in order, is much slower: a row then
// also waits for the thread's earlier rows, which can sit many levels later.
__global__ void __launch_bounds__(kSweepRows) ic0_forward(CgArgs a) {
    if (a.st->done) return;
    __shared__ unsigned long long s_v[kSweepRows];
    __shared__ int s_chunk;
    if (threadIdx.x == 0) s_chunk = static_cast<int>(atomicAdd(a.ic_chunks + 0, 1ull));
    s_v[threadIdx.x] = kPending;
    __syncthreads();
    const int r0 = s_chunk * kSweepRows, row = r0 + static_cast<int>(threadIdx.x);
    if (row >= a.n) return;
    const int b = a.rowptr[row], d = a.diag[row];
    double sum = a.r[row];
    for (int k = b; k < d; ++k) {
        const int c = ld_stream(a.col + k);
        const double v = c >= r0 ? poll_shared(s_v + (c - r0), a.status, row) : poll_global(a.y + c, a.status, row);
        sum = __dsub_rn(sum, __dmul_rn(ld_stream(a.icf + k), v));
    }
    const unsigned long long out = publishable(__dmul_rn(sum, a.icinv[row]));
    reinterpret_cast<volatile unsigned long long*>(s_v)[threadIdx.x] = out;
    st_relaxed_gpu(reinterpret_cast<unsigned long long*>(a.y + row), out);
}

__global__ void __launch_bounds__(kSweepRows) ic0_backward(CgArgs a) {
    if (a.st->done) return;
    __shared__ unsigned long long s_v[kSweepRows];
    __shared__ int s_chunk;
    if (threadIdx.x == 0) s_chunk = static_cast<int>(atomicAdd(a.ic_chunks + 1, 1ull));
    s_v[threadIdx.x] = kPending;
    __syncthreads();
    const int top = a.n - 1 - s_chunk * kSweepRows, row = top - static_cast<int>(threadIdx.x);
    if (row < 0) return;
    const int d = a.diag[row];
    double sum = a.y[row];
    for (int k = a.rowptr[row + 1] - 1; k > d; --k) {
        const int c = ld_stream(a.col + k);
        const double v = c <= top ? poll_shared(s_v + (top - c), a.status, row) : poll_global(a.z + c, a.status, row);
        sum = __dsub_rn(sum, __dmul_rn(ld_stream(a.icf + k), v));
    }
    const unsigned long long out = publishable(__dmul_rn(sum, a.icinv[row]));
    reinterpret_cast<volatile unsigned long long*>(s_v)[threadIdx.x] = out;
    st_relaxed_gpu(reinterpret_cast<unsigned long long*>(a.z + row), out);
}

// ------------------------------------------------------------------ IC(0) level sweeps
// The same two sweeps, scheduled by levels instead of polls: a row's level is one
// more than the deepest row it depends on, so the rows of one level are
// independent.  One cluster of kSweepCluster CTAs walks the levels in order; each
// level's rows are split into one contiguous piece per CTA, one consumer thread
// per row.
//
// Operands arrive by TMA.  The schedule stores each level's rows, entries,
// pivots and right-hand sides contiguously, so a producer warp per CTA copies the
// CTA's piece of a level (row descriptors, entry positions and values, reciprocal
// pivots, right-hand sides) into one of kSweepStages shared-memory stages with
// cp.async.bulk, up to kSweepStages levels ahead; the consumers find their
// operands in shared memory when the level starts.
//
// Results travel through shared memory, not L2: every CTA keeps a ring of the last
// sw_window results (slot = schedule position mod sw_window), and a consumer that
// finishes a row stores its result into every CTA's ring with st.async, which
// also counts the bytes on that CTA's mbarrier of the level.  A CTA starts level L
// once its mbarrier of level L - 1 has seen the whole level (width x size bytes),
// so no cluster-wide barrier runs per level.  CTAs run at most one level apart, so
// the ring spans the longest dependency distance plus two levels
// (ensure_ic0_schedule checks it), and kSweepRingBars mbarriers cycle over the
// levels; the consumer warps of a CTA meet once per level.  Waits are bounded: on
// expiry the kernel records LFGPU_ERR_TIMEOUT and ends the solve.
//
// The arithmetic of a row is the polled sweeps': terms subtracted in the
// reference's order, products and differences rounded separately, so the FP64
// sweeps equal the reference's application bit for bit.  MODE 0 / 1: FP64 forward
// (r -> y in backward order) / backward (-> z); MODE 2 / 3: the mixed loop's FP32
// forward (r32) / backward, which writes z into the (z, p) copy the next product
// reads and reduces r.z (rho and beta, as the subdomain application does).  The
// forward sweep reads r in schedule order (ic0_sweep_inputs gathers it first), the
// backward sweep the forward result, which the forward sweep writes in backward
// order.
constexpr int kSweepUnroll = 12;                // entries of a row whose products are formed together
constexpr int kSweepConsumers = kSweepThreads;   // one row per consumer thread and pass
constexpr int kSweepBlock = kSweepThreads + 32;  // plus the producer warp

__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Address of the same shared-memory variable in CTA `rank` of the cluster.
__device__ __forceinline__ unsigned cluster_address(unsigned addr, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
__device__ __forceinline__ void store_remote(unsigned addr, double v, unsigned bar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.f64 [%0], %1, [%2];" ::"r"(addr), "d"(v),
                 "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void store_remote(unsigned addr, float v, unsigned bar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.f32 [%0], %1, [%2];" ::"r"(addr), "f"(v),
                 "r"(bar)
                 : "memory");
}
__device__ __forceinline__ bool phase_done(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for an mbarrier phase; false when it ran out (or another wait did).
__device__ __forceinline__ bool wait_phase(unsigned long long* bar, unsigned parity, DeviceStatus* status, int level) {
    if (phase_done(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned it = 1;; ++it) {
        if (phase_done(bar, parity)) return true;
        if ((it & 15u) == 0u && wait_expired(status, t0, level)) return false;
    }
}
__device__ __forceinline__ void arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// The consumer warps' own barrier (the producer warp does not take part).
__device__ __forceinline__ void consumers_sync() {
    asm volatile("bar.sync 1, %0;" ::"n"(kSweepConsumers) : "memory");
}

// A row's terms: each product rounded on its own, then subtracted in order.  The
// products do not depend on one another, so they are formed together and only the
// subtractions form the row's dependency chain.
__device__ __forceinline__ double sweep_mul(double l, double v) { return __dmul_rn(l, v); }
__device__ __forceinline__ float sweep_mul(float l, float v) { return __fmul_rn(l, v); }
__device__ __forceinline__ double sweep_sub(double acc, double t) { return __dsub_rn(acc, t); }
__device__ __forceinline__ float sweep_sub(float acc, float t) { return __fsub_rn(acc, t); }

// rho and beta from r.z after a separate preconditioner application (the mixed
// loop's subdomain and IC(0) forms): the first rho after mx_init, then beta =
// r.z / rho, or 0 after a residual replacement in restart mode.
__device__ __forceinline__ void rho_from_application(const CgArgs& a, const double* t) {
    CgState* st = a.st;
    const bool first = st->it == 0;
    if (!(t[0] > 0.0) || !isfinite(t[0])) {
        st->status = first ? LFGPU_ERR_RHO_INITIAL : LFGPU_ERR_RHO;
        st->done = 1;
    } else if (first || (a.restart && st->refine)) {
        st->beta = 0.0;
        st->beta32 = 0.f;
        st->rho = t[0];
    } else {
        float lo;
        pair_quotient(t[0], st->rho, st->beta32, lo);
        st->beta = static_cast<double>(st->beta32) + static_cast<double>(lo);
        st->rho = t[0];
    }
    set_loop(a, !st->done);
}

// Elements of type E that a copy from the 16-byte boundary at or below index i
// carries in front of element i (the array base is 16-byte aligned).
template <typename E>
__device__ __forceinline__ int lead_of(int i) {
    return i & (16 / static_cast<int>(sizeof(E)) - 1);
}

// r gathered into the forward schedule's order (and, for the mixed backward
// sweep's r.z, into the backward schedule's), before the forward sweep.
template <bool MIXED>
__global__ void __launch_bounds__(kThreads) ic0_sweep_inputs(CgArgs a) {
    if (a.st->done) return;
    const int4* __restrict__ fd = a.sw[0].desc;
    const int4* __restrict__ bd = a.sw[1].desc;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        if (MIXED) {
            static_cast<float*>(a.sw_rhs)[p] = a.r32[fd[p].x];
            a.sw_rr[p] = a.r32[bd[p].x];
        } else {
            static_cast<double*>(a.sw_rhs)[p] = a.r[fd[p].x];
        }
    }
}

template <int MODE>
__global__ void __cluster_dims__(kSweepCluster, 1, 1) __launch_bounds__(kSweepBlock) ic0_level_sweep(CgArgs a) {
    using T = typename std::conditional<(MODE < 2), double, float>::type;
    constexpr bool kFwd = (MODE & 1) == 0;
    constexpr int S = kSweepStages;
    constexpr int SR = kSweepRingBars;
    if (a.st->done) return;  // read before the kernel changes anything: the same in every CTA
    extern __shared__ __align__(128) unsigned char sweep_smem[];
    __shared__ __align__(8) unsigned long long full[S], empty[S], ringbar[SR];
    __shared__ int4 piece_of[S];
    __shared__ int rearm_of[S];
    __shared__ int s_failed, s_issued;
    const CgArgs::SweepPlan& sp = a.sw[kFwd ? 0 : 1];
    const int levels = sp.levels;
    const int mask = a.sw_window - 1;
    const unsigned rank = cluster_rank();
    const int tid = threadIdx.x;
    T* ring = reinterpret_cast<T*>(sweep_smem);
    unsigned char* stages = sweep_smem + sweep_round16(a.sw_window * static_cast<int>(sizeof(T)));
    const SweepStageLayout lay = sweep_stage_layout(static_cast<int>(sizeof(T)), a.sw_maxp, a.sw_maxe);
    auto width_bytes = [&](int L) {
        return static_cast<unsigned>(__ldg(sp.level_begin + 2 * L + 2) - __ldg(sp.level_begin + 2 * L)) *
               static_cast<unsigned>(sizeof(T));
    };
    if (tid == 0) {
        s_failed = 0;
        s_issued = 0;
        for (int s = 0; s < S; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        for (int s = 0; s < SR; ++s) mbar_init(ringbar + s, 1);
        mbar_init_fence();
        for (int L = 0; L < SR && L < levels; ++L) mbar_expect_tx(ringbar + L, width_bytes(L));
    }
    cluster_sync_all();  // every CTA's mbarriers are armed before any copy or result arrives
    bool ok = true;
    FloatPair rz;  // the mixed backward sweep's r.z (zero on the producer warp)
    if (tid >= kSweepConsumers) {
        // ---- producer warp: one lane copies each level's piece into its stage.  The
        // warp reads the piece table 32 levels at a time (lane i: level base + i),
        // one batch ahead, so no copy waits on a table load.
        const int lane = tid & 31;
        const unsigned long long policy = l2_evict_first_policy();
        const T* rhs_src = static_cast<const T*>(kFwd ? a.sw_rhs : a.sw_y);
        const int4 none = make_int4(0, 0, 0, 0);
        auto batch = [&](int base, int4& pc, int& rearm) {
            const int L = base + lane;
            pc = none;
            rearm = -1;
            if (L < levels) {
                const int4* e = sp.pieces + 2 * (static_cast<size_t>(L) * kSweepCluster + rank);
                pc = __ldg(e);
                rearm = __ldg(e + 1).x;
            }
        };
        int4 cur_pc, next_pc;
        int cur_rearm, next_rearm;
        int issued = 0;  // levels whose copies lane 0 issued
        batch(0, cur_pc, cur_rearm);
        batch(32, next_pc, next_rearm);
        for (int L = 0; L < levels; ++L) {
            const int i = L & 31;
            if (i == 0 && L > 0) {
                cur_pc = next_pc;
                cur_rearm = next_rearm;
                batch(L + 32, next_pc, next_rearm);
            }
            int4 pc;
            pc.x = __shfl_sync(0xffffffffu, cur_pc.x, i);
            pc.y = __shfl_sync(0xffffffffu, cur_pc.y, i);
            pc.z = __shfl_sync(0xffffffffu, cur_pc.z, i);
            pc.w = __shfl_sync(0xffffffffu, cur_pc.w, i);
            const int rearm = __shfl_sync(0xffffffffu, cur_rearm, i);
            const int s = L % S;
            // The stage is free once the consumers are done with level L - S.  After
            // a wait that ran out nothing more is issued, so a stage never holds more
            // than one outstanding set of copies (no phase gets a second arrival).
            if (lane == 0 && ok && L >= S) ok = wait_phase(empty + s, static_cast<unsigned>(L / S - 1) & 1u, a.status, L);
            if (lane == 0 && ok) {
                issued = L + 1;
                piece_of[s] = pc;
                rearm_of[s] = rearm;
                unsigned char* st = stages + static_cast<size_t>(s) * lay.bytes;
                const int cnt = pc.y - pc.x;
                if (cnt <= 0) {
                    mbar_expect_tx(full + s, 0u);  // an empty piece: the phase completes at once
                } else {
                    const int dep0 = pc.z - lead_of<int>(pc.z), val0 = pc.z - lead_of<T>(pc.z);
                    const int pos0 = pc.x - lead_of<T>(pc.x);
                    const bool entries = pc.w > pc.z;
                    const unsigned b_desc = static_cast<unsigned>(cnt) * 16u;
                    const unsigned b_dep = entries ? static_cast<unsigned>(sweep_round16((pc.w - dep0) * 4)) : 0u;
                    const unsigned b_val =
                        entries ? static_cast<unsigned>(sweep_round16((pc.w - val0) * static_cast<int>(sizeof(T))))
                                : 0u;
                    const unsigned b_pos =
                        static_cast<unsigned>(sweep_round16((pc.y - pos0) * static_cast<int>(sizeof(T))));
                    mbar_expect_tx(full + s, b_desc + b_dep + b_val + (MODE == 3 ? 3u : 2u) * b_pos);
                    bulk_copy(st + lay.desc, sp.desc + pc.x, b_desc, full + s, policy);
                    if (entries) {
                        bulk_copy(st + lay.dep, sp.dep + dep0, b_dep, full + s, policy);
                        bulk_copy(st + lay.val, static_cast<const T*>(sp.val) + val0, b_val, full + s, policy);
                    }
                    bulk_copy(st + lay.inv, static_cast<const T*>(sp.inv) + pos0, b_pos, full + s, policy);
                    bulk_copy(st + lay.rhs, rhs_src + pos0, b_pos, full + s, policy);
                    if (MODE == 3) bulk_copy(st + lay.rr, a.sw_rr + pos0, b_pos, full + s, policy);
                }
            }
            __syncwarp();
        }
        if (lane == 0) s_issued = issued;
    } else {
        // ---- consumers: one row per thread and pass.
        unsigned ring_at[kSweepCluster], bar_at[kSweepCluster];
#pragma unroll
        for (int k = 0; k < kSweepCluster; ++k) {
            ring_at[k] = cluster_address(smem_u32(ring), k);
            bar_at[k] = cluster_address(smem_u32(ringbar), k);
        }
        // The (z, p) copy the next product reads (the mixed backward sweep's output).
        float* zp_out = MODE == 3 ? reinterpret_cast<float*>(zp_buffer(a, a.st->it)) : nullptr;
        for (int L = 0; L < levels; ++L) {
            const int s = L % S;
            ok = wait_phase(full + s, static_cast<unsigned>(L / S) & 1u, a.status, L) && ok;
            const int4 pc = piece_of[s];
            const unsigned char* st = stages + static_cast<size_t>(s) * lay.bytes;
            const int4* sdesc = reinterpret_cast<const int4*>(st + lay.desc);
            const int dep0 = pc.z - lead_of<int>(pc.z), val0 = pc.z - lead_of<T>(pc.z);
            const int pos0 = pc.x - lead_of<T>(pc.x);
            const int* sdep = reinterpret_cast<const int*>(st + lay.dep);  // entry j at [j - dep0]
            const T* sval = reinterpret_cast<const T*>(st + lay.val);      // entry j at [j - val0]
            const T* sinv = reinterpret_cast<const T*>(st + lay.inv);      // position p at [p - pos0]
            const T* srhs = reinterpret_cast<const T*>(st + lay.rhs);
            const T* srr = reinterpret_cast<const T*>(st + lay.rr);
            const unsigned bar_off = static_cast<unsigned>(L % SR) * 8u;
            const int cnt = pc.y - pc.x;
            // The result of a row: into every CTA's ring, and out.
            auto publish = [&](int p, const int4& d, T y, T r) {
                const unsigned slot = static_cast<unsigned>(p & mask) * static_cast<unsigned>(sizeof(T));
#pragma unroll
                for (int k = 0; k < kSweepCluster; ++k) store_remote(ring_at[k] + slot, y, bar_at[k] + bar_off);
                if constexpr (kFwd) {
                    static_cast<T*>(a.sw_y)[d.w] = y;
                } else if constexpr (MODE == 1) {
                    a.z[d.x] = y;
                } else {
                    // z of DOF 2m sits in .x of node m's (z, p) float4, z of DOF 2m + 1 in .z.
                    zp_out[4 * (d.x >> 1) + 2 * (d.x & 1)] = y;
                    rz.add(r * y);
                }
            };
            // This thread's first row: its operands come out of the stage before the
            // wait for level L - 1, so only the ring reads and the arithmetic follow it.
            // A thread whose wait ran out reads nothing of the stage, which may not
            // have arrived, and publishes nothing.
            const bool have = ok && tid < cnt;
            int4 d = make_int4(0, 0, 0, 0);
            T rhs = T(0), inv = T(0), rr = T(0);
            int dk[kSweepUnroll];
            T vk[kSweepUnroll];
            if (have) {
                d = sdesc[tid];
                rhs = srhs[pc.x + tid - pos0];
                inv = sinv[pc.x + tid - pos0];
                if constexpr (MODE == 3) rr = srr[pc.x + tid - pos0];
#pragma unroll
                for (int k = 0; k < kSweepUnroll; ++k) {
                    if (d.y + k < d.z) {
                        dk[k] = sdep[d.y + k - dep0] & mask;
                        vk[k] = sval[d.y + k - val0];
                    }
                }
            }
            if (L > 0) {
                const int prev = L - 1;
                ok = wait_phase(ringbar + prev % SR, static_cast<unsigned>(prev / SR) & 1u, a.status, prev) && ok;
            }
            if (have && ok) {
                T acc = rhs;
                T prod[kSweepUnroll];
#pragma unroll
                for (int k = 0; k < kSweepUnroll; ++k)
                    if (d.y + k < d.z) prod[k] = sweep_mul(vk[k], ring[dk[k]]);
#pragma unroll
                for (int k = 0; k < kSweepUnroll; ++k)
                    if (d.y + k < d.z) acc = sweep_sub(acc, prod[k]);
                for (int j = d.y + kSweepUnroll; j < d.z; ++j)  // rows longer than the unrolled part
                    acc = sweep_sub(acc, sweep_mul(sval[j - val0], ring[sdep[j - dep0] & mask]));
                publish(pc.x + tid, d, sweep_mul(acc, inv), rr);
            }
            // Pieces wider than the consumer threads: further rows, read after the wait.
            for (int t = tid + kSweepConsumers; ok && t < cnt; t += kSweepConsumers) {
                const int p = pc.x + t;
                const int4 e = sdesc[t];
                T acc = srhs[p - pos0];
                for (int j = e.y; j < e.z; ++j)
                    acc = sweep_sub(acc, sweep_mul(sval[j - val0], ring[sdep[j - dep0] & mask]));
                publish(p, e, sweep_mul(acc, sinv[p - pos0]), MODE == 3 ? srr[p - pos0] : T(0));
            }
            consumers_sync();  // every consumer is done with stage s and has seen level L - 1 arrive
            if (tid == 0 && ok) {  // after a wait that ran out: no arrival on a phase that may be pending
                // The ring mbarrier of level L - 1 is free again: armed for level
                // L - 1 + SR, whose width the piece table carries with level L.
                const int rearm = rearm_of[s];
                arrive(empty + s);
                if (rearm >= 0) mbar_expect_tx(ringbar + (L - 1) % SR, static_cast<unsigned>(rearm) * sizeof(T));
            }
        }
        // Every result bound for this CTA has arrived before it exits.
        if (levels > 0)
            ok = wait_phase(ringbar + (levels - 1) % SR, static_cast<unsigned>((levels - 1) / SR) & 1u, a.status,
                            levels - 1) &&
                 ok;
    }
    if (!ok) s_failed = 1;
    __syncthreads();
    // No CTA leaves while a cluster peer is still in its level loop, where it
    // stores into this CTA's ring.  Every CTA gets here: each of its waits is bounded.
    cluster_sync_all();
    if (s_failed) {
        // A wait ran out: end the solve (the status word already says why).  Peers'
        // results issued before the barrier may still be landing in the ring, whose
        // phases this CTA no longer tracks: it stays 100 us before it releases its
        // shared memory.
        if (tid == 0) {
            a.st->status = LFGPU_ERR_TIMEOUT;
            a.st->done = 1;
            set_loop(a, false);
            // This CTA's own copies: at most one outstanding set per stage, the last
            // level issued into it, waited for with a bound the abort does not cut.
            const int issued = s_issued;
            for (int st = 0; st < S && st < issued; ++st) {
                const int last = st + ((issued - 1 - st) / S) * S;
                mbar_drain(full + st, static_cast<unsigned>(last / S) & 1u);
            }
            const unsigned long long t0 = global_ns();
            while (global_ns() - t0 < 100000ull) {
            }
        }
        __syncthreads();
        return;
    }
    if constexpr (MODE == 3) {
        FloatPair vv[1] = {rz};
        reduce_last<1>(a, 2, vv, [&](const double* t) { rho_from_application(a, t); });
    }
}

__device__ __forceinline__ void ic0_mark_pending(const CgArgs& a, int i) {
    if (a.y == nullptr) return;  // the subdomain preconditioner writes z without polls
    const double pending = __longlong_as_double(static_cast<long long>(kPending));
    reinterpret_cast<double2*>(a.y)[i] = make_double2(pending, pending);
    reinterpret_cast<double2*>(a.z)[i] = make_double2(pending, pending);
}

__device__ __forceinline__ void ic0_reset_chunks(const CgArgs& a) {
    if (a.ic_chunks != nullptr && blockIdx.x == 0 && threadIdx.x == 0) {
        a.ic_chunks[0] = 0ull;
        a.ic_chunks[1] = 0ull;
    }
}

// r = f (or the warm-start residual), x = x0 or 0; ||r||.
__global__ void __launch_bounds__(kThreads) ic0_init(CgArgs a) {
    double v[1] = {0.0};
    double2* r2 = reinterpret_cast<double2*>(a.r);
    double2* x2 = reinterpret_cast<double2*>(a.x);
    const double2* f2 = reinterpret_cast<const double2*>(a.f);
    GRID_NODES(i) {
        const double2 rv = a.x0 ? r2[i] : f2[i];
        r2[i] = rv;
        x2[i] = a.x0 ? reinterpret_cast<const double2*>(a.x0)[i] : make_double2(0.0, 0.0);
        ic0_mark_pending(a, i);
        v[0] += rv.x * rv.x + rv.y * rv.y;
    }
    ic0_reset_chunks(a);
    reduce_last<1>(a, 0, v, [&](const double* t) {
        CgState* s = a.st;
        s->r0 = s->rnorm = sqrt(fmax(0.0, t[0]));
        s->it = 0;
        if (s->r0 <= a.target) {
            s->converged = 1;
            s->done = 1;
        }
        set_loop(a, !s->done);
    });
}

// After the first application: p = z, rho = r.z.
__global__ void __launch_bounds__(kThreads) ic0_start(CgArgs a) {
    if (a.st->done) return;
    double v[1] = {0.0};
    const double2* r2 = reinterpret_cast<const double2*>(a.r);
    const double2* z2 = reinterpret_cast<const double2*>(a.z);
    double2* p2 = reinterpret_cast<double2*>(a.p);
    GRID_NODES(i) {
        const double2 rv = r2[i], zv = z2[i];
        p2[i] = zv;
        v[0] += rv.x * zv.x + rv.y * zv.y;
    }
    reduce_last<1>(a, 3, v, [&](const double* t) {
        CgState* s = a.st;
        s->rho = t[0];
        if (!(t[0] > 0.0) || !isfinite(t[0])) {
            s->status = LFGPU_ERR_RHO_INITIAL;
            s->done = 1;
        }
        set_loop(a, !s->done);
    });
}

// x += alpha p, r -= alpha q; ||r|| decides convergence before the sweeps run.
__global__ void __launch_bounds__(kThreads) ic0_update(CgArgs a) {
    if (a.st->done) return;
    const double alpha = a.st->alpha;
    double v[1] = {0.0};
    double2* x2 = reinterpret_cast<double2*>(a.x);
    double2* r2 = reinterpret_cast<double2*>(a.r);
    const double2* p2 = reinterpret_cast<const double2*>(a.p);
    const double2* q2 = reinterpret_cast<const double2*>(a.q);
    GRID_NODES(i) {
        const double2 pv = p2[i], qv = q2[i];
        double2 xv = x2[i], rv = r2[i];
        xv.x += alpha * pv.x;
        xv.y += alpha * pv.y;
        rv.x -= alpha * qv.x;
        rv.y -= alpha * qv.y;
        x2[i] = xv;
        r2[i] = rv;
        ic0_mark_pending(a, i);
        v[0] += rv.x * rv.x + rv.y * rv.y;
    }
    ic0_reset_chunks(a);
    reduce_last<1>(a, 2, v, [&](const double* t) {
        CgState* s = a.st;
        s->it += 1;
        s->rnorm = sqrt(fmax(0.0, t[0]));
        if (s->rnorm <= a.target) {
            s->converged = 1;
            s->done = 1;
        }
        set_loop(a, !s->done);
    });
}

// rho' = r.z after the sweeps; beta = rho' / rho.
__global__ void __launch_bounds__(kThreads) ic0_dot(CgArgs a) {
    if (a.st->done) return;
    double v[1] = {0.0};
    const double2* r2 = reinterpret_cast<const double2*>(a.r);
    const double2* z2 = reinterpret_cast<const double2*>(a.z);
    GRID_NODES(i) {
        const double2 rv = r2[i], zv = z2[i];
        v[0] += rv.x * zv.x + rv.y * zv.y;
    }
    reduce_last<1>(a, 3, v, [&](const double* t) {
        CgState* s = a.st;
        if (!(t[0] > 0.0) || !isfinite(t[0])) {
            s->status = LFGPU_ERR_RHO;
            s->done = 1;
        } else {
            s->beta = t[0] / s->rho;
            s->rho = t[0];
            if (s->it >= a.maxit) s->done = 1;
        }
        set_loop(a, !s->done);
    });
}

// One application z = M^-1 r of the subdomain block-Jacobi preconditioner
// (SubdomainBlockJacobi::apply, src/precond.cpp:242-282): one CTA per subdomain,
// thread i holding local row i.  Forward substitution with the packed lower
// factor, then back substitution with its transpose, column by column: after
// unknown j is final every later row subtracts its term, so each row subtracts
// its terms in the reference's order (ascending forward, descending backward),
// each product and difference rounded on its own.  The result equals the
// reference's bit for bit.  The kernel is bound by the FP64 pipe: a separate
// multiply and subtract per factor entry and sweep.
__global__ void __launch_bounds__(LFGPU_SUBDOMAIN_MAX_DOFS) subdomain_apply(CgArgs a) {
    __shared__ double v[LFGPU_SUBDOMAIN_MAX_DOFS];
    const int s = blockIdx.x, i = threadIdx.x;
    const int begin = a.sub_begin[s], D = a.sub_begin[s + 1] - begin;
    const double* __restrict__ f = a.sub_factor + a.sub_fac[s];
    const bool mine = i < D;
    const int dof = mine ? a.sub_dofs[begin + i] : 0;
    const double* __restrict__ row = f + static_cast<long long>(i) * (i + 1) / 2;  // this thread's factor row
    double acc = mine ? a.r[dof] : 0.0;
    for (int j = 0; j < D; ++j) {
        if (i == j) v[j] = __dmul_rn(acc, row[j]);  // row[j] is the reciprocal pivot
        __syncthreads();
        if (mine && i > j) acc = __dsub_rn(acc, __dmul_rn(row[j], v[j]));
    }
    acc = mine ? v[i] : 0.0;
    double x = 0.0;
    for (int k = D - 1; k >= 0; --k) {
        if (i == k) v[k] = x = __dmul_rn(acc, row[k]);
        __syncthreads();
        if (i < k) acc = __dsub_rn(acc, __dmul_rn(f[static_cast<long long>(k) * (k + 1) / 2 + i], v[k]));
    }
    if (mine) a.z[dof] = x;
}

// The mixed loop's application of the subdomain preconditioner: z = M_s^-1 r on
// every subdomain with the block inverses (FP32 D x D squares, built in FP64 by
// subdomain.cu), on r32; z into the (z, p) copy the next product reads, and r.z.
// Its reduction sets rho and beta: after mx_init the first rho (r0.z0 > 0 or
// "positive initial preconditioned residual"), in the loop beta = r.z / rho, or
// 0 after a residual replacement in restart mode.
//
// A dense product has no dependency chain (the triangular solves of the FP64
// form need one barrier per unknown).  Thread i sums entry i of every row of the
// symmetric inverse, so a warp's loads are consecutive.
__global__ void __launch_bounds__(LFGPU_SUBDOMAIN_MAX_DOFS) mx_sub_apply(CgArgs a) {
    if (a.st->done) return;
    __shared__ float rs[LFGPU_SUBDOMAIN_MAX_DOFS];
    const int s = blockIdx.x, i = threadIdx.x;
    const int begin = a.sub_begin[s], D = a.sub_begin[s + 1] - begin;
    const float* __restrict__ A = a.sub_inv32 + a.sub_sq[s];
    const bool mine = i < D;
    const int dof = mine ? a.sub_dofs[begin + i] : 0;
    const float r = mine ? a.r32[dof] : 0.f;
    rs[i] = r;
    __syncthreads();
    float x = 0.f;
    if (mine) {
        // Eight loads in flight per thread: the stream is latency-bound otherwise.
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        const float* __restrict__ col = A + i;
        int j = 0;
        for (; j + 7 < D; j += 8) {
            float t[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) t[u] = __ldg(col + static_cast<long long>(j + u) * D);
#pragma unroll
            for (int u = 0; u < 8; ++u) acc[u & 3] = fmaf(t[u], rs[j + u], acc[u & 3]);
        }
        for (; j < D; ++j) acc[0] = fmaf(__ldg(col + static_cast<long long>(j) * D), rs[j], acc[0]);
        x = (acc[0] + acc[1]) + (acc[2] + acc[3]);
    }
    FloatPair rz;
    if (mine) {
        // z of DOF 2m sits in .x of node m's (z, p) float4, z of DOF 2m + 1 in .z.
        reinterpret_cast<float*>(zp_buffer(a, a.st->it))[4 * (dof >> 1) + 2 * (dof & 1)] = x;
        rz.add(r * x);
    }
    FloatPair vv[1] = {rz};
    reduce_last<1>(a, 2, vv, [&](const double* t) { rho_from_application(a, t); });
}

// One FP64 application of the Jacobi or 2x2 nodal preconditioner.
template <int PRECOND>
__global__ void __launch_bounds__(kThreads) precond_apply_kernel(CgArgs a) {
    const double2* r2 = reinterpret_cast<const double2*>(a.r);
    double2* z2 = reinterpret_cast<double2*>(a.z);
    GRID_NODES(i) { z2[i] = precond64<PRECOND>(a, i, r2[i]); }
}

// ------------------------------------------------------------------ staged mixed update
// The direct form's update with its operands staged by TMA.  mx_update's threads
// walk three or four nodes each, one round trip to memory per node, and the kernel
// spends most of its time waiting on them (ncu: long-scoreboard and barrier
// stalls, DRAM ~23 % busy).  Here each CTA owns a contiguous range of nodes, and
// a producer warp copies it chunk by chunk (p, q, the correction pair, r and the
// preconditioner's values of kStagedChunk nodes) into kStagedStages shared-memory
// stages with cp.async.bulk, up to kStagedStages chunks ahead: ~50 KB in flight per
// CTA instead of one load per thread.  It refills a stage as soon as every
// consumer warp has arrived on the stage's empty barrier, so no block-wide barrier
// runs per chunk (the 1000x1000 mixed BSR/Jacobi solve on one GB300: 1,032 ms with
// thread 0 refilling after a __syncthreads, 1,016 ms with the producer warp, 1,025
// ms with six stages).  The arithmetic per node is mx_update's, in the same order.
// (z, p) of the CTA's first staged_stash nodes stay in shared memory for the
// direction pass; any further ones read r, p and the preconditioner again from L2.
// alpha: while the producer fills the first stages, the consumers of every CTA add
// the product's CTA pairs of p.q (the order and arithmetic of reduce_tail_pair,
// so alpha is the same in every CTA and the same as a last CTA of the product
// would set) and divide.  That moved the 1000x1000 BSR/Jacobi solve from 1,000 to
// 947 ms on one GB300, same iterations: the product's last CTA had held up the
// end of every product launch.
constexpr int kStagedThreads = 256;  // consumers: one node per thread and chunk
constexpr int kStagedChunk = kStagedThreads;
constexpr int kStagedBlock = kStagedThreads + 32;  // plus the producer warp
constexpr int kStagedWarps = kStagedThreads / 32;
constexpr int kStagedStages = 4;
constexpr int kStagedCtasPerSm = 2;

template <int PRECOND>
constexpr int staged_pc_bytes() {  // preconditioner bytes per node
    return PRECOND == LFGPU_PRECOND_JACOBI ? 8 : 12;
}
template <int PRECOND>
constexpr int staged_stage_bytes() {  // p, q, hi, lo, r (8 bytes a node each) and the preconditioner
    return kStagedChunk * (5 * 8 + staged_pc_bytes<PRECOND>());
}
// Nodes of CTA b: [b * per, min(nb, (b + 1) * per)) with per a multiple of 4, so that
// every copy starts on a 16-byte boundary.  A copy's node count is rounded up to 4:
// the vectors' allocations are padded to 64 elements, the 2x2 factor by 12 floats.
inline __host__ __device__ int staged_per_cta(int nb, int grid) { return ((nb + grid - 1) / grid + 3) & ~3; }

template <int PRECOND>
__global__ void __launch_bounds__(kStagedBlock, kStagedCtasPerSm) mx_update_staged(CgArgs a) {
    constexpr int C = kStagedChunk, S = kStagedStages, PCB = staged_pc_bytes<PRECOND>();
    constexpr int SB = staged_stage_bytes<PRECOND>();
    extern __shared__ __align__(128) unsigned char staged_smem[];
    __shared__ __align__(8) unsigned long long full[S], empty[S];
    __shared__ int s_failed, s_issued;
    if (a.st->done) {
        if (blockIdx.x == 0 && threadIdx.x == 0) set_branch(a, false);
        return;
    }
    const unsigned go0 = a.st->go;  // moves only after every CTA has arrived
    __shared__ float s_alpha[2];
    __shared__ int s_bad;
    const int tid = threadIdx.x;
    const int per = staged_per_cta(a.nb, gridDim.x);
    const int n0 = min(a.nb, static_cast<int>(blockIdx.x) * per), n1 = min(a.nb, n0 + per);
    const int chunks = (n1 - n0 + C - 1) / C;
    const int stash_n = min(n1 - n0, a.staged_stash);
    float4* stash = reinterpret_cast<float4*>(staged_smem + S * SB);  // (z, p) of node n0 + j, j < stash_n
    const float* pc = PRECOND == LFGPU_PRECOND_JACOBI ? a.invd32 : a.blk32;
    auto issue = [&](int k) {  // the producer: chunk k into stage k % S
        const int s = k % S, b = n0 + k * C;
        const unsigned cnt4 = static_cast<unsigned>((min(C, n1 - b) + 3) & ~3);
        unsigned char* st = staged_smem + s * SB;
        mbar_expect_tx(full + s, cnt4 * (5u * 8u + static_cast<unsigned>(PCB)));
        bulk_copy(st, a.p32 + 2 * static_cast<size_t>(b), cnt4 * 8u, full + s);
        bulk_copy(st + C * 8, a.q32 + 2 * static_cast<size_t>(b), cnt4 * 8u, full + s);
        bulk_copy(st + 2 * C * 8, a.xhi + 2 * static_cast<size_t>(b), cnt4 * 8u, full + s);
        bulk_copy(st + 3 * C * 8, a.xlo + 2 * static_cast<size_t>(b), cnt4 * 8u, full + s);
        bulk_copy(st + 4 * C * 8, a.r32 + 2 * static_cast<size_t>(b), cnt4 * 8u, full + s);
        bulk_copy(st + 5 * C * 8, pc + (PCB / 4) * static_cast<size_t>(b), cnt4 * static_cast<unsigned>(PCB), full + s);
    };
    if (tid == 0) {
        s_failed = 0;
        s_issued = 0;
        for (int s = 0; s < S; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, kStagedWarps);
        }
        mbar_init_fence();
    }
    __syncthreads();
    const unsigned long long limit = a.status->wait_limit_ns;
    bool ok = true;
    FloatPair rr, rz;
    float alpha = 0.f, alpha_lo = 0.f;
    bool bad = false;
    if (tid < kStagedThreads) {
        // alpha = rho / p.q from mx_product's CTA pairs, while the producer fills the
        // first stages.  Every CTA adds them in the same order with the same
        // arithmetic, so all CTAs hold the same alpha.
        const float2* part = reinterpret_cast<const float2*>(a.partials + static_cast<size_t>(a.blocks) * kMaxReduce);
        FloatPair acc[1];
        for (int b = tid; b < a.product_grid; b += kStagedThreads) {
            const float2 t = __ldcg(part + b * kMaxReduce);
            acc[0].add(FloatPair{t.x, t.y});
        }
        FloatPair tot[1];
        block_pair_reduce<1, kStagedThreads>(acc, tot);
        if (tid == 0) {
            const double pq = static_cast<double>(tot[0].hi) + static_cast<double>(tot[0].lo);
            s_bad = !(pq > 0.0) || !isfinite(pq);
            float hi = 0.f, lo = 0.f;
            if (!s_bad) pair_quotient(a.st->rho, pq, hi, lo);
            s_alpha[0] = hi;
            s_alpha[1] = lo;
            if (blockIdx.x == 0) {
                if (s_bad) {
                    a.st->status = LFGPU_ERR_NOT_SPD;
                    a.st->done = 1;
                    set_branch(a, false);
                    set_loop(a, false);
                } else {
                    a.st->alpha32 = hi;
                    a.st->alpha32_lo = lo;
                    a.st->alpha = static_cast<double>(hi) + static_cast<double>(lo);
                }
            }
        }
        pair_reduce_sync<kStagedThreads>();
        alpha = s_alpha[0];
        alpha_lo = s_alpha[1];
        bad = s_bad != 0;
    }
    if (tid >= kStagedThreads) {
        // Producer warp: lane 0 refills a stage as soon as every consumer warp is done
        // with it.  If that wait runs out it issues nothing more, so a stage never
        // holds more than one outstanding set of copies: no full-barrier phase gets a
        // second arrival, and no copy lands on data still being read.
        if (tid == kStagedThreads) {
            int k = 0;
            for (; k < chunks; ++k) {
                const int s = k % S;
                if (k >= S && !mbar_wait(empty + s, static_cast<unsigned>(k / S - 1) & 1u, a.status, limit)) {
                    ok = false;
                    break;
                }
                issue(k);
            }
            s_issued = k;
        }
    } else {
    for (int k = 0; k < chunks; ++k) {
        const int s = k % S;
        // A warp goes on only if every lane saw the stage arrive; after a wait that
        // ran out it neither reads nor releases another stage.
        if (!__all_sync(0xffffffffu, mbar_wait(full + s, static_cast<unsigned>(k / S) & 1u, a.status, limit))) {
            ok = false;
            break;
        }
        const unsigned char* st = staged_smem + s * SB;
        const int i = n0 + k * C + tid;
        if (i < n1 && !bad) {
            const float2 pv = reinterpret_cast<const float2*>(st)[tid];
            const float2 qv = reinterpret_cast<const float2*>(st + C * 8)[tid];
            float2 hv = reinterpret_cast<const float2*>(st + 2 * C * 8)[tid];
            float2 lv = reinterpret_cast<const float2*>(st + 3 * C * 8)[tid];
            float2 rv = reinterpret_cast<const float2*>(st + 4 * C * 8)[tid];
            pair_axpy(hv.x, lv.x, alpha, alpha_lo, pv.x);
            pair_axpy(hv.y, lv.y, alpha, alpha_lo, pv.y);
            rv.x -= alpha * qv.x;
            rv.y -= alpha * qv.y;
            const float2 zv = precond32_at<PRECOND>(reinterpret_cast<const float*>(st + 5 * C * 8), tid, rv);
            reinterpret_cast<float2*>(a.xhi)[i] = hv;
            reinterpret_cast<float2*>(a.xlo)[i] = lv;
            reinterpret_cast<float2*>(a.r32)[i] = rv;
            if (i - n0 < stash_n) stash[i - n0] = make_float4(zv.x, zv.y, pv.x, pv.y);
            rr.add(rv.x * rv.x + rv.y * rv.y);
            rz.add(rv.x * zv.x + rv.y * zv.y);
        }
        __syncwarp();
        if ((tid & 31) == 0) arrive(empty + s);  // this warp is done with stage s
    }
    }
    if (!ok) s_failed = 1;
    __syncthreads();
    if (s_failed) {
        // A wait ran out: end the solve (the status word says why).  Copies this CTA
        // issued land before its shared memory is released: each stage has at most
        // one outstanding set, its last chunk's, whose full phase is waited for with
        // a fixed bound that the abort flag does not cut short.
        if (tid == 0) {
            a.st->done = 1;
            set_branch(a, false);
            set_loop(a, false);
            const int issued = s_issued;
            for (int st = 0; st < S && st < issued; ++st) {
                const int last = st + ((issued - 1 - st) / S) * S;  // the last chunk issued into stage st
                mbar_drain(full + st, static_cast<unsigned>(last / S) & 1u);
            }
        }
        __syncthreads();
        return;
    }
    if (s_bad) return;  // p.q not positive: the solve ends (block 0 set the status); every copy has landed
    FloatPair v[2] = {rr, rz};
    const bool last = reduce_last<2>(a, 2, v, [&](const double* t) { update_totals<false>(a, t); });
    if (!wait_for_beta(a, last, go0)) return;
    const float beta = __ldcg(&a.st->beta32);
    float2* pw = reinterpret_cast<float2*>(a.p32);
    for (int j = n0 + tid; tid < C && j < n1; j += C) {  // the nodes this thread updated above
        float2 zv, pv;
        if (j - n0 < stash_n) {
            const float4 t = stash[j - n0];
            zv = make_float2(t.x, t.y);
            pv = make_float2(t.z, t.w);
        } else {
            zv = precond32<PRECOND>(a, j, reinterpret_cast<const float2*>(a.r32)[j]);
            pv = pw[j];
        }
        pw[j] = make_float2(pnew(zv.x, pv.x, beta), pnew(zv.y, pv.y, beta));
    }
}

// ------------------------------------------------------------------ graph assembly
struct GraphBuilder {
    Context& c;
    cudaGraph_t graph = nullptr;
    ~GraphBuilder() {
        if (graph) cudaGraphDestroy(graph);
    }
};

template <typename K>
void add_kernel(cudaGraph_t g, cudaGraphNode_t* node, const cudaGraphNode_t* dep, int ndep, K kernel, int blocks,
                CgArgs* args, int smem = 0, int threads = kThreads, bool cooperative = false) {
    cudaKernelNodeParams p = {};
    p.func = reinterpret_cast<void*>(kernel);
    p.gridDim = dim3(blocks);
    p.blockDim = dim3(threads);
    p.sharedMemBytes = smem;
    void* params[1] = {args};
    p.kernelParams = params;
    LF_CUDA(cudaGraphAddKernelNode(node, g, dep, ndep, &p));
    if (cooperative) {  // every CTA resident at once, or the launch fails
        cudaLaunchAttributeValue v = {};
        v.cooperative = 1;
        LF_CUDA(cudaGraphKernelNodeSetAttribute(*node, cudaLaunchAttributeCooperative, &v));
    }
}

// Launch shape of mx_update_staged: kStagedCtasPerSm CTAs an SM (fewer if they do
// not fit), the stages, and the rest of each CTA's share of the SM's shared memory
// for (z, p).
struct StagedShape {
    int grid, smem, stash;
};
template <int PRECOND>
StagedShape staged_shape(int nb) {
    int dev = 0, sms = 0, smem_sm = 0, per_sm = 0;
    LF_CUDA(cudaGetDevice(&dev));
    LF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    LF_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    const int stages = kStagedStages * staged_stage_bytes<PRECOND>();
    const int share = smem_sm / kStagedCtasPerSm - 4096;  // less the static arrays and the per-CTA reservation
    const int grid = kStagedCtasPerSm * sms;
    const int stash = std::max(0, std::min((share - stages) / 16, staged_per_cta(nb, grid)));
    StagedShape sh{grid, stages + 16 * stash, stash};
    LF_CUDA(cudaFuncSetAttribute(mx_update_staged<PRECOND>, cudaFuncAttributeMaxDynamicSharedMemorySize, sh.smem));
    LF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mx_update_staged<PRECOND>, kStagedBlock, sh.smem));
    LF_REQUIRE(per_sm >= 1, LFGPU_ERR_CUDA, "the staged update does not fit an SM");
    sh.grid = std::min(grid, per_sm * sms);
    return sh;
}

cudaGraphNode_t add_conditional(cudaGraph_t g, const cudaGraphNode_t* dep, int ndep, cudaGraphConditionalHandle h,
                                cudaGraphConditionalNodeType type, cudaGraph_t* body) {
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = type;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    LF_CUDA(cudaGraphAddNode(&node, g, dep, nullptr, ndep, &np));
    *body = np.conditional.phGraph_out[0];
    return node;
}

template <int STORAGE, int PRECOND>
void build_fp64(cudaGraph_t g, CgArgs* a, int blocks) {
    cudaGraphNode_t n_res = nullptr, n_init, n_loop;
    if (a->x0) add_kernel(g, &n_res, nullptr, 0, cg64_residual<STORAGE>, blocks, a);
    add_kernel(g, &n_init, a->x0 ? &n_res : nullptr, a->x0 ? 1 : 0, cg64_init<PRECOND>, blocks, a);
    cudaGraph_t body;
    n_loop = add_conditional(g, &n_init, 1, a->loop, cudaGraphCondTypeWhile, &body);
    (void)n_loop;
    cudaGraphNode_t k1, k2, k3;
    add_kernel(body, &k1, nullptr, 0, cg64_product<STORAGE>, blocks, a);
    add_kernel(body, &k2, &k1, 1, cg64_update<PRECOND>, blocks, a);
    add_kernel(body, &k3, &k2, 1, cg64_direction, blocks, a);
}

constexpr int kBodyIterations = 8;

// The mixed loop's separately applied preconditioners, after `dep`; returns the
// last node.  Subdomain: one kernel (sub_grid CTAs of sub_threads); IC(0): the
// forward and the backward FP32 level sweep (one cluster each, smem bytes of ring).
template <int PRECOND>
cudaGraphNode_t add_mixed_apply(cudaGraph_t g, cudaGraphNode_t dep, CgArgs* a, int sub_grid, int sub_threads,
                                int smem) {
    cudaGraphNode_t n1, n2;
    if constexpr (PRECOND == LFGPU_PRECOND_SUBDOMAIN) {
        add_kernel(g, &n1, &dep, 1, mx_sub_apply, sub_grid, a, 0, sub_threads);
        return n1;
    } else {
        cudaGraphNode_t n0;
        add_kernel(g, &n0, &dep, 1, ic0_sweep_inputs<true>, a->blocks, a);
        add_kernel(g, &n1, &n0, 1, ic0_level_sweep<2>, kSweepCluster, a, smem, kSweepBlock);
        add_kernel(g, &n2, &n1, 1, ic0_level_sweep<3>, kSweepCluster, a, smem, kSweepBlock);
        return n2;
    }
}

// Preconditioners applied by their own kernels add them after mx_init and after
// each iteration's IF node; the branch then holds only the flush and the FP64
// residual, as the kernels after it re-precondition.
template <int STORAGE, int PRECOND, bool DIRECT>
void build_mixed(cudaGraph_t g, CgArgs* a, int blocks, int sub_grid = 0, int sub_threads = 0, int smem = 0) {
    constexpr bool kSub = applied_separately<PRECOND>();
    constexpr bool kDirect = DIRECT;
    StagedShape sh{blocks, 0, 0};
    if constexpr (kDirect) {
        sh = staged_shape<PRECOND>(a->nb);
        a->staged_stash = sh.stash;
    }
    cudaGraphNode_t n_init;
    add_kernel(g, &n_init, nullptr, 0, mx_init<PRECOND, DIRECT>, blocks, a);
    if constexpr (kSub) n_init = add_mixed_apply<PRECOND>(g, n_init, a, sub_grid, sub_threads, smem);
    cudaGraph_t body;
    const cudaGraphNode_t n_loop = add_conditional(g, &n_init, 1, a->loop, cudaGraphCondTypeWhile, &body);
    cudaGraphNode_t n_flush;
    add_kernel(g, &n_flush, &n_loop, 1, mx_flush<true>, blocks, a);
    // The body holds kBodyIterations iterations, dividing the conditional loop's per-pass cost.
    // Each IF node has its own handle (created on the body graph, where the nodes
    // live); the kernels of each half carry the handle of their half, and the
    // second half returns at once when the first one ended the solve.
    CgArgs halves[kBodyIterations];  // kernel parameters are copied into the nodes at creation
    cudaGraphNode_t prev = nullptr;
    for (int h = 0; h < kBodyIterations; ++h) {
        halves[h] = *a;
        CgArgs* ah = &halves[h];
        ah->half = h;
        LF_CUDA(cudaGraphConditionalHandleCreate(&ah->branch, body, 0, 0));
        cudaGraphNode_t k1, k2, k3, k4, k5, k6;
        add_kernel(body, &k1, prev ? &prev : nullptr, prev ? 1 : 0, mx_product<STORAGE, kDirect>, blocks, ah);
        if constexpr (kDirect)
            add_kernel(body, &k2, &k1, 1, mx_update_staged<PRECOND>, sh.grid, ah, sh.smem, kStagedBlock, true);
        else
            add_kernel(body, &k2, &k1, 1, mx_update<PRECOND>, blocks, ah);
        cudaGraph_t branch;
        prev = add_conditional(body, &k2, 1, ah->branch, cudaGraphCondTypeIf, &branch);
        add_kernel(branch, &k3, nullptr, 0, mx_flush<false>, blocks, ah);
        add_kernel(branch, &k4, &k3, 1, mx_residual<STORAGE>, blocks, ah);
        if constexpr (kSub) {
            prev = add_mixed_apply<PRECOND>(body, prev, ah, sub_grid, sub_threads, smem);
        } else {
            add_kernel(branch, &k5, &k4, 1, mx_reprecondition<PRECOND, DIRECT>, blocks, ah);
            if constexpr (kDirect) add_kernel(branch, &k6, &k5, 1, mx_direction, blocks, ah);
        }
    }
}

// Per-kernel device time of the profiling form: an event after every launch; the
// time between consecutive events is charged to that launch's phase slot.
struct EventTrail {
    cudaStream_t stream;
    bool on;
    std::vector<cudaEvent_t> ev;
    std::vector<int> slot;
    EventTrail(cudaStream_t s, bool enabled) : stream(s), on(enabled) { mark(-1); }
    ~EventTrail() {
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
    void mark(int phase) {
        if (!on) return;
        cudaEvent_t e;
        LF_CUDA(cudaEventCreate(&e));
        ev.push_back(e);
        slot.push_back(phase);
        LF_CUDA(cudaEventRecord(e, stream));
    }
    void totals(unsigned long long (&ns)[6]) {
        for (auto& v : ns) v = 0;
        if (!on || ev.size() < 2) return;
        LF_CUDA(cudaEventSynchronize(ev.back()));
        for (size_t i = 1; i < ev.size(); ++i) {
            float ms = 0.f;
            LF_CUDA(cudaEventElapsedTime(&ms, ev[i - 1], ev[i]));
            if (slot[i] >= 0 && slot[i] < 6) ns[slot[i]] += static_cast<unsigned long long>(ms * 1.0e6);
        }
    }
};

// Profiling form: the same kernels launched one by one on the stream for `iters`
// loop passes (the branch kernels run every pass and return unless a replacement
// is due).  Profilers see these launches; they do not descend into graph nodes.
// Phase slots: 0 product, 1 update, 2 FP64 p update or mixed residual
// replacement, 3 mixed re-preconditioning (subdomain: the block solves).
template <int STORAGE, int PRECOND, bool DIRECT = false>
void launch_unrolled(cudaStream_t stream, CgArgs* a, int blocks, bool mixed, int iters, EventTrail& trail,
                     int sub_grid = 0, int sub_threads = 0, int smem = 0) {
    constexpr bool kSub = applied_separately<PRECOND>();
    auto chain = [&](auto kernel, int phase) {
        kernel<<<blocks, kThreads, 0, stream>>>(*a);
        LF_CUDA(cudaGetLastError());
        trail.mark(phase);
    };
    auto sub_apply = [&](int phase) {
        if constexpr (PRECOND == LFGPU_PRECOND_IC0) {
            ic0_sweep_inputs<true><<<a->blocks, kThreads, 0, stream>>>(*a);
            LF_CUDA(cudaGetLastError());
            ic0_level_sweep<2><<<kSweepCluster, kSweepBlock, smem, stream>>>(*a);
            LF_CUDA(cudaGetLastError());
            trail.mark(phase);
            ic0_level_sweep<3><<<kSweepCluster, kSweepBlock, smem, stream>>>(*a);
        } else {
            mx_sub_apply<<<sub_grid, sub_threads, 0, stream>>>(*a);
        }
        LF_CUDA(cudaGetLastError());
        trail.mark(phase);
    };
    constexpr bool kDirect = DIRECT;
    StagedShape sh{blocks, 0, 0};
    if constexpr (kDirect) {
        sh = staged_shape<PRECOND>(a->nb);
        a->staged_stash = sh.stash;
    }
    auto update = [&](int phase) {
        if constexpr (kDirect) {  // its CTAs wait for one another: a cooperative launch
            void* args[1] = {a};
            LF_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(mx_update_staged<PRECOND>), dim3(sh.grid),
                                                dim3(kStagedBlock), args, static_cast<size_t>(sh.smem), stream));
            trail.mark(phase);
        } else {
            chain(mx_update<PRECOND>, phase);
        }
    };
    if (!mixed && a->x0) chain(cg64_residual<STORAGE>, -1);
    if (mixed) chain(mx_init<PRECOND, DIRECT>, -1);
    else if constexpr (!kSub) chain(cg64_init<PRECOND>, -1);
    if (kSub) sub_apply(-1);
    for (int k = 0; k < iters; ++k) {
        if (mixed) {
            chain(mx_product<STORAGE, kDirect>, 0);
            update(1);
            chain(mx_flush<false>, 2);
            chain(mx_residual<STORAGE>, 2);
            if constexpr (kSub) {
                sub_apply(3);
            } else {
                chain(mx_reprecondition<PRECOND, DIRECT>, 3);
                if constexpr (kDirect) chain(mx_direction, 3);
            }
        } else if constexpr (!kSub) {  // the FP64 subdomain form is launch_separate_unrolled
            chain(cg64_product<STORAGE>, 0);
            chain(cg64_update<PRECOND>, 1);
            chain(cg64_direction, 2);
        }
    }
    if (mixed) chain(mx_flush<true>, -1);
}

// The pointwise preconditioners' mixed loop in the direct form or the (z, p_old)
// form, by mesh size (kDirectMinNodes).
template <int STORAGE, int PRECOND>
void build_pointwise(cudaGraph_t g, CgArgs* a, int blocks) {
    if (direct_form(PRECOND, a->nb)) build_mixed<STORAGE, PRECOND, true>(g, a, blocks);
    else build_mixed<STORAGE, PRECOND, false>(g, a, blocks);
}
template <int STORAGE, int PRECOND>
void launch_pointwise(cudaStream_t stream, CgArgs* a, int blocks, bool mixed, int iters, EventTrail& trail) {
    if (mixed && direct_form(PRECOND, a->nb)) launch_unrolled<STORAGE, PRECOND, true>(stream, a, blocks, mixed, iters, trail);
    else launch_unrolled<STORAGE, PRECOND, false>(stream, a, blocks, mixed, iters, trail);
}

// IC(0): init -> forward -> backward -> start -> WHILE { product ; update ;
// forward ; backward ; dot ; p update }.  The sweeps run one CTA per row chunk.
// The subdomain block-Jacobi form is the same with one apply kernel (one CTA per
// subdomain) in place of the two sweeps.
struct SeparateApply {
    bool subdomain;
    int chunks;    // IC(0): row chunks of the polled sweeps
    int sub_grid;  // subdomain: subdomains, and threads per CTA
    int sub_threads;
    bool levels;   // IC(0): the level-scheduled sweeps, with this much shared memory per CTA
    int smem;
};

// Adds the application after `dep`; returns its last node.
cudaGraphNode_t add_apply(cudaGraph_t g, cudaGraphNode_t dep, CgArgs* a, const SeparateApply& ap) {
    cudaGraphNode_t n1, n2;
    if (ap.subdomain) {
        add_kernel(g, &n1, &dep, 1, subdomain_apply, ap.sub_grid, a, 0, ap.sub_threads);
        return n1;
    }
    if (ap.levels) {
        cudaGraphNode_t n0;
        add_kernel(g, &n0, &dep, 1, ic0_sweep_inputs<false>, a->blocks, a);
        add_kernel(g, &n1, &n0, 1, ic0_level_sweep<0>, kSweepCluster, a, ap.smem, kSweepBlock);
        add_kernel(g, &n2, &n1, 1, ic0_level_sweep<1>, kSweepCluster, a, ap.smem, kSweepBlock);
        return n2;
    }
    add_kernel(g, &n1, &dep, 1, ic0_forward, ap.chunks, a, 0, kSweepRows);
    add_kernel(g, &n2, &n1, 1, ic0_backward, ap.chunks, a, 0, kSweepRows);
    return n2;
}

template <int STORAGE>
void build_separate(cudaGraph_t g, CgArgs* a, int blocks, const SeparateApply& ap) {
    cudaGraphNode_t n_res = nullptr, n_init, n_start;
    if (a->x0) add_kernel(g, &n_res, nullptr, 0, cg64_residual<STORAGE>, blocks, a);
    add_kernel(g, &n_init, a->x0 ? &n_res : nullptr, a->x0 ? 1 : 0, ic0_init, blocks, a);
    const cudaGraphNode_t n_apply = add_apply(g, n_init, a, ap);
    add_kernel(g, &n_start, &n_apply, 1, ic0_start, blocks, a);
    cudaGraph_t body;
    add_conditional(g, &n_start, 1, a->loop, cudaGraphCondTypeWhile, &body);
    cudaGraphNode_t k[4];
    add_kernel(body, &k[0], nullptr, 0, cg64_product<STORAGE>, blocks, a);
    add_kernel(body, &k[1], &k[0], 1, ic0_update, blocks, a);
    const cudaGraphNode_t k_apply = add_apply(body, k[1], a, ap);
    add_kernel(body, &k[2], &k_apply, 1, ic0_dot, blocks, a);
    add_kernel(body, &k[3], &k[2], 1, cg64_direction, blocks, a);
}

// Phase slots: 0 product, 1 update, 2 forward sweep (subdomain: the block
// solves), 3 backward sweep, 4 r.z, 5 p update.
template <int STORAGE>
void launch_separate_unrolled(cudaStream_t stream, CgArgs* a, int blocks, const SeparateApply& ap, int iters,
                              EventTrail& trail) {
    auto chain = [&](auto kernel, int phase) {  // the loop kernels
        kernel<<<blocks, kThreads, 0, stream>>>(*a);
        LF_CUDA(cudaGetLastError());
        trail.mark(phase);
    };
    auto apply = [&](bool in_loop) {
        if (ap.subdomain) {
            subdomain_apply<<<ap.sub_grid, ap.sub_threads, 0, stream>>>(*a);
            LF_CUDA(cudaGetLastError());
            trail.mark(in_loop ? 2 : -1);
            return;
        }
        if (ap.levels) {
            ic0_sweep_inputs<false><<<a->blocks, kThreads, 0, stream>>>(*a);
            LF_CUDA(cudaGetLastError());
            ic0_level_sweep<0><<<kSweepCluster, kSweepBlock, ap.smem, stream>>>(*a);
        } else {
            ic0_forward<<<ap.chunks, kSweepRows, 0, stream>>>(*a);  // one CTA per chunk of kSweepRows rows
        }
        LF_CUDA(cudaGetLastError());
        trail.mark(in_loop ? 2 : -1);
        if (ap.levels) {
            ic0_level_sweep<1><<<kSweepCluster, kSweepBlock, ap.smem, stream>>>(*a);
        } else {
            ic0_backward<<<ap.chunks, kSweepRows, 0, stream>>>(*a);
        }
        LF_CUDA(cudaGetLastError());
        trail.mark(in_loop ? 3 : -1);
    };
    if (a->x0) chain(cg64_residual<STORAGE>, -1);
    chain(ic0_init, -1);
    apply(false);
    chain(ic0_start, -1);
    for (int k = 0; k < iters; ++k) {
        chain(cg64_product<STORAGE>, 0);
        chain(ic0_update, 1);
        apply(true);
        chain(ic0_dot, 4);
        chain(cg64_direction, 5);
    }
}

// The subdomain arrays, and the apply kernel's launch shape.
SeparateApply subdomain_args(Context& c, CgArgs& a) {
    a.sub_dofs = c.sub_dofs;
    a.sub_begin = c.sub_begin;
    a.sub_fac = c.sub_fac_begin;
    a.sub_factor = c.sub_factor;
    a.sub_inv32 = c.sub_inv32;
    a.sub_sq = c.sub_sq_begin;
    SeparateApply ap{};
    ap.subdomain = true;
    ap.sub_grid = static_cast<int>(c.sub_count);
    ap.sub_threads = std::max(32, (c.sub_max + 31) / 32 * 32);
    return ap;
}

// The level-scheduled IC(0) sweeps' arrays (fp32: the mixed loop's FP32 factor),
// with the kernels' shared-memory allowance raised to the ring.  Requires
// ensure_ic0, ensure_ic0_schedule and ensure_ic0_sweep_values.
SeparateApply sweep_args(Context& c, CgArgs& a, bool fp32) {
    for (int d = 0; d < 2; ++d) {
        const Context::Sweep& s = c.sweep[d];
        a.sw[d].level_begin = s.level_begin;
        a.sw[d].pieces = s.pieces;
        a.sw[d].desc = s.desc;
        a.sw[d].dep = s.dep;
        a.sw[d].val = fp32 ? static_cast<const void*>(s.val32.p) : static_cast<const void*>(s.val.p);
        a.sw[d].inv = fp32 ? static_cast<const void*>(s.inv32.p) : static_cast<const void*>(s.inv.p);
        a.sw[d].levels = s.levels;
    }
    a.sw_window = c.sweep_window;
    a.sw_maxp = c.sweep_maxp;
    a.sw_maxe = c.sweep_maxe;
    SeparateApply ap{};
    ap.levels = true;
    if (fp32) {
        c.sweep_y32.ensure(c.n + kSweepSlack);
        c.sweep_rhs32.ensure(c.n + kSweepSlack);
        c.sweep_rr32.ensure(c.n + kSweepSlack);
        a.sw_y = c.sweep_y32.p;
        a.sw_rhs = c.sweep_rhs32.p;
        a.sw_rr = c.sweep_rr32.p;
        ap.smem = sweep_smem_bytes(static_cast<int>(sizeof(float)), c.sweep_window, c.sweep_maxp, c.sweep_maxe);
        LF_CUDA(cudaFuncSetAttribute(ic0_level_sweep<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, ap.smem));
        LF_CUDA(cudaFuncSetAttribute(ic0_level_sweep<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, ap.smem));
    } else {
        c.sweep_y.ensure(c.n + kSweepSlack);
        c.sweep_rhs.ensure(c.n + kSweepSlack);
        a.sw_y = c.sweep_y.p;
        a.sw_rhs = c.sweep_rhs.p;
        ap.smem = sweep_smem_bytes(static_cast<int>(sizeof(double)), c.sweep_window, c.sweep_maxp, c.sweep_maxe);
        LF_CUDA(cudaFuncSetAttribute(ic0_level_sweep<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, ap.smem));
        LF_CUDA(cudaFuncSetAttribute(ic0_level_sweep<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, ap.smem));
    }
    return ap;
}

}  // namespace

PcgResult finish_cg(Context& c, const SolveSetup& s);

PcgResult run_cg_graph(Context& c, const SolveSetup& s, float* kernel_ms) {
    const i64 n = c.n;
    LF_REQUIRE(n % 2 == 0, LFGPU_ERR_ARGUMENT, "the GPU PCG needs an even number of DOFs (u,v pairs)");
    const int blocks = c.num_sms * (2048 / kThreads);
    CgArgs a{};
    a.n = static_cast<int>(n);
    a.nb = static_cast<int>(n / 2);
    a.rowptr = c.rowptr;
    a.col = c.col;
    a.K = c.K;
    a.invd64 = c.inv_diag64;
    a.blk64 = c.blk64;
    a.invd32 = c.inv_diag32;
    a.blk32 = c.blk32;
    a.f = s.rhs;
    a.x0 = s.x0;
    a.x = s.x;
    for (auto& b : c.v64) b.ensure(n);
    a.r = c.v64[0];
    a.z = c.v64[1];
    a.p = c.v64[2];
    a.q = c.v64[3];
    a.r64 = c.v64[4];
    if (s.storage == LFGPU_STORAGE_BSR) {
        ensure_bsr(c);
        a.brow = c.brow;
        a.bcol = c.bcol;
        a.bval64 = reinterpret_cast<const double2*>(c.bval64.p);
    }
    if (s.mixed) {
        for (auto& b : c.v32) b.ensure(n);
        a.r32 = c.v32[0];
        a.p32 = c.v32[2];
        a.q32 = c.v32[4];
        for (auto& b : c.zp) b.ensure(n);
        a.zp0 = c.zp[0];
        a.zp1 = c.zp[1];
        c.xhi.ensure(n);
        c.xlo.ensure(n);
        a.xhi = c.xhi;
        a.xlo = c.xlo;
        if (s.storage == LFGPU_STORAGE_BSR || c.paired) {
            // A paired CSR pattern (rows 2i and 2i + 1 share one column list of
            // (2j, 2j + 1) pairs, as every Q4 and bar pattern does) holds the same
            // entries as the BSR form, so its FP32 working copy is the BSR blocks:
            // the FP32 product is the BSR one, bit for bit, while the FP64 products
            // of the refinement keep the CSR storage.  One float4 a block and a
            // 16-bit offset replace 8 bytes of values and the column pair.
            ensure_bsr32(c);
            a.brow = c.brow;
            a.bcol = c.bcol;
            a.bval32 = reinterpret_cast<const float4*>(c.bval32.p);
            a.bcol16 = c.bcol16_ok ? c.bcol16.p : nullptr;
            a.paired = s.storage == LFGPU_STORAGE_CSR ? 1 : 0;
        } else {
            ensure_csr32(c);
            a.K32 = c.K32;
            a.col16 = c.col16_ok ? c.col16.p : nullptr;
        }
        a.dhi = c.diag_hi;
        a.dlo = c.diag_lo;
    }
    const bool sub = s.precond == LFGPU_PRECOND_SUBDOMAIN;
    const bool ic = s.precond == LFGPU_PRECOND_IC0;
    LF_REQUIRE(!(sub || ic) || s.mixed, LFGPU_ERR_ARGUMENT, "the FP64 subdomain and ic0 solves are run_pcg_separate");
    SeparateApply ap{};
    if (sub) {
        ensure_subdomain_inverse(c);  // no-op when the solve's setup built it
        ap = subdomain_args(c, a);
    } else if (ic) {
        ensure_ic0(c);  // no-op when the solve's setup built them
        ic0_use_levels(c, true);
        ensure_ic0_sweep_values(c, true);
        ap = sweep_args(c, a, true);
    }
    // Reduction partials: one per CTA of the widest reducing launch (the subdomain
    // kernel runs a CTA per subdomain).
    const int reducing = std::max(blocks, ap.sub_grid);
    c.partials.ensure(static_cast<size_t>(kSlots) * kMaxReduce * reducing);
    a.partials = c.partials;
    a.blocks = reducing;
    a.product_grid = blocks;
    c.cg_state.ensure(sizeof(CgState));
    a.st = reinterpret_cast<CgState*>(c.cg_state.p);
    a.status = c.status;
    a.target = s.tolerance;
    a.reduction = s.inner_reduction;
    a.maxit = s.max_iterations;
    a.max_ref = s.max_refinements;
    a.restart = s.restart;
    LF_CUDA(cudaMemsetAsync(c.cg_state.p, 0, sizeof(CgState), c.stream));

    const bool csr = s.storage == LFGPU_STORAGE_CSR;
    const bool jac = s.precond == LFGPU_PRECOND_JACOBI;
    a.use_cond = s.unrolled > 0 ? 0 : 1;
    if (s.unrolled > 0) {
        LF_REQUIRE(s.unrolled <= 100000, LFGPU_ERR_ARGUMENT, "profiling runs are limited to 100000 passes");
        const bool mx = s.mixed != 0;
        LF_CUDA(cudaEventRecord(c.ev_a, c.stream));
        EventTrail trail(c.stream, s.unrolled <= kTimedPasses);
        if (sub && csr)
            launch_unrolled<LFGPU_STORAGE_CSR, LFGPU_PRECOND_SUBDOMAIN>(c.stream, &a, blocks, mx, s.unrolled, trail,
                                                                        ap.sub_grid, ap.sub_threads);
        else if (sub)
            launch_unrolled<LFGPU_STORAGE_BSR, LFGPU_PRECOND_SUBDOMAIN>(c.stream, &a, blocks, mx, s.unrolled, trail,
                                                                        ap.sub_grid, ap.sub_threads);
        else if (ic && csr)
            launch_unrolled<LFGPU_STORAGE_CSR, LFGPU_PRECOND_IC0>(c.stream, &a, blocks, mx, s.unrolled, trail, 0, 0,
                                                                  ap.smem);
        else if (ic)
            launch_unrolled<LFGPU_STORAGE_BSR, LFGPU_PRECOND_IC0>(c.stream, &a, blocks, mx, s.unrolled, trail, 0, 0,
                                                                  ap.smem);
        else if (csr && jac) launch_pointwise<LFGPU_STORAGE_CSR, LFGPU_PRECOND_JACOBI>(c.stream, &a, blocks, mx, s.unrolled, trail);
        else if (csr) launch_pointwise<LFGPU_STORAGE_CSR, LFGPU_PRECOND_BLOCK2>(c.stream, &a, blocks, mx, s.unrolled, trail);
        else if (jac) launch_pointwise<LFGPU_STORAGE_BSR, LFGPU_PRECOND_JACOBI>(c.stream, &a, blocks, mx, s.unrolled, trail);
        else launch_pointwise<LFGPU_STORAGE_BSR, LFGPU_PRECOND_BLOCK2>(c.stream, &a, blocks, mx, s.unrolled, trail);
        LF_CUDA(cudaEventRecord(c.ev_b, c.stream));
        *kernel_ms = elapsed_ms(c);
        PcgResult res = finish_cg(c, s);
        trail.totals(res.phase_ns);
        return res;
    }
    GraphBuilder gb{c};
    LF_CUDA(cudaGraphCreate(&gb.graph, 0));
    LF_CUDA(cudaGraphConditionalHandleCreate(&a.loop, gb.graph, 0, 0));
    if (!s.mixed) {
        if (csr && jac) build_fp64<LFGPU_STORAGE_CSR, LFGPU_PRECOND_JACOBI>(gb.graph, &a, blocks);
        else if (csr) build_fp64<LFGPU_STORAGE_CSR, LFGPU_PRECOND_BLOCK2>(gb.graph, &a, blocks);
        else if (jac) build_fp64<LFGPU_STORAGE_BSR, LFGPU_PRECOND_JACOBI>(gb.graph, &a, blocks);
        else build_fp64<LFGPU_STORAGE_BSR, LFGPU_PRECOND_BLOCK2>(gb.graph, &a, blocks);
    } else {
        if (sub && csr)
            build_mixed<LFGPU_STORAGE_CSR, LFGPU_PRECOND_SUBDOMAIN, false>(gb.graph, &a, blocks, ap.sub_grid,
                                                                          ap.sub_threads);
        else if (sub)
            build_mixed<LFGPU_STORAGE_BSR, LFGPU_PRECOND_SUBDOMAIN, false>(gb.graph, &a, blocks, ap.sub_grid,
                                                                          ap.sub_threads);
        else if (ic && csr)
            build_mixed<LFGPU_STORAGE_CSR, LFGPU_PRECOND_IC0, false>(gb.graph, &a, blocks, 0, 0, ap.smem);
        else if (ic)
            build_mixed<LFGPU_STORAGE_BSR, LFGPU_PRECOND_IC0, false>(gb.graph, &a, blocks, 0, 0, ap.smem);
        else if (csr && jac) build_pointwise<LFGPU_STORAGE_CSR, LFGPU_PRECOND_JACOBI>(gb.graph, &a, blocks);
        else if (csr) build_pointwise<LFGPU_STORAGE_CSR, LFGPU_PRECOND_BLOCK2>(gb.graph, &a, blocks);
        else if (jac) build_pointwise<LFGPU_STORAGE_BSR, LFGPU_PRECOND_JACOBI>(gb.graph, &a, blocks);
        else build_pointwise<LFGPU_STORAGE_BSR, LFGPU_PRECOND_BLOCK2>(gb.graph, &a, blocks);
    }
    cudaGraphExec_t exec = nullptr;
    LF_CUDA(cudaGraphInstantiate(&exec, gb.graph, 0));
    cudaError_t err = cudaEventRecord(c.ev_a, c.stream);
    if (err == cudaSuccess) err = cudaGraphLaunch(exec, c.stream);
    if (err == cudaSuccess) err = cudaEventRecord(c.ev_b, c.stream);
    cudaGraphExecDestroy(exec);
    LF_CUDA(err);
    *kernel_ms = elapsed_ms(c);
    return finish_cg(c, s);
}

PcgResult finish_cg(Context& c, const SolveSetup& s) {
    CgState st{};
    LF_CUDA(cudaMemcpyAsync(&st, c.cg_state.p, sizeof(st), cudaMemcpyDeviceToHost, c.stream));
    check_status(c);
    // Kernels that ran: residual (warm start) + init, then per loop pass the body
    // (FP64: product, update, direction; mixed: product, update) and per residual
    // replacement the two branch kernels; the profiling form launches every kernel
    // of every pass.
    // IC(0): residual (warm start), init, two sweeps and start, then six kernels a
    // pass; subdomain block-Jacobi: one apply kernel in place of the two sweeps.
    // IC(0) by levels: a gather of r (ic0_sweep_inputs) before the two sweeps.
    const bool levels = c.ic0_sweep != LFGPU_IC0_SWEEP_POLLED && ic0_levels_chosen(c, s.mixed);
    const int direct = s.mixed && direct_form(s.precond, c.n / 2) ? 1 : 0;
    if (s.precond == LFGPU_PRECOND_IC0 && s.mixed)  // mixed: init, gather and two sweeps, then product, update,
                                                    // gather and two sweeps an iteration, flush and residual per
                                                    // replacement, final flush
        c.launches += 4 + (s.unrolled > 0 ? 7 * static_cast<i64>(s.unrolled)
                                          : 5 * kBodyIterations * ((st.it + kBodyIterations - 1) / kBodyIterations) +
                                                2 * st.refs) +
                      1;
    else if (s.precond == LFGPU_PRECOND_IC0)
        c.launches += (s.x0 ? 1 : 0) + (levels ? 5 : 4) +
                      (levels ? 7 : 6) * (s.unrolled > 0 ? static_cast<i64>(s.unrolled) : st.it);
    else if (s.precond == LFGPU_PRECOND_SUBDOMAIN && !s.mixed)
        c.launches += (s.x0 ? 1 : 0) + 3 + 5 * (s.unrolled > 0 ? static_cast<i64>(s.unrolled) : st.it);
    else if (s.precond == LFGPU_PRECOND_SUBDOMAIN)  // mixed: init + apply, then product, update, apply an
                                                    // iteration, flush and residual per replacement, final flush
        c.launches += 2 + (s.unrolled > 0 ? 5 * static_cast<i64>(s.unrolled)
                                          : 3 * kBodyIterations * ((st.it + kBodyIterations - 1) / kBodyIterations) +
                                                2 * st.refs) +
                      1;
    else if (s.unrolled > 0)
        c.launches += (s.x0 && !s.mixed ? 1 : 0) + 1 + static_cast<i64>(s.unrolled) * (s.mixed ? 5 + direct : 3) +
                      (s.mixed ? 1 : 0);
    else  // mixed: kBodyIterations iterations (two kernels each) a pass, the branch's flush, residual,
          // re-preconditioning (and direction, direct form) per replacement, a final flush after the loop
        c.launches += (s.x0 ? 1 : 0) + 1 +
                      (s.mixed ? 2 * kBodyIterations * ((st.it + kBodyIterations - 1) / kBodyIterations) +
                                     (3 + direct) * st.refs + 1
                               : 3 * st.it);
    PcgResult r{};
    r.iterations = st.it;
    r.refinements = st.refs;
    r.initial_residual = st.r0;
    r.final_residual = s.mixed ? st.rtrue : st.rnorm;
    r.status = st.status;
    r.converged = st.converged;
    r.stagnated = st.stagnated;
    return r;
}

namespace {

// Vectors and IC(0) arrays the sweeps and the solver share.
void ic0_args(Context& c, CgArgs& a) {
    a.diag = c.diag;
    a.icf = c.ic0_val;
    a.icinv = c.ic0_inv;
    a.ic_chunks = c.ic0_misc.p + kIc0ForwardChunk;
}


}  // namespace

PcgResult run_pcg_separate(Context& c, const SolveSetup& s, float* kernel_ms, double* apply_ms) {
    const i64 n = c.n;
    LF_REQUIRE(n % 2 == 0, LFGPU_ERR_ARGUMENT, "the GPU PCG needs an even number of DOFs (u,v pairs)");
    LF_REQUIRE(!s.mixed, LFGPU_ERR_UNSUPPORTED, "mixed precision supports the jacobi and block preconditioners");
    LF_REQUIRE(s.precond == LFGPU_PRECOND_IC0 || s.precond == LFGPU_PRECOND_SUBDOMAIN, LFGPU_ERR_ARGUMENT,
               "separate-kernel preconditioners are ic0 and subdomain");
    const bool sub = s.precond == LFGPU_PRECOND_SUBDOMAIN;
    const int blocks = c.num_sms * (2048 / kThreads);
    CgArgs a{};
    a.n = static_cast<int>(n);
    a.nb = static_cast<int>(n / 2);
    a.rowptr = c.rowptr;
    a.col = c.col;
    a.K = c.K;
    a.f = s.rhs;
    a.x0 = s.x0;
    a.x = s.x;
    for (auto& b : c.v64) b.ensure(n);
    a.r = c.v64[0];
    a.z = c.v64[1];
    a.p = c.v64[2];
    a.q = c.v64[3];
    if (s.storage == LFGPU_STORAGE_BSR) {
        ensure_bsr(c);
        a.brow = c.brow;
        a.bcol = c.bcol;
        a.bval64 = reinterpret_cast<const double2*>(c.bval64.p);
    }
    SeparateApply ap{};
    if (sub) {
        ap = subdomain_args(c, a);
    } else if (ic0_use_levels(c, false)) {
        ensure_ic0_sweep_values(c, false);
        ap = sweep_args(c, a, false);  // no pending marks, no chunk counters: a.y and a.ic_chunks stay null
    } else {
        a.y = c.v64[4];
        ic0_args(c, a);
        ap.chunks = static_cast<int>((n + kSweepRows - 1) / kSweepRows);
    }
    c.partials.ensure(static_cast<size_t>(kSlots) * kMaxReduce * blocks);
    a.partials = c.partials;
    a.blocks = blocks;
    c.cg_state.ensure(sizeof(CgState));
    a.st = reinterpret_cast<CgState*>(c.cg_state.p);
    a.status = c.status;
    a.target = s.tolerance;
    a.maxit = s.max_iterations;
    LF_CUDA(cudaMemsetAsync(c.cg_state.p, 0, sizeof(CgState), c.stream));
    const bool csr = s.storage == LFGPU_STORAGE_CSR;
    a.use_cond = s.unrolled > 0 ? 0 : 1;
    unsigned long long phase_ns[6] = {};
    if (s.unrolled > 0) {
        LF_REQUIRE(s.unrolled <= 100000, LFGPU_ERR_ARGUMENT, "profiling runs are limited to 100000 passes");
        LF_CUDA(cudaEventRecord(c.ev_a, c.stream));
        EventTrail trail(c.stream, s.unrolled <= kTimedPasses);
        if (csr) launch_separate_unrolled<LFGPU_STORAGE_CSR>(c.stream, &a, blocks, ap, s.unrolled, trail);
        else launch_separate_unrolled<LFGPU_STORAGE_BSR>(c.stream, &a, blocks, ap, s.unrolled, trail);
        LF_CUDA(cudaEventRecord(c.ev_b, c.stream));
        *kernel_ms = elapsed_ms(c);
        trail.totals(phase_ns);
    } else {
        GraphBuilder gb{c};
        LF_CUDA(cudaGraphCreate(&gb.graph, 0));
        LF_CUDA(cudaGraphConditionalHandleCreate(&a.loop, gb.graph, 0, 0));
        if (csr) build_separate<LFGPU_STORAGE_CSR>(gb.graph, &a, blocks, ap);
        else build_separate<LFGPU_STORAGE_BSR>(gb.graph, &a, blocks, ap);
        cudaGraphExec_t exec = nullptr;
        LF_CUDA(cudaGraphInstantiate(&exec, gb.graph, 0));
        cudaError_t err = cudaEventRecord(c.ev_a, c.stream);
        if (err == cudaSuccess) err = cudaGraphLaunch(exec, c.stream);
        if (err == cudaSuccess) err = cudaEventRecord(c.ev_b, c.stream);
        cudaGraphExecDestroy(exec);
        LF_CUDA(err);
        *kernel_ms = elapsed_ms(c);
    }
    PcgResult res = finish_cg(c, s);
    for (int k = 0; k < 6; ++k) res.phase_ns[k] = phase_ns[k];
    // Time one standalone application (forward + backward sweep, or the block
    // solves) on the final residual; the solve made iterations + 1 of them.
    LF_CUDA(cudaEventRecord(c.ev_a, c.stream));
    launch_precond_apply(c, s.precond, c.v64[0], c.v64[5]);
    LF_CUDA(cudaEventRecord(c.ev_b, c.stream));
    const double one = elapsed_ms(c);
    check_status(c);
    if (apply_ms) *apply_ms = one * static_cast<double>(res.iterations + 1);
    return res;
}

void launch_precond_apply(Context& c, int precond, const double* r, double* z) {
    const i64 n = c.n;
    LF_REQUIRE(n % 2 == 0, LFGPU_ERR_ARGUMENT, "the GPU preconditioners need an even number of DOFs (u,v pairs)");
    const int blocks = c.num_sms * (2048 / kThreads);
    CgArgs a{};
    a.n = static_cast<int>(n);
    a.nb = static_cast<int>(n / 2);
    a.rowptr = c.rowptr;
    a.col = c.col;
    a.r = const_cast<double*>(r);
    a.z = z;
    a.status = c.status;
    a.invd64 = c.inv_diag64;
    a.blk64 = c.blk64;
    if (precond == LFGPU_PRECOND_IC0 && ic0_use_levels(c, false)) {
        // The sweeps read the done flag of a solver state: give them a fresh one.
        c.cg_state.ensure(sizeof(CgState));
        a.st = reinterpret_cast<CgState*>(c.cg_state.p);
        LF_CUDA(cudaMemsetAsync(c.cg_state.p, 0, sizeof(CgState), c.stream));
        ensure_ic0_sweep_values(c, false);
        const SeparateApply ap = sweep_args(c, a, false);
        ic0_sweep_inputs<false><<<blocks, kThreads, 0, c.stream>>>(a);
        LF_CUDA(cudaGetLastError());
        ic0_level_sweep<0><<<kSweepCluster, kSweepBlock, ap.smem, c.stream>>>(a);
        LF_CUDA(cudaGetLastError());
        ic0_level_sweep<1><<<kSweepCluster, kSweepBlock, ap.smem, c.stream>>>(a);
        c.launches += 3;
    } else if (precond == LFGPU_PRECOND_IC0) {
        // The sweeps read the done flag of a solver state: give them a fresh one.
        c.cg_state.ensure(sizeof(CgState));
        a.st = reinterpret_cast<CgState*>(c.cg_state.p);
        LF_CUDA(cudaMemsetAsync(c.cg_state.p, 0, sizeof(CgState), c.stream));
        c.v64[4].ensure(n);
        a.y = c.v64[4];
        ic0_args(c, a);
        LF_CUDA(cudaMemsetAsync(a.y, 0xFF, sizeof(double) * n, c.stream));
        LF_CUDA(cudaMemsetAsync(z, 0xFF, sizeof(double) * n, c.stream));
        LF_CUDA(cudaMemsetAsync(a.ic_chunks, 0, 2 * sizeof(unsigned long long), c.stream));
        const int chunks = static_cast<int>((n + kSweepRows - 1) / kSweepRows);
        ic0_forward<<<chunks, kSweepRows, 0, c.stream>>>(a);
        ic0_backward<<<chunks, kSweepRows, 0, c.stream>>>(a);
        c.launches += 2;
    } else if (precond == LFGPU_PRECOND_SUBDOMAIN) {
        const SeparateApply ap = subdomain_args(c, a);
        if (ap.sub_grid > 0) subdomain_apply<<<ap.sub_grid, ap.sub_threads, 0, c.stream>>>(a);
        c.launches += ap.sub_grid > 0 ? 1 : 0;
    } else if (precond == LFGPU_PRECOND_JACOBI) {
        precond_apply_kernel<LFGPU_PRECOND_JACOBI><<<blocks, kThreads, 0, c.stream>>>(a);
        c.launches += 1;
    } else {
        precond_apply_kernel<LFGPU_PRECOND_BLOCK2><<<blocks, kThreads, 0, c.stream>>>(a);
        c.launches += 1;
    }
    LF_CUDA(cudaGetLastError());
}

}  // namespace lfgpu
