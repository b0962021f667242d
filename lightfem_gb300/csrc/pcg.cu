// Persistent preconditioned CG: the whole Krylov loop in one cooperative launch.
//
// Replaces pcg_solve<Matrix, Preconditioner> (src/solver.cpp:532-627) for CSR and
// 2x2 BSR storage (src/sparse.cpp:104-120, :179-204) with the Jacobi
// (src/solver.cpp:497-509) or 2x2 nodal block-Jacobi (src/precond.cpp:242-291 with
// one node per subdomain) preconditioner.
//
// Matrix streaming.  Every CTA owns a contiguous range of nodes (2 DOFs each) for
// the whole solve, hence a contiguous slice of the matrix.  A host-built schedule
// cuts that slice into tiles of whole rows; the product phase streams the tiles
// through a ring of shared-memory stages with 1-D bulk async copies
// (cp.async.bulk, completion on an mbarrier, L2 evict-first policy), issued
// kStages tiles ahead by one thread, so HBM latency overlaps the arithmetic.
// Inside a tile a quarter warp sums one row (CSR) or one 2x2 block row (BSR),
// reading values and columns from shared memory and gathering x from L2, where the
// iteration vectors stay resident.  Every mbarrier wait is bounded in time.
//
// FP64 iteration, phases separated by grid-wide barriers:
//   1. q = K p, partial p.q
//   2. alpha; x += alpha p; r -= alpha q; z = M^-1 r; partial r.r and r.z
//   3. beta; p = z + beta p
// Grid sums are published per CTA and added in CTA order by every CTA, so all
// CTAs take the same decisions from bit-identical scalars and runs are
// deterministic.  Grid barriers are bounded in time (common.cuh).
//
// Mixed precision: K (FP32 off-diagonals plus a compensated diagonal held as an
// FP32 hi/lo pair, see sparse.cu), the preconditioner and the Krylov vectors r,
// z, p, q in FP32; the solution update x += alpha p, the true residual
// r = f - K x with the FP64 matrix, and the convergence test in FP64.  When the
// FP32 recursive residual has dropped by `reduction` since the last replacement
// (or claims convergence) the FP64 residual is recomputed, tested, and replaces
// the FP32 one; the search direction is kept (reliable updates, Sleijpen & van der
// Vorst 1996) or dropped (restarted refinement).  In FP32 the p update is folded
// into the product: the gather forms z + beta p_old on the fly and each CTA writes
// p for its own rows into the other buffer, which removes the third barrier.
#include "common.cuh"
#include "kernels.hpp"

#include <algorithm>

namespace lfgpu {
namespace {

constexpr int kPcgThreads = 512;
constexpr int kStages = 3;
constexpr int kStageBytes = 32768;                 // data bytes per stage
constexpr int kSlack = 16;                         // units of alignment slack per tile
constexpr int kBatch = 6;                          // units per lane gathered together
constexpr int kDynSmem = kStages * (kStageBytes + 1024);
constexpr unsigned long long kCopyWaitNs = 2000000000ull;

enum Format { kCsr64 = 0, kCsr32 = 1, kBsr64 = 2, kBsr32 = 3 };
constexpr int kUnitBytes[4] = {8, 4, 32, 16};      // value bytes per unit (nonzero or 2x2 block)

// Units per tile for a format: value + column bytes of (units + slack) fit a stage.
constexpr int tile_units(int f) { return ((kStageBytes / (kUnitBytes[f] + 4)) - kSlack) / 8 * 8; }

struct TileSet {
    const int* ptr;        // row pointer in units (CSR rowptr or BSR block row pointer)
    const char* vals;      // unit values
    const int* cols;       // unit columns
    const int2* tiles;     // row range of every tile, CTA after CTA
    const int* cta;        // first tile of each CTA (G + 1 entries)
    int unit_bytes;
    int cols_offset;       // byte offset of the column area inside a stage
};

struct PcgArgs {
    int nb;
    TileSet mat64;          // FP64 matrix (the solve matrix, or the residual matrix when mixed)
    TileSet mat32;          // FP32 inner matrix (mixed)
    const float* dhi;       // compensated diagonal of the FP32 matrix
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
    float* z32;
    float* pa32;
    float* pb32;
    float* q32;
    double target;
    long long maxit;
    double reduction;
    long long max_ref;
    int restart;
    double* partials;
    unsigned long long* bar;
    DeviceStatus* status;
    PcgResult* result;
};

struct Shared {
    double red[32 * kMaxReduce];
    unsigned long long full[kStages];
    int flag;
};

// Ring of shared-memory stages fed by bulk copies.  `count` numbers the tiles
// this CTA has consumed since launch: tile g lives in stage g % kStages and its
// mbarrier completes phase (g / kStages) & 1.
struct Pipe {
    char* stage;
    unsigned long long* full;
    unsigned long long policy;
    unsigned count;

    __device__ char* base(int s) const { return stage + s * (kStageBytes + 1024); }

    // One thread: copy the aligned unit span of `tile` into stage s.
    __device__ void issue(const TileSet& m, int tile, int s) const {
        const int2 tr = m.tiles[tile];
        const int ua = __ldg(m.ptr + tr.x) & ~7;
        const int ub = (__ldg(m.ptr + tr.y) + 7) & ~7;
        const unsigned nv = static_cast<unsigned>(ub - ua) * m.unit_bytes;
        const unsigned nc = static_cast<unsigned>(ub - ua) * 4u;
        mbar_expect_tx(full + s, nv + nc);
        bulk_copy(base(s), m.vals + static_cast<size_t>(ua) * m.unit_bytes, nv, full + s, policy);
        bulk_copy(base(s) + m.cols_offset, m.cols + ua, nc, full + s, policy);
    }
};

__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 operator+(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
template <typename P> __device__ __forceinline__ P zero();
template <> __device__ __forceinline__ float zero<float>() { return 0.f; }
template <> __device__ __forceinline__ double zero<double>() { return 0.0; }
template <> __device__ __forceinline__ float2 zero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ double2 zero<double2>() { return make_double2(0.0, 0.0); }
__device__ __forceinline__ float lane_sum4(float v) {
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    return v + __shfl_xor_sync(0xffffffffu, v, 2);
}
__device__ __forceinline__ double lane_sum4(double v) {
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    return v + __shfl_xor_sync(0xffffffffu, v, 2);
}
__device__ __forceinline__ float2 lane_sum4(float2 v) { return make_float2(lane_sum4(v.x), lane_sum4(v.y)); }
__device__ __forceinline__ double2 lane_sum4(double2 v) { return make_double2(lane_sum4(v.x), lane_sum4(v.y)); }

// Product of one staged unit with the gathered x.
template <int F> struct UnitOp;
template <> struct UnitOp<kCsr64> {
    using P = double;
    template <typename G>
    static __device__ __forceinline__ P apply(const char* v, const int* c, int k, const G& g) {
        return reinterpret_cast<const double*>(v)[k] * g(c[k]);
    }
};
template <> struct UnitOp<kCsr32> {
    using P = float;
    template <typename G>
    static __device__ __forceinline__ P apply(const char* v, const int* c, int k, const G& g) {
        return reinterpret_cast<const float*>(v)[k] * g(c[k]);
    }
};
template <> struct UnitOp<kBsr64> {
    using P = double2;
    template <typename G>
    static __device__ __forceinline__ P apply(const char* v, const int* c, int k, const G& g) {
        const double2 top = reinterpret_cast<const double2*>(v)[2 * k];
        const double2 bot = reinterpret_cast<const double2*>(v)[2 * k + 1];
        const double2 x = g(c[k]);
        return make_double2(top.x * x.x + top.y * x.y, bot.x * x.x + bot.y * x.y);
    }
};
template <> struct UnitOp<kBsr32> {
    using P = float2;
    template <typename G>
    static __device__ __forceinline__ P apply(const char* v, const int* c, int k, const G& g) {
        const float4 a = reinterpret_cast<const float4*>(v)[k];
        const float2 x = g(c[k]);
        return make_float2(a.x * x.x + a.y * x.y, a.z * x.x + a.w * x.y);
    }
};

// Stream the CTA's tiles of matrix `m` and hand each row's product to
// finish(row, sum).  Returns false if a copy never completed (abort recorded).
template <int F, typename Gather, typename Finish>
__device__ __forceinline__ bool product(const TileSet& m, Pipe& pipe, DeviceStatus* status, const Gather& g,
                                        Finish&& finish) {
    using P = typename UnitOp<F>::P;
    const int t0 = m.cta[blockIdx.x], t1 = m.cta[blockIdx.x + 1];
    const int nt = t1 - t0;
    if (threadIdx.x == 0) {
        fence_proxy_async();
        for (int j = 0; j < nt && j < kStages; ++j) pipe.issue(m, t0 + j, (pipe.count + j) % kStages);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int sub = lane & 3;
    for (int j = 0; j < nt; ++j) {
        const unsigned gidx = pipe.count + j;
        const int s = gidx % kStages;
        const bool ok = mbar_wait(pipe.full + s, (gidx / kStages) & 1u, status, kCopyWaitNs);
        if (!__syncthreads_and(ok)) {
            // Let the copies already in flight land before the CTA gives up: this
            // tile's, whose wait ran out, and the ones issued ahead of it.
            if (threadIdx.x == 0) {
                for (int k = j; k < nt && k < j + kStages; ++k) {
                    const unsigned gk = pipe.count + k;
                    mbar_drain(pipe.full + gk % kStages, (gk / kStages) & 1u);
                }
            }
            __syncthreads();
            return false;
        }
        const int2 tr = m.tiles[t0 + j];
        const int ua = __ldg(m.ptr + tr.x) & ~7;
        const char* vals = pipe.base(s);
        const int* cols = reinterpret_cast<const int*>(pipe.base(s) + m.cols_offset);
        for (int rb = tr.x + warp * 8; rb < tr.y; rb += nwarps * 8) {
            const int row = rb + (lane >> 2);
            P acc = zero<P>();
            if (row < tr.y) {
                const int kb = __ldg(m.ptr + row) - ua, ke = __ldg(m.ptr + row + 1) - ua;
                // Up to kBatch units per lane at once: every gather of the batch is in
                // flight before the first product is summed.
                for (int k0 = kb + sub; k0 < ke; k0 += 4 * kBatch) {
                    P part[kBatch];
#pragma unroll
                    for (int b = 0; b < kBatch; ++b) {
                        const int k = k0 + 4 * b;
                        part[b] = k < ke ? UnitOp<F>::apply(vals, cols, k, g) : zero<P>();
                    }
#pragma unroll
                    for (int b = 0; b < kBatch; ++b) acc = acc + part[b];
                }
            }
            acc = lane_sum4(acc);
            if (row < tr.y && sub == 0) finish(row, acc);
        }
        __syncthreads();
        if (threadIdx.x == 0 && j + kStages < nt) {
            fence_proxy_async();
            pipe.issue(m, t0 + j + kStages, s);
        }
    }
    pipe.count += nt;
    return true;
}

// 2x2 nodal block solve with the packed factor (1/L00, L10, 1/L11): forward then
// backward substitution, each product and difference rounded separately as in
// SubdomainBlockJacobi::apply (src/precond.cpp:271-287).
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

__device__ __forceinline__ void write_result(const PcgArgs& a, long long it, long long refs, double r0, double rf,
                                             int status, int converged, int stagnated, const unsigned long long* t) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.result->iterations = it;
        a.result->refinements = refs;
        a.result->initial_residual = r0;
        a.result->final_residual = rf;
        a.result->status = status;
        a.result->converged = converged;
        a.result->stagnated = stagnated;
        for (int k = 0; k < 6; ++k) a.result->phase_ns[k] = t ? t[k] : 0ull;
    }
}

// Phase clock of CTA 0 (thread 0): accumulates the time between marks.
struct PhaseClock {
    unsigned long long t[6] = {0, 0, 0, 0, 0, 0};
    unsigned long long last = 0;
    __device__ __forceinline__ void start() {
        if (blockIdx.x == 0 && threadIdx.x == 0) last = global_ns();
    }
    __device__ __forceinline__ void mark(int k) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            const unsigned long long now = global_ns();
            t[k] += now - last;
            last = now;
        }
    }
};

__device__ __forceinline__ void pipe_init(Shared& sh, Pipe& pipe, char* dyn) {
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&sh.full[s], 1);
        mbar_init_fence();
    }
    __syncthreads();
    pipe.stage = dyn;
    pipe.full = sh.full;
    pipe.policy = l2_evict_first_policy();
    pipe.count = 0;
}

// FP64 product over the CTA's rows with gather x; out.row(dof, y) for CSR,
// out.node(node, y2) for BSR.
template <int STORAGE, typename Out>
__device__ __forceinline__ bool product64(const PcgArgs& a, Pipe& pipe, const double* x, Out& out) {
    if (STORAGE == LFGPU_STORAGE_CSR) {
        return product<kCsr64>(a.mat64, pipe, a.status, [&](int c) { return x[c]; },
                               [&](int row, double y) { out.row(row, y); });
    }
    const double2* x2 = reinterpret_cast<const double2*>(x);
    return product<kBsr64>(a.mat64, pipe, a.status, [&](int c) { return x2[c]; },
                           [&](int node, double2 y) { out.node(node, y); });
}

// ------------------------------------------------------------------ FP64 PCG
template <int STORAGE, int PRECOND>
__global__ void __launch_bounds__(kPcgThreads) pcg64_kernel(PcgArgs a) {
    extern __shared__ __align__(128) char dyn[];
    __shared__ Shared sh;
    Pipe pipe;
    pipe_init(sh, pipe, dyn);
    const int G = gridDim.x;
    const int n0 = static_cast<int>(static_cast<long long>(a.nb) * blockIdx.x / G);
    const int n1 = static_cast<int>(static_cast<long long>(a.nb) * (blockIdx.x + 1) / G);
    unsigned long long episode = 0;
    int slot = 0;
    auto next_target = [&]() { return (++episode) * static_cast<unsigned long long>(G); };
    auto next_slot = [&]() {
        slot = (slot + 1) % kSlots;
        return slot;
    };
    double* __restrict__ rd = a.r;
    double* __restrict__ pd = a.p;
    double* __restrict__ qd = a.q;
    const double* __restrict__ fd = a.f;
    double2* x2 = reinterpret_cast<double2*>(a.x);
    double2* r2 = reinterpret_cast<double2*>(a.r);
    double2* z2 = reinterpret_cast<double2*>(a.z);
    double2* p2 = reinterpret_cast<double2*>(a.p);
    double2* q2 = reinterpret_cast<double2*>(a.q);
    const double2* f2 = reinterpret_cast<const double2*>(a.f);
    PhaseClock clk;

    // r0 = f - K x0 (x0 = 0 when no warm start).
    if (a.x0) {
        struct {
            double* r;
            const double* f;
            __device__ void row(int i, double y) { r[i] = f[i] - y; }
            __device__ void node(int i, double2 y) {
                r[2 * i] = f[2 * i] - y.x;
                r[2 * i + 1] = f[2 * i + 1] - y.y;
            }
        } res{rd, fd};
        if (!product64<STORAGE>(a, pipe, a.x0, res)) {
            write_result(a, 0, 0, 0.0, 0.0, LFGPU_ERR_TIMEOUT, 0, 0, nullptr);
            return;
        }
        __syncthreads();
    }
    double v2[2] = {0.0, 0.0};
    for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
        const double2 rv = a.x0 ? r2[i] : f2[i];
        double2 zv;
        if (PRECOND == LFGPU_PRECOND_JACOBI) {
            zv = make_double2(a.invd64[2 * i] * rv.x, a.invd64[2 * i + 1] * rv.y);
        } else {
            zv = block2_apply(a.blk64, i, rv.x, rv.y);
        }
        r2[i] = rv;
        z2[i] = zv;
        p2[i] = zv;
        x2[i] = a.x0 ? reinterpret_cast<const double2*>(a.x0)[i] : make_double2(0.0, 0.0);
        v2[0] += rv.x * rv.x + rv.y * rv.y;
        v2[1] += rv.x * zv.x + rv.y * zv.y;
    }
    if (!grid_sum<2>(v2, a.partials, next_slot(), a.bar, next_target(), a.status, sh.red, &sh.flag)) {
        write_result(a, 0, 0, 0.0, 0.0, LFGPU_ERR_TIMEOUT, 0, 0, nullptr);
        return;
    }
    const double r0 = sqrt(fmax(0.0, v2[0]));
    double rho = v2[1];
    double rnorm = r0;
    if (r0 <= a.target) {
        write_result(a, 0, 0, r0, r0, LFGPU_OK, 1, 0, nullptr);
        return;
    }
    if (!(rho > 0.0) || !isfinite(rho)) {
        write_result(a, 0, 0, r0, r0, LFGPU_ERR_RHO_INITIAL, 0, 0, nullptr);
        return;
    }

    long long it = 0;
    int status = LFGPU_OK, converged = 0;
    clk.start();
    for (it = 1; it <= a.maxit; ++it) {
        // Phase 1: q = K p, partial p.q
        double v1[1] = {0.0};
        struct {
            double* q;
            const double* p;
            double* dot;
            __device__ void row(int i, double y) {
                q[i] = y;
                *dot += p[i] * y;
            }
            __device__ void node(int i, double2 y) {
                reinterpret_cast<double2*>(q)[i] = y;
                const double2 pv = reinterpret_cast<const double2*>(p)[i];
                *dot += pv.x * y.x + pv.y * y.y;
            }
        } qo{qd, pd, &v1[0]};
        if (!product64<STORAGE>(a, pipe, pd, qo)) {
            status = LFGPU_ERR_TIMEOUT;
            break;
        }
        clk.mark(0);
        if (!grid_sum<1>(v1, a.partials, next_slot(), a.bar, next_target(), a.status, sh.red, &sh.flag)) {
            status = LFGPU_ERR_TIMEOUT;
            break;
        }
        clk.mark(1);
        const double curvature = v1[0];
        if (!(curvature > 0.0) || !isfinite(curvature)) {
            status = LFGPU_ERR_NOT_SPD;
            break;
        }
        const double alpha = rho / curvature;

        // Phase 2: x, r, z and the two dot products
        double v[2] = {0.0, 0.0};
#pragma unroll 2
        for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
            const double2 pv = p2[i], qv = q2[i];
            double2 xv = x2[i], rv = r2[i];
            xv.x += alpha * pv.x;
            xv.y += alpha * pv.y;
            rv.x -= alpha * qv.x;
            rv.y -= alpha * qv.y;
            double2 zv;
            if (PRECOND == LFGPU_PRECOND_JACOBI) {
                const double2 dv = reinterpret_cast<const double2*>(a.invd64)[i];
                zv = make_double2(dv.x * rv.x, dv.y * rv.y);
            } else {
                zv = block2_apply(a.blk64, i, rv.x, rv.y);
            }
            x2[i] = xv;
            r2[i] = rv;
            z2[i] = zv;
            v[0] += rv.x * rv.x + rv.y * rv.y;
            v[1] += rv.x * zv.x + rv.y * zv.y;
        }
        clk.mark(2);
        if (!grid_sum<2>(v, a.partials, next_slot(), a.bar, next_target(), a.status, sh.red, &sh.flag)) {
            status = LFGPU_ERR_TIMEOUT;
            break;
        }
        clk.mark(3);
        rnorm = sqrt(fmax(0.0, v[0]));
        if (rnorm <= a.target) {
            converged = 1;
            break;
        }
        const double next_rho = v[1];
        if (!(next_rho > 0.0) || !isfinite(next_rho)) {
            status = LFGPU_ERR_RHO;
            break;
        }
        const double beta = next_rho / rho;
        rho = next_rho;

        // Phase 3: p = z + beta p
#pragma unroll 2
        for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
            const double2 zv = z2[i];
            double2 pv = p2[i];
            pv.x = zv.x + beta * pv.x;
            pv.y = zv.y + beta * pv.y;
            p2[i] = pv;
        }
        clk.mark(4);
        if (!grid_barrier(a.bar, next_target(), a.status, &sh.flag)) {
            status = LFGPU_ERR_TIMEOUT;
            break;
        }
        clk.mark(5);
    }
    if (it > a.maxit) it = a.maxit;
    write_result(a, it, 0, r0, rnorm, status, converged, 0, clk.t);
}

// ------------------------------------------------------------------ mixed precision
__device__ __forceinline__ float pnew(float z, float p, float beta) { return __fmaf_rn(beta, p, z); }

// Compensated diagonal term of the FP32 matrix: off + (hi + lo) x.
__device__ __forceinline__ float with_diag(float off, float hi, float lo, float x) { return fmaf(hi, x, off) + lo * x; }

template <int STORAGE, int PRECOND>
__global__ void __launch_bounds__(kPcgThreads) pcg_mixed_kernel(PcgArgs a) {
    extern __shared__ __align__(128) char dyn[];
    __shared__ Shared sh;
    Pipe pipe;
    pipe_init(sh, pipe, dyn);
    const int G = gridDim.x;
    const int n0 = static_cast<int>(static_cast<long long>(a.nb) * blockIdx.x / G);
    const int n1 = static_cast<int>(static_cast<long long>(a.nb) * (blockIdx.x + 1) / G);
    unsigned long long episode = 0;
    int slot = 0;
    auto next_target = [&]() { return (++episode) * static_cast<unsigned long long>(G); };
    auto next_slot = [&]() {
        slot = (slot + 1) % kSlots;
        return slot;
    };
    double2* x2 = reinterpret_cast<double2*>(a.x);
    double2* r64 = reinterpret_cast<double2*>(a.r64);
    const double2* f2 = reinterpret_cast<const double2*>(a.f);
    float2* r32 = reinterpret_cast<float2*>(a.r32);
    float2* z32 = reinterpret_cast<float2*>(a.z32);
    float2* q32 = reinterpret_cast<float2*>(a.q32);
    PhaseClock clk;

    auto precond = [&](int i, float2 rv) {
        if (PRECOND == LFGPU_PRECOND_JACOBI) {
            const float2 dv = reinterpret_cast<const float2*>(a.invd32)[i];
            return make_float2(dv.x * rv.x, dv.y * rv.y);
        }
        return block2_apply32(a.blk32, i, rv.x, rv.y);
    };

    // x = 0, r64 = f, r32 = f, z = M r, p buffers zero.
    double v2[2] = {0.0, 0.0};
    for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
        const double2 fv = f2[i];
        const float2 rv = make_float2(static_cast<float>(fv.x), static_cast<float>(fv.y));
        const float2 zv = precond(i, rv);
        x2[i] = make_double2(0.0, 0.0);
        r64[i] = fv;
        r32[i] = rv;
        z32[i] = zv;
        reinterpret_cast<float2*>(a.pa32)[i] = make_float2(0.f, 0.f);
        reinterpret_cast<float2*>(a.pb32)[i] = make_float2(0.f, 0.f);
        v2[0] += fv.x * fv.x + fv.y * fv.y;
        v2[1] += static_cast<double>(rv.x * zv.x + rv.y * zv.y);
    }
    if (!grid_sum<2>(v2, a.partials, next_slot(), a.bar, next_target(), a.status, sh.red, &sh.flag)) {
        write_result(a, 0, 0, 0.0, 0.0, LFGPU_ERR_TIMEOUT, 0, 0, nullptr);
        return;
    }
    const double r0 = sqrt(fmax(0.0, v2[0]));
    double rho = v2[1];
    if (r0 <= a.target) {
        write_result(a, 0, 0, r0, r0, LFGPU_OK, 1, 0, nullptr);
        return;
    }
    if (!(rho > 0.0) || !isfinite(rho)) {
        write_result(a, 0, 0, r0, r0, LFGPU_ERR_RHO_INITIAL, 0, 0, nullptr);
        return;
    }

    float beta = 0.f;
    float* p_old = a.pa32;
    float* p_cur = a.pb32;
    double rmax = r0, rtrue_prev = r0, rtrue = r0;
    long long it = 0, refs = 0;
    int status = LFGPU_OK, converged = 0, stagnated = 0, no_progress = 0;
    clk.start();
    for (it = 1; it <= a.maxit; ++it) {
        // Phase 1: p = z + beta p_old (own rows), q = K32 p with p gathered on the fly
        float acc = 0.f;
        bool ok;
        if (STORAGE == LFGPU_STORAGE_CSR) {
            const float* zz = a.z32;
            const float* po = p_old;
            float* pc = p_cur;
            float* qq = a.q32;
            ok = product<kCsr32>(a.mat32, pipe, a.status, [&](int c) { return pnew(zz[c], po[c], beta); },
                                 [&](int row, float off) {
                                     const float pn = pnew(zz[row], po[row], beta);
                                     const float y = with_diag(off, a.dhi[row], a.dlo[row], pn);
                                     pc[row] = pn;
                                     qq[row] = y;
                                     acc += pn * y;
                                 });
        } else {
            const float2* po2 = reinterpret_cast<const float2*>(p_old);
            float2* pc2 = reinterpret_cast<float2*>(p_cur);
            const float2* hi2 = reinterpret_cast<const float2*>(a.dhi);
            const float2* lo2 = reinterpret_cast<const float2*>(a.dlo);
            ok = product<kBsr32>(a.mat32, pipe, a.status,
                                 [&](int c) {
                                     const float2 zv = z32[c], pv = po2[c];
                                     return make_float2(pnew(zv.x, pv.x, beta), pnew(zv.y, pv.y, beta));
                                 },
                                 [&](int node, float2 off) {
                                     const float2 zv = z32[node], pv = po2[node];
                                     const float2 pn = make_float2(pnew(zv.x, pv.x, beta), pnew(zv.y, pv.y, beta));
                                     const float2 h = hi2[node], l = lo2[node];
                                     const float2 y = make_float2(with_diag(off.x, h.x, l.x, pn.x),
                                                                  with_diag(off.y, h.y, l.y, pn.y));
                                     pc2[node] = pn;
                                     q32[node] = y;
                                     acc += pn.x * y.x + pn.y * y.y;
                                 });
        }
        if (!ok) {
            status = LFGPU_ERR_TIMEOUT;
            break;
        }
        double v1[1] = {acc};
        clk.mark(0);
        if (!grid_sum<1>(v1, a.partials, next_slot(), a.bar, next_target(), a.status, sh.red, &sh.flag)) {
            status = LFGPU_ERR_TIMEOUT;
            break;
        }
        clk.mark(1);
        const double curvature = v1[0];
        if (!(curvature > 0.0) || !isfinite(curvature)) {
            status = LFGPU_ERR_NOT_SPD;
            break;
        }
        const double alpha64 = rho / curvature;
        const float alpha = static_cast<float>(alpha64);

        // Phase 2: FP64 solution update, FP32 residual and preconditioned residual
        float s_rr = 0.f, s_rz = 0.f;
        const float2* pc2 = reinterpret_cast<const float2*>(p_cur);
#pragma unroll 2
        for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
            const float2 pv = pc2[i], qv = q32[i];
            double2 xv = x2[i];
            float2 rv = r32[i];
            xv.x += alpha64 * static_cast<double>(pv.x);
            xv.y += alpha64 * static_cast<double>(pv.y);
            rv.x -= alpha * qv.x;
            rv.y -= alpha * qv.y;
            const float2 zv = precond(i, rv);
            x2[i] = xv;
            r32[i] = rv;
            z32[i] = zv;
            s_rr += rv.x * rv.x + rv.y * rv.y;
            s_rz += rv.x * zv.x + rv.y * zv.y;
        }
        double v[2] = {s_rr, s_rz};
        clk.mark(2);
        if (!grid_sum<2>(v, a.partials, next_slot(), a.bar, next_target(), a.status, sh.red, &sh.flag)) {
            status = LFGPU_ERR_TIMEOUT;
            break;
        }
        clk.mark(3);
        const double rn = sqrt(fmax(0.0, v[0]));
        double next_rho = v[1];
        rmax = fmax(rmax, rn);
        bool restart_now = false;
        if (rn <= a.reduction * rmax || rn <= a.target || it == a.maxit) {
            // Residual replacement: r64 = f - K64 x, tested in FP64, copied to r32.
            ++refs;
            double vr[1] = {0.0};
            struct {
                double2* r64;
                float2* r32;
                const double2* f;
                double* dot;
                __device__ void node(int i, double2 y) {
                    const double2 fv = f[i];
                    const double2 rv = make_double2(fv.x - y.x, fv.y - y.y);
                    r64[i] = rv;
                    r32[i] = make_float2(static_cast<float>(rv.x), static_cast<float>(rv.y));
                    *dot += rv.x * rv.x + rv.y * rv.y;
                }
                __device__ void row(int i, double y) {
                    const double rv = reinterpret_cast<const double*>(f)[i] - y;
                    reinterpret_cast<double*>(r64)[i] = rv;
                    reinterpret_cast<float*>(r32)[i] = static_cast<float>(rv);
                    *dot += rv * rv;
                }
            } ro{r64, r32, f2, &vr[0]};
            if (!product64<STORAGE>(a, pipe, a.x, ro)) {
                status = LFGPU_ERR_TIMEOUT;
                break;
            }
            if (!grid_sum<1>(vr, a.partials, next_slot(), a.bar, next_target(), a.status, sh.red, &sh.flag)) {
                status = LFGPU_ERR_TIMEOUT;
                break;
            }
            rtrue = sqrt(fmax(0.0, vr[0]));
            if (rtrue <= a.target) {
                converged = 1;
                break;
            }
            if (refs >= a.max_ref || it == a.maxit) break;
            no_progress = rtrue >= rtrue_prev ? no_progress + 1 : 0;
            if (no_progress >= 3) {
                stagnated = 1;
                break;
            }
            rtrue_prev = fmin(rtrue_prev, rtrue);
            rmax = rtrue;
            restart_now = a.restart != 0;
            float s_rz2 = 0.f;
            for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
                const float2 rv = r32[i];
                const float2 zv = precond(i, rv);
                z32[i] = zv;
                s_rz2 += rv.x * zv.x + rv.y * zv.y;
            }
            double vz[1] = {s_rz2};
            if (!grid_sum<1>(vz, a.partials, next_slot(), a.bar, next_target(), a.status, sh.red, &sh.flag)) {
                status = LFGPU_ERR_TIMEOUT;
                break;
            }
            next_rho = vz[0];
            clk.mark(4);
        }
        if (!(next_rho > 0.0) || !isfinite(next_rho)) {
            status = LFGPU_ERR_RHO;
            break;
        }
        beta = restart_now ? 0.f : static_cast<float>(next_rho / rho);
        rho = next_rho;
        float* t = p_old;
        p_old = p_cur;
        p_cur = t;
    }
    if (it > a.maxit) it = a.maxit;
    write_result(a, it, refs, r0, rtrue, status, converged, stagnated, clk.t);
}

// Build (or reuse) the tile schedule of one format for a grid of G CTAs.
const Context::Schedule& schedule(Context& c, int format, int G) {
    Context::Schedule& s = c.sched[format];
    if (s.version == c.pattern_version && s.grid == G) return s;
    const bool bsr = format == kBsr64 || format == kBsr32;
    const std::vector<int>& ptr = bsr ? c.h_brow : c.h_rowptr_cache;
    const int T = tile_units(format);
    const int nb = static_cast<int>(c.n / 2);
    std::vector<int2> tiles;
    std::vector<int> cta(static_cast<size_t>(G) + 1, 0);
    for (int b = 0; b < G; ++b) {
        const int n0 = static_cast<int>(static_cast<long long>(nb) * b / G);
        const int n1 = static_cast<int>(static_cast<long long>(nb) * (b + 1) / G);
        const int r1 = bsr ? n1 : 2 * n1;
        int r = bsr ? n0 : 2 * n0;
        cta[b] = static_cast<int>(tiles.size());
        while (r < r1) {
            const int start = r;
            while (r < r1 && ptr[r + 1] - ptr[start] <= T) ++r;
            LF_REQUIRE(r > start, LFGPU_ERR_UNSUPPORTED, "a matrix row is longer than one streaming tile");
            tiles.push_back(make_int2(start, r));
        }
    }
    cta[G] = static_cast<int>(tiles.size());
    s.tiles.ensure(std::max<size_t>(tiles.size(), 1));
    s.cta.ensure(cta.size());
    if (!tiles.empty())
        LF_CUDA(cudaMemcpyAsync(s.tiles.p, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                c.stream));
    LF_CUDA(cudaMemcpyAsync(s.cta.p, cta.data(), cta.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    LF_CUDA(cudaStreamSynchronize(c.stream));
    s.grid = G;
    s.units = T;
    s.version = c.pattern_version;
    return s;
}

TileSet tileset(Context& c, int format, int G) {
    const Context::Schedule& s = schedule(c, format, G);
    TileSet t{};
    const bool bsr = format == kBsr64 || format == kBsr32;
    t.ptr = bsr ? c.brow.p : c.rowptr.p;
    t.cols = bsr ? c.bcol.p : c.col.p;
    switch (format) {
        case kCsr64: t.vals = reinterpret_cast<const char*>(c.K.p); break;
        case kCsr32: t.vals = reinterpret_cast<const char*>(c.K32.p); break;
        case kBsr64: t.vals = reinterpret_cast<const char*>(c.bval64.p); break;
        default: t.vals = reinterpret_cast<const char*>(c.bval32.p); break;
    }
    t.tiles = s.tiles;
    t.cta = s.cta;
    t.unit_bytes = kUnitBytes[format];
    t.cols_offset = ((s.units + kSlack) * kUnitBytes[format] + 127) / 128 * 128;
    return t;
}

template <typename K>
void launch_coop(Context& c, K kernel, PcgArgs& args, bool mixed, int storage, float* ms) {
    LF_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kDynSmem));
    int occ = 0;
    LF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kPcgThreads, kDynSmem));
    LF_REQUIRE(occ > 0, LFGPU_ERR_CUDA, "PCG kernel cannot be resident");
    const int per_sm = occ >= 2 ? 2 : 1;
    const int grid = c.num_sms * per_sm;
    const bool bsr = storage == LFGPU_STORAGE_BSR;
    args.mat64 = tileset(c, bsr ? kBsr64 : kCsr64, grid);
    if (mixed) args.mat32 = tileset(c, bsr ? kBsr32 : kCsr32, grid);
    c.partials.ensure(static_cast<size_t>(kSlots) * kMaxReduce * grid);
    c.bar.ensure(1);
    LF_CUDA(cudaMemsetAsync(c.bar.p, 0, sizeof(unsigned long long), c.stream));
    args.partials = c.partials;
    args.bar = c.bar;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kPcgThreads);
    cfg.dynamicSmemBytes = kDynSmem;
    cfg.stream = c.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    LF_CUDA(cudaEventRecord(c.ev_a, c.stream));
    LF_CUDA(cudaLaunchKernelEx(&cfg, kernel, args));
    c.launches += 1;
    LF_CUDA(cudaEventRecord(c.ev_b, c.stream));
    *ms = elapsed_ms(c);
}

}  // namespace

PcgResult run_pcg(Context& c, const SolveSetup& s, float* kernel_ms) {
    const i64 n = c.n;
    LF_REQUIRE(n % 2 == 0, LFGPU_ERR_ARGUMENT, "the GPU PCG needs an even number of DOFs (u,v pairs)");
    PcgArgs a{};
    a.nb = static_cast<int>(n / 2);
    a.invd64 = c.inv_diag64;
    a.blk64 = c.blk64;
    a.invd32 = c.inv_diag32;
    a.blk32 = c.blk32;
    a.f = s.rhs;
    a.x0 = s.x0;
    a.x = s.x;
    a.target = s.tolerance;  // absolute target, computed by the caller
    a.maxit = s.max_iterations;
    a.reduction = s.inner_reduction;
    a.max_ref = s.max_refinements;
    a.restart = s.restart;
    a.status = c.status;
    c.pcg_result.ensure(1);
    a.result = c.pcg_result;
    for (auto& b : c.v64) b.ensure(n);
    a.r = c.v64[0];
    a.z = c.v64[1];
    a.p = c.v64[2];
    a.q = c.v64[3];
    a.r64 = c.v64[4];
    if (s.storage == LFGPU_STORAGE_BSR) ensure_bsr(c);
    if (s.mixed) {
        for (auto& b : c.v32) b.ensure(n);
        a.r32 = c.v32[0];
        a.z32 = c.v32[1];
        a.pa32 = c.v32[2];
        a.pb32 = c.v32[3];
        a.q32 = c.v32[4];
        if (s.storage == LFGPU_STORAGE_BSR) ensure_bsr32(c);
        else ensure_csr32(c);
        a.dhi = c.diag_hi;
        a.dlo = c.diag_lo;
    }
    const int st = s.storage;
    const bool csr = st == LFGPU_STORAGE_CSR;
    const bool jac = s.precond == LFGPU_PRECOND_JACOBI;
    const bool mx = s.mixed != 0;
    if (!mx) {
        if (csr && jac) launch_coop(c, pcg64_kernel<LFGPU_STORAGE_CSR, LFGPU_PRECOND_JACOBI>, a, mx, st, kernel_ms);
        else if (csr) launch_coop(c, pcg64_kernel<LFGPU_STORAGE_CSR, LFGPU_PRECOND_BLOCK2>, a, mx, st, kernel_ms);
        else if (jac) launch_coop(c, pcg64_kernel<LFGPU_STORAGE_BSR, LFGPU_PRECOND_JACOBI>, a, mx, st, kernel_ms);
        else launch_coop(c, pcg64_kernel<LFGPU_STORAGE_BSR, LFGPU_PRECOND_BLOCK2>, a, mx, st, kernel_ms);
    } else {
        if (csr && jac) launch_coop(c, pcg_mixed_kernel<LFGPU_STORAGE_CSR, LFGPU_PRECOND_JACOBI>, a, mx, st, kernel_ms);
        else if (csr) launch_coop(c, pcg_mixed_kernel<LFGPU_STORAGE_CSR, LFGPU_PRECOND_BLOCK2>, a, mx, st, kernel_ms);
        else if (jac) launch_coop(c, pcg_mixed_kernel<LFGPU_STORAGE_BSR, LFGPU_PRECOND_JACOBI>, a, mx, st, kernel_ms);
        else launch_coop(c, pcg_mixed_kernel<LFGPU_STORAGE_BSR, LFGPU_PRECOND_BLOCK2>, a, mx, st, kernel_ms);
    }
    PcgResult res{};
    LF_CUDA(cudaMemcpyAsync(&res, c.pcg_result.p, sizeof(res), cudaMemcpyDeviceToHost, c.stream));
    check_status(c);
    return res;
}

}  // namespace lfgpu
