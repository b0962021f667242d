// Persistent preconditioned CG: the whole Krylov loop in one cooperative launch.
//
// Replaces pcg_solve<Matrix, Preconditioner> (src/solver.cpp:532-627) for CSR and
// 2x2 BSR storage (src/sparse.cpp:104-120, :179-204) with the Jacobi
// (src/solver.cpp:497-509) or 2x2 nodal block-Jacobi (src/precond.cpp:242-291 with
// one node per subdomain) preconditioner.
//
// Layout: every CTA owns a contiguous range of nodes (2 DOFs each) for the whole
// solve.  One iteration is three phases separated by grid-wide barriers:
//   1. q = K p over the CTA's rows (a quarter warp per CSR row / BSR block row),
//      partial p.q
//   2. alpha; x += alpha p; r -= alpha q; z = M^-1 r; partial r.r and r.z
//   3. beta; p = z + beta p
// Grid sums are published per CTA and added in CTA order by every CTA, so every
// CTA takes the same decisions from bit-identical scalars and a run is
// deterministic.  Barriers are bounded in time (common.cuh): a stuck wait records
// LFGPU_ERR_TIMEOUT and every CTA leaves the loop.
//
// The mixed-precision kernel runs the same recurrence with K, the preconditioner
// and every Krylov vector in FP32, inside FP64 iterative refinement: the solution
// lives in FP64, and whenever the FP32 recursive residual has dropped by
// `reduction` since the last refinement (or claims convergence), the FP32
// correction is added to the FP64 solution, the true residual r = f - K u is
// recomputed in FP64 with the FP64 matrix, tested against the tolerance, and
// replaces the FP32 residual.  The search direction is kept across the update
// (reliable updates, Sleijpen & van der Vorst 1996), or dropped (classic restarted
// refinement) when `restart` is set.  In FP32 the p update is folded into the
// product: phase 1 gathers z + beta p_old on the fly and each CTA writes p for its
// own rows into the other buffer, which saves the third barrier.
#include "common.cuh"
#include "kernels.hpp"

namespace lfgpu {
namespace {

constexpr int kPcgThreads = 512;

struct PcgArgs {
    int nb;
    const int* rowptr;
    const int* col;
    const double* val64;
    const float* val32;
    const int* brow;
    const int* bcol;
    const double2* bval64;  // two double2 per block: (a00, a01), (a10, a11)
    const float4* bval32;
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
    float* x32;
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

// ------------------------------------------------------------------ products
// CSR, 8 lanes per node: lanes 0-3 sum row 2i, lanes 4-7 row 2i+1.  Lane 0 of the
// group returns both row sums.
template <typename T, typename Gather>
__device__ __forceinline__ void csr_node(bool active, int node, int sub, const int* __restrict__ rowptr,
                                         const int* __restrict__ col, const T* __restrict__ val, const Gather& g,
                                         T& y0, T& y1) {
    T s = T(0);
    if (active) {
        const int row = 2 * node + (sub >> 2);
        const int b = __ldg(rowptr + row), e = __ldg(rowptr + row + 1);
        for (int k = b + (sub & 3); k < e; k += 4) s += ld_stream(val + k) * g(ld_stream(col + k));
    }
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    y0 = s;
    y1 = __shfl_down_sync(0xffffffffu, s, 4);
}

// BSR FP64, 4 lanes per block row.
template <typename Gather2>
__device__ __forceinline__ void bsr_node64(bool active, int node, int sub, const int* __restrict__ brow,
                                           const int* __restrict__ bcol, const double2* __restrict__ bval,
                                           const Gather2& g, double& y0, double& y1) {
    double s0 = 0.0, s1 = 0.0;
    if (active) {
        const int b = __ldg(brow + node), e = __ldg(brow + node + 1);
        for (int k = b + sub; k < e; k += 4) {
            const double2 top = ld_stream(bval + 2 * static_cast<size_t>(k));
            const double2 bot = ld_stream(bval + 2 * static_cast<size_t>(k) + 1);
            const double2 xv = g(ld_stream(bcol + k));
            s0 += top.x * xv.x + top.y * xv.y;
            s1 += bot.x * xv.x + bot.y * xv.y;
        }
    }
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
    s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
    y0 = s0;
    y1 = s1;
}

template <typename Gather2>
__device__ __forceinline__ void bsr_node32(bool active, int node, int sub, const int* __restrict__ brow,
                                           const int* __restrict__ bcol, const float4* __restrict__ bval,
                                           const Gather2& g, float& y0, float& y1) {
    float s0 = 0.f, s1 = 0.f;
    if (active) {
        const int b = __ldg(brow + node), e = __ldg(brow + node + 1);
        for (int k = b + sub; k < e; k += 4) {
            const float4 v = ld_stream(bval + k);
            const float2 xv = g(ld_stream(bcol + k));
            s0 += v.x * xv.x + v.y * xv.y;
            s1 += v.z * xv.x + v.w * xv.y;
        }
    }
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
    s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
    y0 = s0;
    y1 = s1;
}

// Visit the CTA's nodes [n0, n1) with LPN lanes per node; f(active, node, sub,
// leader) is called by every lane of the warp each step (shuffles need all lanes).
template <int LPN, typename F>
__device__ __forceinline__ void for_nodes_grouped(int n0, int n1, F&& f) {
    constexpr int kNodesPerWarp = 32 / LPN;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int sub = lane & (LPN - 1);
    for (int base = n0 + warp * kNodesPerWarp; base < n1; base += nwarps * kNodesPerWarp) {
        const int node = base + lane / LPN;
        f(node < n1, node, sub, sub == 0);
    }
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
                                             int status, int converged, int stagnated) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.result->iterations = it;
        a.result->refinements = refs;
        a.result->initial_residual = r0;
        a.result->final_residual = rf;
        a.result->status = status;
        a.result->converged = converged;
        a.result->stagnated = stagnated;
    }
}

// ------------------------------------------------------------------ FP64 PCG
template <int STORAGE, int PRECOND>
__global__ void __launch_bounds__(kPcgThreads) pcg64_kernel(PcgArgs a) {
    __shared__ double s_red[32 * kMaxReduce];
    __shared__ int s_flag;
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
    double2* r2 = reinterpret_cast<double2*>(a.r);
    double2* z2 = reinterpret_cast<double2*>(a.z);
    double2* p2 = reinterpret_cast<double2*>(a.p);
    double2* q2 = reinterpret_cast<double2*>(a.q);
    const double2* f2 = reinterpret_cast<const double2*>(a.f);

    // r0 = f - K x0 (x0 = 0 when no warm start).
    if (a.x0) {
        const double* x0 = a.x0;
        if (STORAGE == LFGPU_STORAGE_CSR) {
            for_nodes_grouped<8>(n0, n1, [&](bool act, int node, int sub, bool lead) {
                double y0, y1;
                csr_node<double>(act, node, sub, a.rowptr, a.col, a.val64, [&](int c) { return x0[c]; }, y0, y1);
                if (act && lead) {
                    const double2 fv = f2[node];
                    r2[node] = make_double2(fv.x - y0, fv.y - y1);
                }
            });
        } else {
            const double2* x02 = reinterpret_cast<const double2*>(x0);
            for_nodes_grouped<4>(n0, n1, [&](bool act, int node, int sub, bool lead) {
                double y0, y1;
                bsr_node64(act, node, sub, a.brow, a.bcol, a.bval64, [&](int c) { return x02[c]; }, y0, y1);
                if (act && lead) {
                    const double2 fv = f2[node];
                    r2[node] = make_double2(fv.x - y0, fv.y - y1);
                }
            });
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
    if (!grid_sum<2>(v2, a.partials, next_slot(), a.bar, next_target(), a.status, s_red, &s_flag)) {
        write_result(a, 0, 0, 0.0, 0.0, LFGPU_ERR_TIMEOUT, 0, 0);
        return;
    }
    const double r0 = sqrt(fmax(0.0, v2[0]));
    double rho = v2[1];
    double rnorm = r0;
    if (r0 <= a.target) {
        write_result(a, 0, 0, r0, r0, LFGPU_OK, 1, 0);
        return;
    }
    if (!(rho > 0.0) || !isfinite(rho)) {
        write_result(a, 0, 0, r0, r0, LFGPU_ERR_RHO_INITIAL, 0, 0);
        return;
    }

    long long it = 0;
    int status = LFGPU_OK, converged = 0;
    for (it = 1; it <= a.maxit; ++it) {
        // Phase 1: q = K p, partial p.q
        double v1[1] = {0.0};
        if (STORAGE == LFGPU_STORAGE_CSR) {
            const double* p = a.p;
            for_nodes_grouped<8>(n0, n1, [&](bool act, int node, int sub, bool lead) {
                double y0, y1;
                csr_node<double>(act, node, sub, a.rowptr, a.col, a.val64, [&](int c) { return p[c]; }, y0, y1);
                if (act && lead) {
                    q2[node] = make_double2(y0, y1);
                    const double2 pv = p2[node];
                    v1[0] += pv.x * y0 + pv.y * y1;
                }
            });
        } else {
            for_nodes_grouped<4>(n0, n1, [&](bool act, int node, int sub, bool lead) {
                double y0, y1;
                bsr_node64(act, node, sub, a.brow, a.bcol, a.bval64, [&](int c) { return p2[c]; }, y0, y1);
                if (act && lead) {
                    q2[node] = make_double2(y0, y1);
                    const double2 pv = p2[node];
                    v1[0] += pv.x * y0 + pv.y * y1;
                }
            });
        }
        if (!grid_sum<1>(v1, a.partials, next_slot(), a.bar, next_target(), a.status, s_red, &s_flag)) {
            status = LFGPU_ERR_TIMEOUT;
            break;
        }
        const double curvature = v1[0];
        if (!(curvature > 0.0) || !isfinite(curvature)) {
            status = LFGPU_ERR_NOT_SPD;
            break;
        }
        const double alpha = rho / curvature;

        // Phase 2: x, r, z and the two dot products
        double v[2] = {0.0, 0.0};
        for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
            const double2 pv = p2[i], qv = q2[i];
            double2 xv = x2[i], rv = r2[i];
            xv.x += alpha * pv.x;
            xv.y += alpha * pv.y;
            rv.x -= alpha * qv.x;
            rv.y -= alpha * qv.y;
            double2 zv;
            if (PRECOND == LFGPU_PRECOND_JACOBI) {
                zv = make_double2(a.invd64[2 * i] * rv.x, a.invd64[2 * i + 1] * rv.y);
            } else {
                zv = block2_apply(a.blk64, i, rv.x, rv.y);
            }
            x2[i] = xv;
            r2[i] = rv;
            z2[i] = zv;
            v[0] += rv.x * rv.x + rv.y * rv.y;
            v[1] += rv.x * zv.x + rv.y * zv.y;
        }
        if (!grid_sum<2>(v, a.partials, next_slot(), a.bar, next_target(), a.status, s_red, &s_flag)) {
            status = LFGPU_ERR_TIMEOUT;
            break;
        }
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
        for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
            const double2 zv = z2[i];
            double2 pv = p2[i];
            pv.x = zv.x + beta * pv.x;
            pv.y = zv.y + beta * pv.y;
            p2[i] = pv;
        }
        if (!grid_barrier(a.bar, next_target(), a.status, &s_flag)) {
            status = LFGPU_ERR_TIMEOUT;
            break;
        }
    }
    if (it > a.maxit) it = a.maxit;
    write_result(a, it, 0, r0, rnorm, status, converged, 0);
}

// ------------------------------------------------------------------ mixed precision
__device__ __forceinline__ float pnew(float z, float p, float beta) { return __fmaf_rn(beta, p, z); }

template <int STORAGE, int PRECOND>
__global__ void __launch_bounds__(kPcgThreads) pcg_mixed_kernel(PcgArgs a) {
    __shared__ double s_red[32 * kMaxReduce];
    __shared__ int s_flag;
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
    float2* c32 = reinterpret_cast<float2*>(a.x32);

    auto precond = [&](int i, float2 rv) {
        if (PRECOND == LFGPU_PRECOND_JACOBI) return make_float2(a.invd32[2 * i] * rv.x, a.invd32[2 * i + 1] * rv.y);
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
        c32[i] = make_float2(0.f, 0.f);
        reinterpret_cast<float2*>(a.pa32)[i] = make_float2(0.f, 0.f);
        reinterpret_cast<float2*>(a.pb32)[i] = make_float2(0.f, 0.f);
        v2[0] += fv.x * fv.x + fv.y * fv.y;
        v2[1] += static_cast<double>(rv.x * zv.x + rv.y * zv.y);
    }
    if (!grid_sum<2>(v2, a.partials, next_slot(), a.bar, next_target(), a.status, s_red, &s_flag)) {
        write_result(a, 0, 0, 0.0, 0.0, LFGPU_ERR_TIMEOUT, 0, 0);
        return;
    }
    const double r0 = sqrt(fmax(0.0, v2[0]));
    double rho = v2[1];
    if (r0 <= a.target) {
        write_result(a, 0, 0, r0, r0, LFGPU_OK, 1, 0);
        return;
    }
    if (!(rho > 0.0) || !isfinite(rho)) {
        write_result(a, 0, 0, r0, r0, LFGPU_ERR_RHO_INITIAL, 0, 0);
        return;
    }

    float beta = 0.f;
    float* p_old = a.pa32;
    float* p_cur = a.pb32;
    double rmax = r0, rtrue_prev = r0, rtrue = r0;
    long long it = 0, refs = 0;
    int status = LFGPU_OK, converged = 0, stagnated = 0;
    for (it = 1; it <= a.maxit; ++it) {
        // Phase 1: p = z + beta p_old (own rows), q = K32 p with p gathered on the fly
        double v1[1] = {0.0};
        const float* zz = a.z32;
        const float* po = p_old;
        float2* pc2 = reinterpret_cast<float2*>(p_cur);
        const float2* po2 = reinterpret_cast<const float2*>(p_old);
        float acc = 0.f;
        if (STORAGE == LFGPU_STORAGE_CSR) {
            for_nodes_grouped<8>(n0, n1, [&](bool act, int node, int sub, bool lead) {
                float y0, y1;
                csr_node<float>(act, node, sub, a.rowptr, a.col, a.val32,
                                [&](int c) { return pnew(zz[c], po[c], beta); }, y0, y1);
                if (act && lead) {
                    const float2 zv = z32[node], pv = po2[node];
                    const float2 pn = make_float2(pnew(zv.x, pv.x, beta), pnew(zv.y, pv.y, beta));
                    pc2[node] = pn;
                    q32[node] = make_float2(y0, y1);
                    acc += pn.x * y0 + pn.y * y1;
                }
            });
        } else {
            for_nodes_grouped<4>(n0, n1, [&](bool act, int node, int sub, bool lead) {
                float y0, y1;
                bsr_node32(act, node, sub, a.brow, a.bcol, a.bval32,
                           [&](int c) {
                               const float2 zv = z32[c], pv = po2[c];
                               return make_float2(pnew(zv.x, pv.x, beta), pnew(zv.y, pv.y, beta));
                           },
                           y0, y1);
                if (act && lead) {
                    const float2 zv = z32[node], pv = po2[node];
                    const float2 pn = make_float2(pnew(zv.x, pv.x, beta), pnew(zv.y, pv.y, beta));
                    pc2[node] = pn;
                    q32[node] = make_float2(y0, y1);
                    acc += pn.x * y0 + pn.y * y1;
                }
            });
        }
        v1[0] = acc;
        if (!grid_sum<1>(v1, a.partials, next_slot(), a.bar, next_target(), a.status, s_red, &s_flag)) {
            status = LFGPU_ERR_TIMEOUT;
            break;
        }
        const double curvature = v1[0];
        if (!(curvature > 0.0) || !isfinite(curvature)) {
            status = LFGPU_ERR_NOT_SPD;
            break;
        }
        const float alpha = static_cast<float>(rho / curvature);

        // Phase 2: correction, residual, preconditioned residual
        float s_rr = 0.f, s_rz = 0.f;
        for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
            const float2 pv = pc2[i], qv = q32[i];
            float2 cv = c32[i], rv = r32[i];
            cv.x += alpha * pv.x;
            cv.y += alpha * pv.y;
            rv.x -= alpha * qv.x;
            rv.y -= alpha * qv.y;
            const float2 zv = precond(i, rv);
            c32[i] = cv;
            r32[i] = rv;
            z32[i] = zv;
            s_rr += rv.x * rv.x + rv.y * rv.y;
            s_rz += rv.x * zv.x + rv.y * zv.y;
        }
        double v[2] = {s_rr, s_rz};
        if (!grid_sum<2>(v, a.partials, next_slot(), a.bar, next_target(), a.status, s_red, &s_flag)) {
            status = LFGPU_ERR_TIMEOUT;
            break;
        }
        const double rn = sqrt(fmax(0.0, v[0]));
        double next_rho = v[1];
        rmax = fmax(rmax, rn);
        bool restart_now = false;
        if (rn <= a.reduction * rmax || rn <= a.target || it == a.maxit) {
            // FP64 refinement: u += c; r = f - K u; r32 = r
            ++refs;
            for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
                const float2 cv = c32[i];
                double2 xv = x2[i];
                xv.x += static_cast<double>(cv.x);
                xv.y += static_cast<double>(cv.y);
                x2[i] = xv;
                c32[i] = make_float2(0.f, 0.f);
            }
            if (!grid_barrier(a.bar, next_target(), a.status, &s_flag)) {
                status = LFGPU_ERR_TIMEOUT;
                break;
            }
            double vr[1] = {0.0};
            if (STORAGE == LFGPU_STORAGE_CSR) {
                const double* xx = a.x;
                for_nodes_grouped<8>(n0, n1, [&](bool act, int node, int sub, bool lead) {
                    double y0, y1;
                    csr_node<double>(act, node, sub, a.rowptr, a.col, a.val64, [&](int c) { return xx[c]; }, y0,
                                     y1);
                    if (act && lead) {
                        const double2 fv = f2[node];
                        const double2 rv = make_double2(fv.x - y0, fv.y - y1);
                        r64[node] = rv;
                        r32[node] = make_float2(static_cast<float>(rv.x), static_cast<float>(rv.y));
                        vr[0] += rv.x * rv.x + rv.y * rv.y;
                    }
                });
            } else {
                for_nodes_grouped<4>(n0, n1, [&](bool act, int node, int sub, bool lead) {
                    double y0, y1;
                    bsr_node64(act, node, sub, a.brow, a.bcol, a.bval64, [&](int c) { return x2[c]; }, y0, y1);
                    if (act && lead) {
                        const double2 fv = f2[node];
                        const double2 rv = make_double2(fv.x - y0, fv.y - y1);
                        r64[node] = rv;
                        r32[node] = make_float2(static_cast<float>(rv.x), static_cast<float>(rv.y));
                        vr[0] += rv.x * rv.x + rv.y * rv.y;
                    }
                });
            }
            if (!grid_sum<1>(vr, a.partials, next_slot(), a.bar, next_target(), a.status, s_red, &s_flag)) {
                status = LFGPU_ERR_TIMEOUT;
                break;
            }
            rtrue = sqrt(fmax(0.0, vr[0]));
            if (rtrue <= a.target) {
                converged = 1;
                break;
            }
            if (refs >= a.max_ref || it == a.maxit) break;
            if (rtrue >= rtrue_prev) {
                stagnated = 1;
                break;
            }
            rtrue_prev = rtrue;
            rmax = rtrue;
            restart_now = a.restart != 0;
            // z = M r32 for the replaced residual
            float s_rz2 = 0.f;
            for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
                const float2 rv = r32[i];
                const float2 zv = precond(i, rv);
                z32[i] = zv;
                s_rz2 += rv.x * zv.x + rv.y * zv.y;
            }
            double vz[1] = {s_rz2};
            if (!grid_sum<1>(vz, a.partials, next_slot(), a.bar, next_target(), a.status, s_red, &s_flag)) {
                status = LFGPU_ERR_TIMEOUT;
                break;
            }
            next_rho = vz[0];
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
    write_result(a, it, refs, r0, rtrue, status, converged, stagnated);
}

template <typename K>
void launch_coop(Context& c, K kernel, PcgArgs& args, float* ms) {
    int occ = 0;
    LF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kPcgThreads, 0));
    LF_REQUIRE(occ > 0, LFGPU_ERR_CUDA, "PCG kernel cannot be resident");
    const int per_sm = occ >= 2 ? 2 : 1;
    const int grid = c.num_sms * per_sm;
    c.partials.ensure(static_cast<size_t>(kSlots) * kMaxReduce * grid);
    c.bar.ensure(1);
    LF_CUDA(cudaMemsetAsync(c.bar.p, 0, sizeof(unsigned long long), c.stream));
    args.partials = c.partials;
    args.bar = c.bar;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kPcgThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = c.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    LF_CUDA(cudaEventRecord(c.ev_a, c.stream));
    LF_CUDA(cudaLaunchKernelEx(&cfg, kernel, args));
    LF_CUDA(cudaEventRecord(c.ev_b, c.stream));
    *ms = elapsed_ms(c);
}

}  // namespace

PcgResult run_pcg(Context& c, const SolveSetup& s, float* kernel_ms) {
    const i64 n = c.n;
    LF_REQUIRE(n % 2 == 0, LFGPU_ERR_ARGUMENT, "the GPU PCG needs an even number of DOFs (u,v pairs)");
    PcgArgs a{};
    a.nb = static_cast<int>(n / 2);
    a.rowptr = c.rowptr;
    a.col = c.col;
    a.val64 = c.K;
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
    if (s.storage == LFGPU_STORAGE_BSR) {
        ensure_bsr(c);
        a.brow = c.brow;
        a.bcol = c.bcol;
        a.bval64 = reinterpret_cast<const double2*>(c.bval64.p);
    }
    if (s.mixed) {
        for (auto& b : c.v32) b.ensure(n);
        a.r32 = c.v32[0];
        a.z32 = c.v32[1];
        a.pa32 = c.v32[2];
        a.pb32 = c.v32[3];
        a.q32 = c.v32[4];
        a.x32 = c.v32[5];
        if (s.storage == LFGPU_STORAGE_BSR) {
            ensure_bsr32(c);
            a.bval32 = reinterpret_cast<const float4*>(c.bval32.p);
        } else {
            ensure_csr32(c);
            a.val32 = c.K32;
        }
    }
    const bool csr = s.storage == LFGPU_STORAGE_CSR;
    const bool jac = s.precond == LFGPU_PRECOND_JACOBI;
    if (!s.mixed) {
        if (csr && jac) launch_coop(c, pcg64_kernel<LFGPU_STORAGE_CSR, LFGPU_PRECOND_JACOBI>, a, kernel_ms);
        else if (csr) launch_coop(c, pcg64_kernel<LFGPU_STORAGE_CSR, LFGPU_PRECOND_BLOCK2>, a, kernel_ms);
        else if (jac) launch_coop(c, pcg64_kernel<LFGPU_STORAGE_BSR, LFGPU_PRECOND_JACOBI>, a, kernel_ms);
        else launch_coop(c, pcg64_kernel<LFGPU_STORAGE_BSR, LFGPU_PRECOND_BLOCK2>, a, kernel_ms);
    } else {
        if (csr && jac) launch_coop(c, pcg_mixed_kernel<LFGPU_STORAGE_CSR, LFGPU_PRECOND_JACOBI>, a, kernel_ms);
        else if (csr) launch_coop(c, pcg_mixed_kernel<LFGPU_STORAGE_CSR, LFGPU_PRECOND_BLOCK2>, a, kernel_ms);
        else if (jac) launch_coop(c, pcg_mixed_kernel<LFGPU_STORAGE_BSR, LFGPU_PRECOND_JACOBI>, a, kernel_ms);
        else launch_coop(c, pcg_mixed_kernel<LFGPU_STORAGE_BSR, LFGPU_PRECOND_BLOCK2>, a, kernel_ms);
    }
    PcgResult res{};
    LF_CUDA(cudaMemcpyAsync(&res, c.pcg_result.p, sizeof(res), cudaMemcpyDeviceToHost, c.stream));
    check_status(c);
    return res;
}

}  // namespace lfgpu
