// Sparse-matrix kernels of the solve path: diagonal lookup, symmetric Dirichlet
// elimination, CSR and 2x2-BSR products in FP64 and FP32, CSR->BSR conversion,
// FP32 copies and the Jacobi / 2x2 nodal block-Jacobi setup.
//
// All of these are bandwidth-bound.  Products use a quarter warp per row (CSR) or
// per block row (BSR) so a warp reads eight rows' contiguous value/column streams
// at once; matrix data is loaded with the streaming (evict-first) hint so the
// dense vectors stay resident in the 129 MB L2.
#include "common.cuh"
#include "kernels.hpp"

#include <cmath>
#include <limits>

namespace lfgpu {
namespace {

constexpr int kThreads = 256;

__global__ void find_diagonal_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                     int* __restrict__ diag) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    int lo = rowptr[r], hi = rowptr[r + 1];
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (col[mid] < r) lo = mid + 1;
        else hi = mid;
    }
    diag[r] = (lo < rowptr[r + 1] && col[lo] == r) ? lo : -1;
}

// apply_dirichlet, src/solver.cpp:386-412.  One thread per row, entries in column
// order, products and differences rounded separately exactly as the host code
// rounds them, so K and f come out bit-identical to the reference.
__global__ void dirichlet_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                 const int* __restrict__ diag, const unsigned char* __restrict__ fixed,
                                 const double* __restrict__ prescribed, double* __restrict__ K, double* __restrict__ f) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int b = rowptr[r], e = rowptr[r + 1];
    if (fixed[r]) {
        for (int k = b; k < e; ++k) K[k] = 0.0;
        K[diag[r]] = 1.0;
        f[r] = prescribed[r];
        return;
    }
    double fr = f[r];
    bool touched = false;
    for (int k = b; k < e; ++k) {
        const int c = col[k];
        if (!fixed[c]) continue;
        const double v = K[k];
        if (v == 0.0) continue;
        fr = __dsub_rn(fr, __dmul_rn(v, prescribed[c]));
        K[k] = 0.0;
        touched = true;
    }
    if (touched) f[r] = fr;
}

__global__ void abs_max_kernel(int n, const double* __restrict__ v, unsigned long long* __restrict__ out) {
    double m = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = fmax(m, fabs(v[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, static_cast<unsigned long long>(__double_as_longlong(m)));
}

// Zero-pivot sweep, src/solver.cpp:920-940.
__global__ void zero_pivot_kernel(int n, const int* __restrict__ diag, const unsigned long long* __restrict__ scale_bits,
                                  double* __restrict__ K, double* __restrict__ f, DeviceStatus* status) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double scale = __longlong_as_double(static_cast<long long>(*scale_bits));
    if (scale <= 0.0) scale = 1.0;
    const double d = K[diag[r]];
    if (fabs(d) > 1.0e-30) return;
    if (fabs(f[r]) > 1.0e-12 * scale) {
        record_failure(status, LFGPU_ERR_MECHANISM, r);
        return;
    }
    K[diag[r]] = 1.0;
    f[r] = 0.0;
}

// ---------------------------------------------------------------- products
template <typename T>
__global__ void __launch_bounds__(kThreads) spmv_csr_kernel(int n, const int* __restrict__ rowptr,
                                                            const int* __restrict__ col, const T* __restrict__ val,
                                                            const T* __restrict__ x, T* __restrict__ y,
                                                            const T* __restrict__ sub, const float* __restrict__ dhi,
                                                            const float* __restrict__ dlo) {
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 2;
    const int q = threadIdx.x & 3;
    T s = T(0);
    if (row < n) {
        const int b = __ldg(rowptr + row), e = __ldg(rowptr + row + 1);
        for (int k = b + q; k < e; k += 8) {  // two independent units in flight per lane
            const bool two = k + 4 < e;
            const int c0 = ld_stream(col + k), c1 = two ? ld_stream(col + k + 4) : c0;
            const T v0 = ld_stream(val + k), v1 = two ? ld_stream(val + k + 4) : T(0);
            const T x0 = x[c0], x1 = x[c1];
            s += v0 * x0;
            s += v1 * x1;
        }
    }
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    if (row < n && q == 0) {
        if (dhi) {  // FP32 matrix: add the compensated diagonal (hi + lo) x
            const T xv = x[row];
            s = fma(static_cast<T>(dhi[row]), xv, s) + static_cast<T>(dlo[row]) * xv;
        }
        y[row] = sub ? s - sub[row] : s;
    }
}

__global__ void __launch_bounds__(kThreads) spmv_bsr64_kernel(int nb, const int* __restrict__ brow,
                                                              const int* __restrict__ bcol,
                                                              const double2* __restrict__ bval,
                                                              const double2* __restrict__ x, double2* __restrict__ y) {
    // A quarter warp per block row, whole 2x2 blocks per lane (top and bottom
    // rows as two 16-byte loads), three blocks in flight per lane, fused
    // multiply-adds only: GB300's FP64 pipe is the bound.
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 2;
    const int q = threadIdx.x & 3;
    double s0 = 0.0, s1 = 0.0;
    if (row < nb) {
        const int b = __ldg(brow + row), e = __ldg(brow + row + 1);
        for (int k = b + q; k < e; k += 12) {
            const double2 zero = make_double2(0.0, 0.0);
            const bool t1 = k + 4 < e, t2 = k + 8 < e;
            const int c0 = ld_stream(bcol + k), c1 = t1 ? ld_stream(bcol + k + 4) : c0,
                      c2 = t2 ? ld_stream(bcol + k + 8) : c0;
            const double2 u0 = ld_stream(bval + 2 * static_cast<size_t>(k));
            const double2 w0 = ld_stream(bval + 2 * static_cast<size_t>(k) + 1);
            const double2 u1 = t1 ? ld_stream(bval + 2 * static_cast<size_t>(k + 4)) : zero;
            const double2 w1 = t1 ? ld_stream(bval + 2 * static_cast<size_t>(k + 4) + 1) : zero;
            const double2 u2 = t2 ? ld_stream(bval + 2 * static_cast<size_t>(k + 8)) : zero;
            const double2 w2 = t2 ? ld_stream(bval + 2 * static_cast<size_t>(k + 8) + 1) : zero;
            const double2 x0 = x[c0], x1 = x[c1], x2 = x[c2];
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
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
    s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
    if (row < nb && q == 0) y[row] = make_double2(s0, s1);
}

__global__ void __launch_bounds__(kThreads) spmv_bsr32_kernel(int nb, const int* __restrict__ brow,
                                                              const int* __restrict__ bcol,
                                                              const float4* __restrict__ bval,
                                                              const float2* __restrict__ x, float2* __restrict__ y,
                                                              const float2* __restrict__ dhi,
                                                              const float2* __restrict__ dlo) {
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 2;
    const int q = threadIdx.x & 3;
    float s0 = 0.f, s1 = 0.f;
    if (row < nb) {
        const int b = __ldg(brow + row), e = __ldg(brow + row + 1);
        for (int k = b + q; k < e; k += 8) {  // two blocks in flight per lane
            const bool two = k + 4 < e;
            const float4 v0 = ld_stream(bval + k);
            const float4 v1 = two ? ld_stream(bval + k + 4) : make_float4(0.f, 0.f, 0.f, 0.f);
            const int c0 = ld_stream(bcol + k), c1 = two ? ld_stream(bcol + k + 4) : c0;
            const float2 x0 = x[c0], x1 = x[c1];
            s0 += v0.x * x0.x + v0.y * x0.y;
            s1 += v0.z * x0.x + v0.w * x0.y;
            s0 += v1.x * x1.x + v1.y * x1.y;
            s1 += v1.z * x1.x + v1.w * x1.y;
        }
    }
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
    s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
    if (row < nb && q == 0) {
        const float2 xv = x[row], h = dhi[row], l = dlo[row];
        s0 = fmaf(h.x, xv.x, s0) + l.x * xv.x;
        s1 = fmaf(h.y, xv.y, s1) + l.y * xv.y;
        y[row] = make_float2(s0, s1);
    }
}

// ---------------------------------------------------------------- CSR -> BSR
// Paired patterns (rows 2i and 2i+1 share one column list made of (2j, 2j+1)
// pairs): block row i starts at rowptr[2i] / 4 and block k of it is a pure gather.
__global__ void bsr_paired_structure_kernel(int nb, const int* __restrict__ rowptr, const int* __restrict__ col,
                                            int* __restrict__ brow, int* __restrict__ bcol) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > nb) return;
    if (i == nb) {
        brow[nb] = rowptr[2 * nb] / 4;
        return;
    }
    const int b = rowptr[2 * i], e = rowptr[2 * i + 1];
    const int out = b / 4;
    brow[i] = out;
    for (int k = b; k < e; k += 2) bcol[out + (k - b) / 2] = col[k] >> 1;
}

__global__ void bsr_paired_values_kernel(int nb, const int* __restrict__ rowptr, const int* __restrict__ brow,
                                         const double* __restrict__ K, double2* __restrict__ bval) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= nb) return;
    const int b0 = rowptr[2 * i], b1 = rowptr[2 * i + 1];
    const int len = (b1 - b0) / 2;
    const int out = brow[i];
    for (int m = 0; m < len; ++m) {
        const double2 top = *reinterpret_cast<const double2*>(K + b0 + 2 * m);
        const double2 bot = *reinterpret_cast<const double2*>(K + b1 + 2 * m);
        bval[2 * static_cast<size_t>(out + m)] = top;
        bval[2 * static_cast<size_t>(out + m) + 1] = bot;
    }
}

// General patterns: merge walk of the two rows of each block row
// (BsrMatrix::from_csr, src/sparse.cpp:128-177).  Pass 1 counts, pass 2 fills.
__device__ __forceinline__ int merge_walk(int i, const int* rowptr, const int* col, const double* K, int* bcol,
                                          double2* bval, bool fill, int out) {
    int p0 = rowptr[2 * i], p1 = rowptr[2 * i + 1];
    const int e0 = rowptr[2 * i + 1], e1 = rowptr[2 * i + 2];
    int count = 0;
    while (p0 < e0 || p1 < e1) {
        const int c0 = p0 < e0 ? col[p0] : 0x7fffffff;
        const int c1 = p1 < e1 ? col[p1] : 0x7fffffff;
        const int bc = min(c0, c1) >> 1;
        double blk[4] = {0.0, 0.0, 0.0, 0.0};
        for (; p0 < e0 && (col[p0] >> 1) == bc; ++p0) blk[col[p0] - 2 * bc] = K[p0];
        for (; p1 < e1 && (col[p1] >> 1) == bc; ++p1) blk[2 + col[p1] - 2 * bc] = K[p1];
        if (fill) {
            bcol[out + count] = bc;
            bval[2 * static_cast<size_t>(out + count)] = make_double2(blk[0], blk[1]);
            bval[2 * static_cast<size_t>(out + count) + 1] = make_double2(blk[2], blk[3]);
        }
        ++count;
    }
    return count;
}

__global__ void bsr_count_kernel(int nb, const int* rowptr, const int* col, int* counts) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nb) counts[i] = merge_walk(i, rowptr, col, nullptr, nullptr, nullptr, false, 0);
}

__global__ void bsr_fill_kernel(int nb, const int* rowptr, const int* col, const double* K, const int* brow,
                                int* bcol, double2* bval) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nb) merge_walk(i, rowptr, col, K, bcol, bval, true, brow[i]);
}

// FP32 inner matrix with a compensated diagonal.  Rounding the off-diagonal
// entries to FP32 breaks the exact row sums that make K annihilate rigid
// translations, and the perturbation lands on the lowest-energy modes, which then
// converge far more slowly in the FP32 inner PCG.  So the diagonal is kept apart,
// absorbs each row's rounding error over its same-component off-diagonals (the
// rows sums for both translations stay what they are in FP64), and is stored as an
// unevaluated FP32 pair hi + lo applied with one FMA.  Off-diagonals stay FP32;
// the stored FP32 diagonal slot is zero.
__global__ void compensated_diag_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                        const double* __restrict__ K, float* __restrict__ K32,
                                        float* __restrict__ dhi, float* __restrict__ dlo) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double err = 0.0, d = 0.0;
    for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) {
        const int c = col[k];
        const double v = K[k];
        if (c == r) {
            d = v;
            if (K32) K32[k] = 0.f;
            continue;
        }
        const float v32 = static_cast<float>(v);
        if (K32) K32[k] = v32;
        if ((c & 1) == (r & 1)) err += v - static_cast<double>(v32);
    }
    const double comp = d + err;
    const float hi = static_cast<float>(comp);
    dhi[r] = hi;
    dlo[r] = static_cast<float>(comp - static_cast<double>(hi));
}

// BSR32 values from BSR64 with the diagonal entries of the diagonal block zeroed.
__global__ void bsr32_values_kernel(int nb, const int* __restrict__ brow, const int* __restrict__ bcol,
                                    const double2* __restrict__ b64, float4* __restrict__ b32) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    for (int k = brow[i]; k < brow[i + 1]; ++k) {
        const double2 top = b64[2 * static_cast<size_t>(k)], bot = b64[2 * static_cast<size_t>(k) + 1];
        float4 v = make_float4(static_cast<float>(top.x), static_cast<float>(top.y), static_cast<float>(bot.x),
                               static_cast<float>(bot.y));
        if (bcol[k] == i) {
            v.x = 0.f;
            v.w = 0.f;
        }
        b32[k] = v;
    }
}

__global__ void to_float_kernel(i64 count, const double* __restrict__ in, float* __restrict__ out) {
    for (i64 i = blockIdx.x * static_cast<i64>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<i64>(gridDim.x) * blockDim.x)
        out[i] = static_cast<float>(in[i]);
}

// ---------------------------------------------------------------- preconditioners
// inverse_diagonal_of (src/solver.cpp:656-669) and the 2x2 nodal case of
// SubdomainBlockJacobi (src/precond.cpp:186-231): Cholesky of
// [[K(2i,2i), .], [K(2i+1,2i), K(2i+1,2i+1)]] with reciprocal pivots stored as
// (1/L00, L10, 1/L11); a block that is not positive definite becomes the identity.
// A non-finite diagonal is only an error for the Jacobi preconditioner, so the
// kernel records the first such DOF in ``nonfinite`` and the solve decides.
__global__ void precond_setup_kernel(int nb, const int* __restrict__ rowptr, const int* __restrict__ col,
                                     const int* __restrict__ diag, const double* __restrict__ K,
                                     double* __restrict__ inv_diag, double* __restrict__ blk,
                                     int* __restrict__ degenerate, int* __restrict__ nonfinite) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const double d0 = K[diag[2 * i]], d1 = K[diag[2 * i + 1]];
    if (!isfinite(d0) || !isfinite(d1)) atomicMin(nonfinite, isfinite(d0) ? 2 * i + 1 : 2 * i);
    inv_diag[2 * i] = fabs(d0) > 1.0e-30 ? 1.0 / d0 : 1.0;
    inv_diag[2 * i + 1] = fabs(d1) > 1.0e-30 ? 1.0 / d1 : 1.0;
    // K(2i+1, 2i): search row 2i+1 for column 2i.
    double d10 = 0.0;
    for (int k = rowptr[2 * i + 1]; k < rowptr[2 * i + 2]; ++k) {
        if (col[k] == 2 * i) {
            d10 = K[k];
            break;
        }
        if (col[k] > 2 * i) break;
    }
    double f0 = 1.0, f1 = 0.0, f2 = 1.0;
    bool ok = d0 > 0.0 && isfinite(d0);
    if (ok) {
        const double l00 = sqrt(d0);
        const double l10 = d10 / l00;
        const double s = d1 - l10 * l10;
        ok = s > 0.0 && isfinite(s);
        if (ok) {
            const double l11 = sqrt(s);
            f0 = 1.0 / l00;
            f1 = l10;
            f2 = 1.0 / l11;
        }
    }
    if (!ok) {
        f0 = 1.0;
        f1 = 0.0;
        f2 = 1.0;
        atomicAdd(degenerate, 1);
    }
    blk[3 * i] = f0;
    blk[3 * i + 1] = f1;
    blk[3 * i + 2] = f2;
}

__global__ void norm_partials_kernel(i64 n, const double* __restrict__ v, double* __restrict__ partial) {
    double s = 0.0;
    for (i64 i = blockIdx.x * static_cast<i64>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<i64>(gridDim.x) * blockDim.x)
        s += v[i] * v[i];
    __shared__ double red[32];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        s = warp_sum(s);
        if (threadIdx.x == 0) partial[blockIdx.x] = s;
    }
}

__global__ void sum_partials_kernel(int m, const double* __restrict__ partial, double* __restrict__ out) {
    double s = 0.0;
    for (int i = threadIdx.x; i < m; i += 32) s += partial[i];
    s = warp_sum(s);
    if (threadIdx.x == 0) out[0] = s;
}

__global__ void axpby_kernel(i64 n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
    for (i64 i = blockIdx.x * static_cast<i64>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<i64>(gridDim.x) * blockDim.x)
        y[i] = a * x[i] + b * y[i];
}

__global__ void capture_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                               unsigned long long* __restrict__ inside) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long cnt = 0;
    if (r < n)
        for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) cnt += (col[k] >> 1) == (r >> 1);
    cnt = warp_sum(cnt);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(inside, cnt);
}

}  // namespace

void launch_find_diagonal(Context& c) {
    find_diagonal_kernel<<<grid_for(c.n, kThreads), kThreads, 0, c.stream>>>(static_cast<int>(c.n), c.rowptr, c.col,
                                                                            c.diag);
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
}

void launch_dirichlet(Context& c) {
    const int n = static_cast<int>(c.n);
    if (c.n_constraints > 0) {
        dirichlet_kernel<<<grid_for(n, kThreads), kThreads, 0, c.stream>>>(n, c.rowptr, c.col, c.diag, c.fixed,
                                                                          c.prescribed, c.K, c.f);
        c.launches += 1;
        LF_CUDA(cudaGetLastError());
    }
    c.scratch64.ensure(64);
    unsigned long long* bits = reinterpret_cast<unsigned long long*>(c.scratch64.p);
    LF_CUDA(cudaMemsetAsync(bits, 0, sizeof(unsigned long long), c.stream));
    abs_max_kernel<<<grid_for(n, kThreads, 4 * c.num_sms), kThreads, 0, c.stream>>>(n, c.f, bits);
    c.launches += 1;
    zero_pivot_kernel<<<grid_for(n, kThreads), kThreads, 0, c.stream>>>(n, c.diag, bits, c.K, c.f, c.status);
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
}

void launch_spmv_csr64(Context& c, const double* val, const double* x, double* y, const double* sub) {
    const int n = static_cast<int>(c.n);
    spmv_csr_kernel<double><<<grid_for(4LL * n, kThreads), kThreads, 0, c.stream>>>(n, c.rowptr, c.col, val, x, y,
                                                                                   sub, nullptr, nullptr);
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
}

void launch_spmv_csr32(Context& c, const float* val, const float* x, float* y) {
    const int n = static_cast<int>(c.n);
    spmv_csr_kernel<float><<<grid_for(4LL * n, kThreads), kThreads, 0, c.stream>>>(n, c.rowptr, c.col, val, x, y,
                                                                                  nullptr, c.diag_hi, c.diag_lo);
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
}

void launch_spmv_bsr64(Context& c, const double* x, double* y) {
    const int nb = static_cast<int>(c.n / 2);
    spmv_bsr64_kernel<<<grid_for(4LL * nb, kThreads), kThreads, 0, c.stream>>>(
        nb, c.brow, c.bcol, reinterpret_cast<const double2*>(c.bval64.p), reinterpret_cast<const double2*>(x),
        reinterpret_cast<double2*>(y));
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
}

void launch_spmv_bsr32(Context& c, const float* x, float* y) {
    const int nb = static_cast<int>(c.n / 2);
    spmv_bsr32_kernel<<<grid_for(4LL * nb, kThreads), kThreads, 0, c.stream>>>(
        nb, c.brow, c.bcol, reinterpret_cast<const float4*>(c.bval32.p), reinterpret_cast<const float2*>(x),
        reinterpret_cast<float2*>(y), reinterpret_cast<const float2*>(c.diag_hi.p),
        reinterpret_cast<const float2*>(c.diag_lo.p));
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
}

void ensure_bsr(Context& c) {
    if (c.bsr_version == c.k_version) return;
    LF_REQUIRE(c.n % 2 == 0, LFGPU_ERR_ARGUMENT, "BSR conversion needs an even number of rows (u,v DOF pairs)");
    const int nb = static_cast<int>(c.n / 2);
    LF_CUDA(cudaEventRecord(c.ev_a, c.stream));
    c.brow.ensure(nb + 1);
    if (c.paired) {
        c.nblocks = c.nnz / 4;
        c.h_brow.resize(static_cast<size_t>(nb) + 1);
        for (int i = 0; i <= nb; ++i) c.h_brow[i] = c.h_rowptr_cache[2 * static_cast<size_t>(i)] / 4;
        c.bcol.ensure(c.nblocks);
        c.bval64.ensure(4 * c.nblocks);
        bsr_paired_structure_kernel<<<grid_for(nb + 1, kThreads), kThreads, 0, c.stream>>>(nb, c.rowptr, c.col,
                                                                                          c.brow, c.bcol);
        c.launches += 1;
        bsr_paired_values_kernel<<<grid_for(nb, kThreads), kThreads, 0, c.stream>>>(
            nb, c.rowptr, c.brow, c.K, reinterpret_cast<double2*>(c.bval64.p));
        c.launches += 1;
    } else {
        Buf<int> counts;
        counts.ensure(nb);
        bsr_count_kernel<<<grid_for(nb, kThreads), kThreads, 0, c.stream>>>(nb, c.rowptr, c.col, counts);
        c.launches += 1;
        std::vector<int> h(nb), ptr(nb + 1, 0);
        LF_CUDA(cudaMemcpyAsync(h.data(), counts.p, sizeof(int) * nb, cudaMemcpyDeviceToHost, c.stream));
        LF_CUDA(cudaStreamSynchronize(c.stream));
        for (int i = 0; i < nb; ++i) ptr[i + 1] = ptr[i] + h[i];
        c.nblocks = ptr[nb];
        c.h_brow = ptr;
        LF_CUDA(cudaMemcpyAsync(c.brow.p, ptr.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, c.stream));
        c.bcol.ensure(c.nblocks);
        c.bval64.ensure(4 * c.nblocks);
        bsr_fill_kernel<<<grid_for(nb, kThreads), kThreads, 0, c.stream>>>(
            nb, c.rowptr, c.col, c.K, c.brow, c.bcol, reinterpret_cast<double2*>(c.bval64.p));
        c.launches += 1;
        LF_CUDA(cudaStreamSynchronize(c.stream));
        counts.release();
    }
    LF_CUDA(cudaGetLastError());
    LF_CUDA(cudaEventRecord(c.ev_b, c.stream));
    c.last_convert_ms = elapsed_ms(c);
    c.bsr_version = c.k_version;
}

void launch_to_float(Context& c, const double* in, float* out, i64 count) {
    to_float_kernel<<<grid_for(count, kThreads, 16 * c.num_sms), kThreads, 0, c.stream>>>(count, in, out);
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
}

// Block columns as 16-bit offsets from the block row (the FP32 product's column
// stream at half the bytes); *wide is set when an offset does not fit.
__global__ void bsr_offsets_kernel(int nb, const int* __restrict__ brow, const int* __restrict__ bcol,
                                   short* __restrict__ off, int* __restrict__ wide) {
    const int node = blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nb) return;
    for (int k = brow[node]; k < brow[node + 1]; ++k) {
        const int d = bcol[k] - node;
        if (d < -32768 || d > 32767) {
            atomicOr(wide, 1);
            return;
        }
        off[k] = static_cast<short>(d);
    }
}

void ensure_bsr32(Context& c) {
    ensure_bsr(c);
    if (c.b32_version == c.k_version) return;
    const int nb = static_cast<int>(c.n / 2);
    c.bval32.ensure(4 * c.nblocks);
    c.diag_hi.ensure(c.n);
    c.diag_lo.ensure(c.n);
    bsr32_values_kernel<<<grid_for(nb, kThreads), kThreads, 0, c.stream>>>(
        nb, c.brow, c.bcol, reinterpret_cast<const double2*>(c.bval64.p), reinterpret_cast<float4*>(c.bval32.p));
    c.launches += 1;
    compensated_diag_kernel<<<grid_for(c.n, kThreads), kThreads, 0, c.stream>>>(static_cast<int>(c.n), c.rowptr,
                                                                               c.col, c.K, nullptr, c.diag_hi,
                                                                               c.diag_lo);
    c.launches += 1;
    c.bcol16.ensure(static_cast<size_t>(c.nblocks));
    c.scratch64.ensure(64);
    int* wide = reinterpret_cast<int*>(c.scratch64.p + 40);
    LF_CUDA(cudaMemsetAsync(wide, 0, sizeof(int), c.stream));
    bsr_offsets_kernel<<<grid_for(nb, kThreads), kThreads, 0, c.stream>>>(nb, c.brow, c.bcol, c.bcol16, wide);
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
    int h = 0;
    LF_CUDA(cudaMemcpyAsync(&h, wide, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    LF_CUDA(cudaStreamSynchronize(c.stream));
    c.bcol16_ok = h == 0;
    c.b32_version = c.k_version;
}

// Columns as 16-bit offsets from the row (the FP32 CSR product's column stream
// at half the bytes); *wide is set when an offset does not fit.
__global__ void csr_offsets_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                   short* __restrict__ off, int* __restrict__ wide) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    for (int k = rowptr[row]; k < rowptr[row + 1]; ++k) {
        const int d = col[k] - row;
        if (d < -32768 || d > 32767) {
            atomicOr(wide, 1);
            return;
        }
        off[k] = static_cast<short>(d);
    }
}

void ensure_csr32(Context& c) {
    if (c.k32_version == c.k_version) return;
    c.K32.ensure(c.nnz);
    c.diag_hi.ensure(c.n);
    c.diag_lo.ensure(c.n);
    compensated_diag_kernel<<<grid_for(c.n, kThreads), kThreads, 0, c.stream>>>(static_cast<int>(c.n), c.rowptr,
                                                                               c.col, c.K, c.K32, c.diag_hi,
                                                                               c.diag_lo);
    c.launches += 1;
    c.col16.ensure(static_cast<size_t>(c.nnz));
    c.scratch64.ensure(64);
    int* wide = reinterpret_cast<int*>(c.scratch64.p + 44);
    LF_CUDA(cudaMemsetAsync(wide, 0, sizeof(int), c.stream));
    csr_offsets_kernel<<<grid_for(c.n, kThreads), kThreads, 0, c.stream>>>(static_cast<int>(c.n), c.rowptr, c.col,
                                                                           c.col16, wide);
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
    int h = 0;
    LF_CUDA(cudaMemcpyAsync(&h, wide, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    LF_CUDA(cudaStreamSynchronize(c.stream));
    c.col16_ok = h == 0;
    c.k32_version = c.k_version;
}

static void setup_preconditioners(Context& c) {
    const int nb = static_cast<int>(c.n / 2);
    c.inv_diag64.ensure(c.n);
    c.blk64.ensure(3 * static_cast<size_t>(nb));
    c.inv_diag32.ensure(c.n);
    c.blk32.ensure(3 * static_cast<size_t>(nb) + 12);  // the staged update copies whole groups of four nodes
    c.scratch64.ensure(64);
    // flags[0]: degenerate 2x2 blocks; flags[1]: first non-finite diagonal DOF.
    int* flags = reinterpret_cast<int*>(c.scratch64.p + 8);
    static const int init[2] = {0, std::numeric_limits<int>::max()};
    LF_CUDA(cudaMemcpyAsync(flags, init, sizeof(init), cudaMemcpyHostToDevice, c.stream));
    precond_setup_kernel<<<grid_for(nb, kThreads), kThreads, 0, c.stream>>>(nb, c.rowptr, c.col, c.diag, c.K,
                                                                           c.inv_diag64, c.blk64, flags,
                                                                           flags + 1);
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
    launch_to_float(c, c.inv_diag64, c.inv_diag32, c.n);
    launch_to_float(c, c.blk64, c.blk32, 3LL * nb);
    int h[2] = {0, 0};
    LF_CUDA(cudaMemcpyAsync(h, flags, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
    check_status(c);
    c.degenerate_blocks = h[0];
    c.nonfinite_diag = h[1] == std::numeric_limits<int>::max() ? -1 : h[1];
    c.pre_version = c.k_version;
}

void ensure_preconditioners(Context& c, int precond) {
    if (c.pre_version != c.k_version) setup_preconditioners(c);
    // inverse_diagonal_of, src/solver.cpp:656-669: only the Jacobi setup checks.
    if (precond == LFGPU_PRECOND_JACOBI && c.nonfinite_diag >= 0)
        throw Error{LFGPU_ERR_NONFINITE_DIAG, "Jacobi preconditioner encountered a non-finite diagonal (dof " +
                                                  std::to_string(c.nonfinite_diag) + ")"};
}

double device_norm2(Context& c, const double* v, i64 count) {
    const int blocks = 2 * c.num_sms;
    c.scratch64.ensure(64 + blocks + 1);
    double* partial = c.scratch64.p + 64;
    norm_partials_kernel<<<blocks, kThreads, 0, c.stream>>>(count, v, partial);
    c.launches += 1;
    sum_partials_kernel<<<1, 32, 0, c.stream>>>(blocks, partial, partial + blocks);
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
    double h = 0.0;
    LF_CUDA(cudaMemcpyAsync(&h, partial + blocks, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    LF_CUDA(cudaStreamSynchronize(c.stream));
    return std::sqrt(h);
}

void launch_axpby(Context& c, i64 count, double a, const double* x, double b, double* y) {
    axpby_kernel<<<grid_for(count, kThreads, 16 * c.num_sms), kThreads, 0, c.stream>>>(count, a, x, b, y);
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
}

double capture_ratio_2x2(Context& c) {
    c.scratch64.ensure(64);
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(c.scratch64.p + 16);
    LF_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), c.stream));
    capture_kernel<<<grid_for(c.n, kThreads), kThreads, 0, c.stream>>>(static_cast<int>(c.n), c.rowptr, c.col, cnt);
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
    unsigned long long h = 0;
    LF_CUDA(cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
    LF_CUDA(cudaStreamSynchronize(c.stream));
    return c.nnz ? static_cast<double>(h) / static_cast<double>(c.nnz) : 0.0;
}

}  // namespace lfgpu
