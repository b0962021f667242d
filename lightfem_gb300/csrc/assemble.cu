// Q4 element stiffness fused with the numeric assembly through the element->CSR
// value map, and the consistent element loads.
//
// Replaces q4_stiffness (src/element.cpp:130-161) + coloring_assembly /
// atomic_assembly (src/solver.cpp:144-179) and the load part of assemble
// (src/solver.cpp:303-332, q4_body_force / q4_edge_* src/element.cpp:163-210).
//
// One thread per element.  The four Gauss points' shape-function derivatives are
// kept in registers and K_e is produced 2x2 node block by 2x2 node block: for
// isotropic D (D02 = D12 = 0, D11 = D00) block (a, b) only needs the four sums
// s_xx = sum w Nx_a Nx_b, s_yy, s_xy, s_yx, and K_e symmetry gives block (b, a)
// for free, so a Q4 costs ~10 blocks x 24 FMA instead of 64 x 12.  The element's
// 64 map entries are staged through shared memory with coalesced loads (the map
// is the dominant HBM stream, 256 B per element).  When every map pair
// (2b, 2b+1) lands on an aligned value pair (always true for Q4 patterns) a block
// row is scattered as one double2 read-modify-write.
//
// Colouring strategy: one launch per colour, no two elements of a launch share a
// node, so plain read-modify-writes are race-free and the sum order is fixed.
// Atomic strategy: one launch, atomicAdd on every entry.
#include "common.cuh"
#include "kernels.hpp"

namespace lfgpu {
namespace {

constexpr int kAsmThreads = 128;
constexpr double kG = 0.57735026918962576451;

struct AsmArgs {
    const double2* xy;
    const int4* elem_nodes;
    const int* elem_mat;
    const double* young;
    const double* nu;
    const double* thick;
    const int* map;
    const int* elems;  // element list of this launch, or nullptr for 0..count-1
    int count;
    int plane_strain;
    int paired;
    double* K;
    double* f;
    const double* body_bx;  // per element or nullptr
    const double* body_by;
    const int* edge_ptr;    // per element CSR, or nullptr
    const int* edge_side;
    const int* edge_kind;
    const double* edge_a;
    const double* edge_b;
    DeviceStatus* status;
};

template <bool ATOMIC>
__device__ __forceinline__ void add_value(double* K, int idx, double v) {
    if (ATOMIC) {
        atomicAdd(K + idx, v);
    } else {
        K[idx] += v;
    }
}

template <bool ATOMIC>
__device__ __forceinline__ void add_pair(double* K, int idx, double a, double b, int paired, int idx_b) {
    if (ATOMIC) {
        atomicAdd(K + idx, a);
        atomicAdd(K + idx_b, b);
    } else if (paired) {
        double2* p = reinterpret_cast<double2*>(K + idx);
        double2 v = *p;
        v.x += a;
        v.y += b;
        *p = v;
    } else {
        K[idx] += a;
        K[idx_b] += b;
    }
}

template <bool ATOMIC>
__global__ void __launch_bounds__(kAsmThreads) q4_assemble_kernel(AsmArgs a) {
    __shared__ int s_map[kAsmThreads * 64];
    const int base = blockIdx.x * kAsmThreads;
    const int local_count = min(kAsmThreads, a.count - base);

    // Stage this CTA's map rows: one warp copies one element's 64 entries
    // (256 B) per step as 32 x int2.
    {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int k = warp; k < local_count; k += kAsmThreads / 32) {
            const int e = a.elems ? __ldg(a.elems + base + k) : base + k;
            const int2 v = ld_stream(reinterpret_cast<const int2*>(a.map + static_cast<size_t>(e) * 64) + lane);
            reinterpret_cast<int2*>(s_map + k * 64)[lane] = v;
        }
    }
    __syncthreads();
    if (static_cast<int>(threadIdx.x) >= local_count) return;

    const int e = a.elems ? __ldg(a.elems + base + threadIdx.x) : base + threadIdx.x;
    const int4 nd = __ldg(a.elem_nodes + e);
    const int m = __ldg(a.elem_mat + e);
    const double E = __ldg(a.young + m), nu = __ldg(a.nu + m), t = __ldg(a.thick + m);
    const double2 c0 = __ldg(a.xy + nd.x), c1 = __ldg(a.xy + nd.y), c2 = __ldg(a.xy + nd.z), c3 = __ldg(a.xy + nd.w);
    const double X[4] = {c0.x, c1.x, c2.x, c3.x};
    const double Y[4] = {c0.y, c1.y, c2.y, c3.y};

    // constitutive_matrix, src/element.cpp:16-32 (D11 = D00, D02 = D12 = 0).
    double d00, d01, d22;
    if (!a.plane_strain) {
        const double fct = E / (1.0 - nu * nu);
        d00 = fct;
        d01 = fct * nu;
        d22 = fct * (1.0 - nu) * 0.5;
    } else {
        const double fct = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
        d00 = fct * (1.0 - nu);
        d01 = fct * nu;
        d22 = fct * (1.0 - 2.0 * nu) * 0.5;
    }

    // q4_kinematics at the 2x2 Gauss points, src/element.cpp:34-73.
    double nx[4][4], ny[4][4], w[4];
    bool ok = true;
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        const double xi = (g == 0 || g == 3) ? -kG : kG;
        const double eta = (g < 2) ? -kG : kG;
        const double dxi[4] = {-0.25 * (1.0 - eta), 0.25 * (1.0 - eta), 0.25 * (1.0 + eta), -0.25 * (1.0 + eta)};
        const double deta[4] = {-0.25 * (1.0 - xi), -0.25 * (1.0 + xi), 0.25 * (1.0 + xi), 0.25 * (1.0 - xi)};
        double j00 = 0.0, j01 = 0.0, j10 = 0.0, j11 = 0.0;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            j00 += dxi[i] * X[i];
            j01 += deta[i] * X[i];
            j10 += dxi[i] * Y[i];
            j11 += deta[i] * Y[i];
        }
        const double det = j00 * j11 - j01 * j10;
        ok = ok && (det > 1.0e-14) && isfinite(det);
        const double inv = 1.0 / det;
        const double i00 = j11 * inv, i01 = -j01 * inv, i10 = -j10 * inv, i11 = j00 * inv;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            nx[g][i] = i00 * dxi[i] + i10 * deta[i];
            ny[g][i] = i01 * dxi[i] + i11 * deta[i];
        }
        w[g] = det * t;
    }
    if (!ok) {
        record_failure(a.status, LFGPU_ERR_JACOBIAN, e);
        return;
    }

    const int* mp = s_map + threadIdx.x * 64;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int j = i; j < 4; ++j) {
            double sxx = 0.0, syy = 0.0, sxy = 0.0, syx = 0.0;
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                const double wx = w[g] * nx[g][i], wy = w[g] * ny[g][i];
                sxx += wx * nx[g][j];
                sxy += wx * ny[g][j];
                syy += wy * ny[g][j];
                syx += wy * nx[g][j];
            }
            const double kxx = d00 * sxx + d22 * syy;
            const double kxy = d01 * sxy + d22 * syx;
            const double kyx = d01 * syx + d22 * sxy;
            const double kyy = d00 * syy + d22 * sxx;
            // block (i, j): rows 2i, 2i+1, columns 2j, 2j+1
            add_pair<ATOMIC>(a.K, mp[(2 * i) * 8 + 2 * j], kxx, kxy, a.paired, mp[(2 * i) * 8 + 2 * j + 1]);
            add_pair<ATOMIC>(a.K, mp[(2 * i + 1) * 8 + 2 * j], kyx, kyy, a.paired, mp[(2 * i + 1) * 8 + 2 * j + 1]);
            if (j != i) {
                // block (j, i) = block (i, j)^T
                add_pair<ATOMIC>(a.K, mp[(2 * j) * 8 + 2 * i], kxx, kyx, a.paired, mp[(2 * j) * 8 + 2 * i + 1]);
                add_pair<ATOMIC>(a.K, mp[(2 * j + 1) * 8 + 2 * i], kxy, kyy, a.paired, mp[(2 * j + 1) * 8 + 2 * i + 1]);
            }
        }
    }

    // Consistent element loads.
    const bool body = a.body_bx != nullptr;
    const int r0 = a.edge_ptr ? __ldg(a.edge_ptr + e) : 0;
    const int r1 = a.edge_ptr ? __ldg(a.edge_ptr + e + 1) : 0;
    if (!body && r0 == r1) return;
    double fe[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (body) {
        const double bx = __ldg(a.body_bx + e), by = __ldg(a.body_by + e);
        if (bx != 0.0 || by != 0.0) {
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                const double xi = (g == 0 || g == 3) ? -kG : kG;
                const double eta = (g < 2) ? -kG : kG;
                const double N[4] = {0.25 * (1.0 - xi) * (1.0 - eta), 0.25 * (1.0 + xi) * (1.0 - eta),
                                     0.25 * (1.0 + xi) * (1.0 + eta), 0.25 * (1.0 - xi) * (1.0 + eta)};
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    fe[2 * i] += N[i] * bx * w[g];
                    fe[2 * i + 1] += N[i] * by * w[g];
                }
            }
        }
    }
    for (int r = r0; r < r1; ++r) {
        const int side = __ldg(a.edge_side + r);
        const int first = side - 1, second = side % 4;
        const double dx = X[second] - X[first], dy = Y[second] - Y[first];
        const double len = hypot(dx, dy);
        if (!(len > 1.0e-14)) {
            record_failure(a.status, LFGPU_ERR_EDGE, e);
            return;
        }
        double tx = __ldg(a.edge_a + r), ty = __ldg(a.edge_b + r);
        if (__ldg(a.edge_kind + r) == LFGPU_EDGE_PRESSURE) {
            const double p = tx;
            tx = -p * dy / len;
            ty = p * dx / len;
        }
        const double wt = 0.5 * len * t;
        // First and second edge node (edge_nodes, src/element.cpp:102-110).
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (i == first || i == second) {
                fe[2 * i] += wt * tx;
                fe[2 * i + 1] += wt * ty;
            }
        }
    }
    const int nodes[4] = {nd.x, nd.y, nd.z, nd.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) add_pair<ATOMIC>(a.f, 2 * nodes[i], fe[2 * i], fe[2 * i + 1], 1, 2 * nodes[i] + 1);
}

}  // namespace

void launch_assembly(Context& c, int strategy) {
    AsmArgs a{};
    a.xy = c.xy;
    a.elem_nodes = c.elem_nodes;
    a.elem_mat = c.elem_mat;
    a.young = c.mat_young;
    a.nu = c.mat_nu;
    a.thick = c.mat_t;
    a.map = c.map;
    a.plane_strain = c.plane_mode == LFGPU_PLANE_STRAIN;
    a.paired = c.paired ? 1 : 0;
    a.K = c.K;
    a.f = c.f;
    a.body_bx = c.have_body ? c.body_bx.p : nullptr;
    a.body_by = c.have_body ? c.body_by.p : nullptr;
    a.edge_ptr = c.have_edges ? c.edge_ptr.p : nullptr;
    a.edge_side = c.edge_side;
    a.edge_kind = c.edge_kind;
    a.edge_a = c.edge_a;
    a.edge_b = c.edge_b;
    a.status = c.status;
    if (strategy == LFGPU_ASSEMBLY_ATOMIC) {
        a.elems = nullptr;
        a.count = static_cast<int>(c.n_elem);
        if (a.count > 0)
            q4_assemble_kernel<true><<<grid_for(a.count, kAsmThreads), kAsmThreads, 0, c.stream>>>(a);
            c.launches += 1;
        LF_CUDA(cudaGetLastError());
        return;
    }
    for (int k = 0; k < c.n_colors; ++k) {
        const int lo = c.color_offsets[k], hi = c.color_offsets[k + 1];
        if (hi <= lo) continue;
        a.elems = c.color_elems.p + lo;
        a.count = hi - lo;
        q4_assemble_kernel<false><<<grid_for(a.count, kAsmThreads), kAsmThreads, 0, c.stream>>>(a);
        c.launches += 1;
        LF_CUDA(cudaGetLastError());
    }
}

}  // namespace lfgpu
