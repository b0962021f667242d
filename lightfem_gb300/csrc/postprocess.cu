// Post-processing on the device: element strain/stress/von Mises at the centre and
// the four Gauss points (q4_center_field and q4_gauss_point_fields,
// src/element.cpp:212-248, as postprocess calls them, src/solver.cpp:756-771), and
// nodal stress smoothing by Gauss-point extrapolation (smooth_nodal_stresses,
// src/solver.cpp:807-871).
//
// Every operation follows the reference's order without contraction, so for the
// same displacements the fields equal the reference's bit for bit.  The nodal sums
// take each node's elements in ascending element order, as the reference's element
// loop does.
//
// Layouts: fields[35 e + 7 k + j], k = 0 centre, 1..4 Gauss points (-g,-g),
// (g,-g), (g,g), (-g,g); j = strain xx, yy, xy, stress xx, yy, xy, von Mises.
// nodal[4 i + j]: stress xx, yy, xy, von Mises; a node in no element gets zeros.
#include "common.cuh"
#include "kernels.hpp"

namespace lfgpu {
namespace {

constexpr int kThreads = 256;
constexpr double kGauss = 0.57735026918962576451;

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }

// constitutive_matrix, src/element.cpp:16-32.
__device__ void constitutive(double e, double nu, int plane_strain, double d[9]) {
    for (int k = 0; k < 9; ++k) d[k] = 0.0;
    if (!plane_strain) {
        const double f = div(e, sub(1.0, mul(nu, nu)));
        d[0] = f;
        d[1] = mul(f, nu);
        d[3] = mul(f, nu);
        d[4] = f;
        d[8] = mul(mul(f, sub(1.0, nu)), 0.5);
    } else {
        const double f = div(e, mul(add(1.0, nu), sub(1.0, mul(2.0, nu))));
        d[0] = mul(f, sub(1.0, nu));
        d[1] = mul(f, nu);
        d[3] = mul(f, nu);
        d[4] = mul(f, sub(1.0, nu));
        d[8] = mul(mul(f, sub(1.0, mul(2.0, nu))), 0.5);
    }
}

// q4_kinematics, src/element.cpp:34-73: the 3x8 B matrix; false for a
// non-positive or non-finite Jacobian.
__device__ bool kinematics(const double x[4], const double y[4], double xi, double eta, double b[24]) {
    const double dxi[4] = {mul(-0.25, sub(1.0, eta)), mul(+0.25, sub(1.0, eta)), mul(+0.25, add(1.0, eta)),
                           mul(-0.25, add(1.0, eta))};
    const double deta[4] = {mul(-0.25, sub(1.0, xi)), mul(-0.25, add(1.0, xi)), mul(+0.25, add(1.0, xi)),
                            mul(+0.25, sub(1.0, xi))};
    double j00 = 0.0, j01 = 0.0, j10 = 0.0, j11 = 0.0;
    for (int i = 0; i < 4; ++i) {
        j00 = add(j00, mul(dxi[i], x[i]));
        j01 = add(j01, mul(deta[i], x[i]));
        j10 = add(j10, mul(dxi[i], y[i]));
        j11 = add(j11, mul(deta[i], y[i]));
    }
    const double det = sub(mul(j00, j11), mul(j01, j10));
    if (!(det > 1.0e-14) || !isfinite(det)) return false;
    const double i00 = div(j11, det), i01 = div(-j01, det), i10 = div(-j10, det), i11 = div(j00, det);
    for (int i = 0; i < 4; ++i) {
        const double nx = add(mul(i00, dxi[i]), mul(i10, deta[i]));
        const double ny = add(mul(i01, dxi[i]), mul(i11, deta[i]));
        b[2 * i] = nx;
        b[2 * i + 1] = 0.0;
        b[8 + 2 * i] = 0.0;
        b[8 + 2 * i + 1] = ny;
        b[16 + 2 * i] = ny;
        b[16 + 2 * i + 1] = nx;
    }
    return true;
}

__device__ __forceinline__ double von_mises(double sx, double sy, double txy) {
    const double v = add(add(sub(mul(sx, sx), mul(sx, sy)), mul(sy, sy)), mul(mul(3.0, txy), txy));
    return __dsqrt_rn(fmax(0.0, v));
}

// strain = B u (multiply_3x8), stress = D strain (multiply_3x3), von Mises.
__device__ void field(const double b[24], const double d[9], const double u[8], double* out) {
    double strain[3], stress[3];
    for (int r = 0; r < 3; ++r) {
        double s = 0.0;
        for (int c = 0; c < 8; ++c) s = add(s, mul(b[8 * r + c], u[c]));
        strain[r] = s;
    }
    for (int r = 0; r < 3; ++r) {
        double s = 0.0;
        for (int c = 0; c < 3; ++c) s = add(s, mul(d[3 * r + c], strain[c]));
        stress[r] = s;
    }
    for (int r = 0; r < 3; ++r) {
        out[r] = strain[r];
        out[3 + r] = stress[r];
    }
    out[6] = von_mises(stress[0], stress[1], stress[2]);
}

__global__ void __launch_bounds__(kThreads) element_fields_kernel(int ne, const double2* __restrict__ xy,
                                                                  const int4* __restrict__ en,
                                                                  const int* __restrict__ mat,
                                                                  const double* __restrict__ young,
                                                                  const double* __restrict__ nu, int plane_strain,
                                                                  const double* __restrict__ u, double* fields,
                                                                  DeviceStatus* status) {
    const double pts[5][2] = {{0.0, 0.0}, {-kGauss, -kGauss}, {kGauss, -kGauss}, {kGauss, kGauss}, {-kGauss, kGauss}};
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        const int4 q = en[e];
        const int nd[4] = {q.x, q.y, q.z, q.w};
        double x[4], y[4], ue[8];
        for (int a = 0; a < 4; ++a) {
            const double2 p = xy[nd[a]];
            x[a] = p.x;
            y[a] = p.y;
            const double2 v = reinterpret_cast<const double2*>(u)[nd[a]];
            ue[2 * a] = v.x;
            ue[2 * a + 1] = v.y;
        }
        double d[9], b[24];
        const int m = mat[e];
        constitutive(young[m], nu[m], plane_strain, d);
        double* out = fields + 35LL * e;
        for (int k = 0; k < 5; ++k) {
            if (!kinematics(x, y, pts[k][0], pts[k][1], b)) {
                record_failure(status, LFGPU_ERR_JACOBIAN, e);
                break;
            }
            field(b, d, ue, out + 7 * k);
        }
    }
}

// smooth_nodal_stresses, src/solver.cpp:807-871 (Q4 part).
__global__ void __launch_bounds__(kThreads) nodal_smoothing_kernel(int nn, const int* __restrict__ ptr,
                                                                   const int* __restrict__ list,
                                                                   const int4* __restrict__ en,
                                                                   const double* __restrict__ fields,
                                                                   double* nodal) {
    const double root_three = 1.7320508075688772935;
    const double alpha = mul(0.5, add(1.0, root_three)), beta = mul(0.5, sub(1.0, root_three));
    const double aa = mul(alpha, alpha), ab = mul(alpha, beta), bb = mul(beta, beta);
    const double ext[4][4] = {{aa, ab, bb, ab}, {ab, aa, ab, bb}, {bb, ab, aa, ab}, {ab, bb, ab, aa}};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        double s[3] = {0.0, 0.0, 0.0};
        int count = 0;
        for (int k = ptr[i]; k < ptr[i + 1]; ++k) {  // elements in ascending order
            const int e = list[k];
            const int4 q = en[e];
            const int nd[4] = {q.x, q.y, q.z, q.w};
            const double* fe = fields + 35LL * e;
            for (int a = 0; a < 4; ++a) {
                if (nd[a] != i) continue;
                for (int c = 0; c < 3; ++c)
                    for (int g = 0; g < 4; ++g) s[c] = add(s[c], mul(ext[a][g], fe[7 * (g + 1) + 3 + c]));
                ++count;
            }
        }
        double* out = nodal + 4LL * i;
        if (count == 0) {
            out[0] = out[1] = out[2] = out[3] = 0.0;
            continue;
        }
        for (int c = 0; c < 3; ++c) out[c] = div(s[c], static_cast<double>(count));
        out[3] = von_mises(out[0], out[1], out[2]);
    }
}

}  // namespace

void launch_postprocess(Context& c, const double* u, double* fields, double* nodal) {
    const int ne = static_cast<int>(c.n_elem), nn = static_cast<int>(c.n_nodes);
    ensure_node_elements(c);
    if (ne > 0)
        element_fields_kernel<<<grid_for(ne, kThreads, 16 * c.num_sms), kThreads, 0, c.stream>>>(
            ne, c.xy, c.elem_nodes, c.elem_mat, c.mat_young, c.mat_nu, c.plane_mode, u, fields, c.status);
    nodal_smoothing_kernel<<<grid_for(nn, kThreads, 16 * c.num_sms), kThreads, 0, c.stream>>>(
        nn, c.ne_ptr, c.ne_list, c.elem_nodes, fields, nodal);
    c.launches += ne > 0 ? 2 : 1;
    LF_CUDA(cudaGetLastError());
}

}  // namespace lfgpu
