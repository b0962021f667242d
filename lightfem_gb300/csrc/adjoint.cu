// Element sensitivities of an objective with respect to the element moduli (no
// counterpart in the reference; the FP64 CPU restatement in the oracle checks it).
//
// K = sum_e E_e Khat_e, so for J(u(E)) with K lambda = dJ/du:
//     dJ/dE_e = -lambda_e^T Khat_e u_e = -lambda_e^T K_e u_e / E_e.
// Khat_e is rebuilt on the fly from the element geometry with a unit modulus
// (the same 2x2 block form as the assembly kernel), so the kernel streams only the
// connectivity, the material index and the two gathered vectors: about
// 16 + 4 + 2 x 64 bytes per element, most of the vector bytes from L2.
#include "common.cuh"
#include "kernels.hpp"

namespace lfgpu {
namespace {

constexpr double kG = 0.57735026918962576451;

__global__ void adjoint_grad_kernel(int E, const double2* __restrict__ xy, const int4* __restrict__ en,
                                    const int* __restrict__ mat, const double* __restrict__ nu_t,
                                    const double* __restrict__ thick, int plane_strain,
                                    const double2* __restrict__ u, const double2* __restrict__ lam,
                                    double* __restrict__ grad, DeviceStatus* status) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const int4 nd = __ldg(en + e);
    const int m = __ldg(mat + e);
    const double nu = __ldg(nu_t + m), t = __ldg(thick + m);
    const int nodes[4] = {nd.x, nd.y, nd.z, nd.w};
    double X[4], Y[4], ux[4], uy[4], lx[4], ly[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const double2 c = __ldg(xy + nodes[i]);
        const double2 uv = __ldg(u + nodes[i]);
        const double2 lv = __ldg(lam + nodes[i]);
        X[i] = c.x;
        Y[i] = c.y;
        ux[i] = uv.x;
        uy[i] = uv.y;
        lx[i] = lv.x;
        ly[i] = lv.y;
    }
    double d00, d01, d22;
    if (!plane_strain) {
        const double f = 1.0 / (1.0 - nu * nu);
        d00 = f;
        d01 = f * nu;
        d22 = f * (1.0 - nu) * 0.5;
    } else {
        const double f = 1.0 / ((1.0 + nu) * (1.0 - 2.0 * nu));
        d00 = f * (1.0 - nu);
        d01 = f * nu;
        d22 = f * (1.0 - 2.0 * nu) * 0.5;
    }
    // lambda^T Khat u = sum_g w_g (B lambda)^T Dhat (B u): strains of both fields at
    // each Gauss point, then the 3x3 contraction.
    double acc = 0.0;
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
        ok = ok && det > 1.0e-14 && isfinite(det);
        const double inv = 1.0 / det;
        double eu[3] = {0, 0, 0}, el[3] = {0, 0, 0};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const double nx = (j11 * dxi[i] - j10 * deta[i]) * inv;
            const double ny = (-j01 * dxi[i] + j00 * deta[i]) * inv;
            eu[0] += nx * ux[i];
            eu[1] += ny * uy[i];
            eu[2] += ny * ux[i] + nx * uy[i];
            el[0] += nx * lx[i];
            el[1] += ny * ly[i];
            el[2] += ny * lx[i] + nx * ly[i];
        }
        const double s0 = d00 * eu[0] + d01 * eu[1];
        const double s1 = d01 * eu[0] + d00 * eu[1];
        const double s2 = d22 * eu[2];
        acc += det * t * (el[0] * s0 + el[1] * s1 + el[2] * s2);
    }
    if (!ok) {
        record_failure(status, LFGPU_ERR_JACOBIAN, e);
        return;
    }
    grad[e] = -acc;
}

}  // namespace

void launch_adjoint_grad(Context& c, const double* u, const double* lam, double* grad) {
    const int E = static_cast<int>(c.n_elem);
    if (E == 0) return;
    adjoint_grad_kernel<<<grid_for(E, 128), 128, 0, c.stream>>>(
        E, c.xy, c.elem_nodes, c.elem_mat, c.mat_nu, c.mat_t, c.plane_mode == LFGPU_PLANE_STRAIN,
        reinterpret_cast<const double2*>(u), reinterpret_cast<const double2*>(lam), grad, c.status);
    c.launches += 1;
    LF_CUDA(cudaGetLastError());
}

}  // namespace lfgpu
