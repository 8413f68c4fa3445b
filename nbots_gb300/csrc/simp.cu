// SIMP sensitivities on the GPU (no counterpart in nbots, which lists a
// topology-optimisation bot without code).
//
// With E_e(rho) = Emin + rho_e^p (E0 - Emin), the element stiffness is
// K_e = E_e Ke0_e where Ke0_e is the element stiffness for E = 1, so for any
// objective J with adjoint lambda (K lambda = dJ/du):
//     dJ/drho_e = -dE_e/drho_e * lambda_e^T Ke0_e u_e,
//     dE_e/drho_e = p rho_e^(p-1) (E0 - Emin).
// Compliance F^T u is self-adjoint (lambda = u); one nodal output u_k needs
// one adjoint solve K lambda = e_k.  With nbots' Dirichlet elimination
// (rows and columns of constrained dofs replaced by the identity) both u and
// lambda vanish at homogeneous Dirichlet dofs, so the full Ke0 may be used.
//
// One thread per element integrates Ke0 (2x2 Gauss for Q4, one point for
// T3, nbots' tables) in FP64 with FMAs and contracts it with a_e and b_e on
// the fly; Ke0 is never stored.
#include <cstdint>

#include "common.cuh"

namespace {

#define QD 0.394337567297
#define QE 0.105662432703
__constant__ double c_dpsi4[16] = {-QD, -QD, -QE, -QE, QD, QD, QE, QE,
                                   QE,  QE,  QD,  QD,  -QE, -QE, -QD, -QD};
__constant__ double c_deta4[16] = {-QD, -QE, -QE, -QD, -QE, -QD, -QD, -QE,
                                   QE,  QD,  QD,  QE,  QD,  QE,  QE,  QD};
__constant__ double c_dpsi3[3] = {-1.0, 1.0, 0.0};
__constant__ double c_deta3[3] = {-1.0, 0.0, 1.0};

template <int NN>
__global__ void __launch_bounds__(128) k_simp_sens(uint32_t N_elem, const double* __restrict__ nod,
                                                   const uint32_t* __restrict__ conn, double nu,
                                                   double th, const double* __restrict__ rho,
                                                   double penal, double E0, double Emin,
                                                   const double* __restrict__ a,
                                                   const double* __restrict__ b,
                                                   double* __restrict__ out) {
    constexpr int NGP = NN == 4 ? 4 : 1;
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= N_elem) return;
    double x[NN], y[NN], ax[NN], ay[NN], bx[NN], by[NN];
#pragma unroll
    for (int i = 0; i < NN; i++) {
        const uint32_t n = conn[(size_t)e * NN + i];
        x[i] = nod[2 * (size_t)n];
        y[i] = nod[2 * (size_t)n + 1];
        ax[i] = a[2 * (size_t)n];
        ay[i] = a[2 * (size_t)n + 1];
        bx[i] = b[2 * (size_t)n];
        by[i] = b[2 * (size_t)n + 1];
    }
    // plane stress with E = 1 (formulas.c:48-54)
    const double D0 = 1.0 / (1.0 - nu * nu), D1 = nu * D0, D2 = D0, D3 = 1.0 / (2.0 * (1.0 + nu));
    const double w = NN == 4 ? 1.0 : 0.5;
    double s = 0.0;
#pragma unroll
    for (int gp = 0; gp < NGP; gp++) {
        double dxp = 0.0, dyp = 0.0, dxe = 0.0, dye = 0.0;
#pragma unroll
        for (int i = 0; i < NN; i++) {
            const double dp = NN == 4 ? c_dpsi4[i * 4 + gp] : c_dpsi3[i];
            const double de = NN == 4 ? c_deta4[i * 4 + gp] : c_deta3[i];
            dxp = fma(dp, x[i], dxp);
            dxe = fma(de, x[i], dxe);
            dyp = fma(dp, y[i], dyp);
            dye = fma(de, y[i], dye);
        }
        const double detJ = dxp * dye - dyp * dxe;
        const double inv = 1.0 / detJ;
        // strains of a and b at this point: B a and B b
        double ea0 = 0.0, ea1 = 0.0, ea2 = 0.0, eb0 = 0.0, eb1 = 0.0, eb2 = 0.0;
#pragma unroll
        for (int i = 0; i < NN; i++) {
            const double dp = NN == 4 ? c_dpsi4[i * 4 + gp] : c_dpsi3[i];
            const double de = NN == 4 ? c_deta4[i * 4 + gp] : c_deta3[i];
            const double dx = (dye * dp - dyp * de) * inv;
            const double dy = (-dxe * dp + dxp * de) * inv;
            ea0 = fma(dx, ax[i], ea0);
            ea1 = fma(dy, ay[i], ea1);
            ea2 = fma(dy, ax[i], fma(dx, ay[i], ea2));
            eb0 = fma(dx, bx[i], eb0);
            eb1 = fma(dy, by[i], eb1);
            eb2 = fma(dy, bx[i], fma(dx, by[i], eb2));
        }
        // (B a)^T D (B b) detJ t w
        const double q = ea0 * (D0 * eb0 + D1 * eb1) + ea1 * (D1 * eb0 + D2 * eb1) + ea2 * D3 * eb2;
        s = fma(q, detJ * th * w, s);
    }
    const double r = rho[e];
    const double dE = penal * pow(r, penal - 1.0) * (E0 - Emin);
    out[e] = -dE * s;
}

// E_e = Emin + rho_e^p (E0 - Emin), rounded step by step (no contraction).
__global__ void k_simp_modulus(uint32_t n, const double* __restrict__ rho, double penal,
                               double E0, double Emin, double* __restrict__ E) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) E[e] = nbg::add(Emin, nbg::mul(pow(rho[e], penal), nbg::sub(E0, Emin)));
}

}  // namespace

extern "C" int nbg_simp_modulus_f64(uint32_t N_elem, const double* rho, double penal, double E0,
                                    double Emin, double* E, void* stream) {
    if (N_elem == 0) return NBG_OK;
    k_simp_modulus<<<(N_elem + 255) / 256, 256, 0, (cudaStream_t)stream>>>(N_elem, rho, penal,
                                                                          E0, Emin, E);
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}

extern "C" int nbg_simp_sensitivity_f64(uint32_t nen, uint32_t N_elem, const double* nod,
                                        const uint32_t* conn, double nu, double thickness,
                                        const double* rho, double penal, double E0, double Emin,
                                        const double* a, const double* b, double* out,
                                        void* stream) {
    if (N_elem == 0) return NBG_OK;
    const unsigned g = (N_elem + 127) / 128;
    cudaStream_t s = (cudaStream_t)stream;
    if (nen == 4)
        k_simp_sens<4><<<g, 128, 0, s>>>(N_elem, nod, conn, nu, thickness, rho, penal, E0, Emin,
                                         a, b, out);
    else if (nen == 3)
        k_simp_sens<3><<<g, 128, 0, s>>>(N_elem, nod, conn, nu, thickness, rho, penal, E0, Emin,
                                         a, b, out);
    else
        return NBG_ERR_ARG;
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}
