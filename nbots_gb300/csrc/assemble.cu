// FEM assembly kernels: element stiffness, deterministic row-gather into the
// nbots CSR pattern, load increments, Dirichlet elimination, strain, stress.
//
// Parity: every floating-point step repeats nbots' operation order with
// explicitly rounded operations (no FMA), so K, F, strain and stress equal
// the reference's bits.  The gather visits, for each CSR 2x2 node block, the
// elements shared by its two nodes in ascending element id: that is the
// order in which nbots' serial element loop adds into each slot
// (pde_bot/finite_element/solid_mechanics/pipeline.c:60-69), so no float
// atomics and no colouring are needed for bitwise determinism.
#include <cstdint>

#include "common.cuh"

using namespace nbg;

namespace {

// nbots' element tables (pde_bot/finite_element/element.c:54-121), Q4 with
// its 12-significant-digit truncation; node-major [node * N_gp + gp].
#define QA 0.622008467928
#define QB 0.166666666667
#define QC 0.044658198739
#define QD 0.394337567297
#define QE 0.105662432703
__constant__ double c_q4_N[16] = {QA, QB, QC, QB, QB, QA, QB, QC, QC, QB, QA, QB, QB, QC, QB, QA};
__constant__ double c_q4_dpsi[16] = {-QD, -QD, -QE, -QE, QD, QD, QE, QE,
                                     QE,  QE,  QD,  QD,  -QE, -QE, -QD, -QD};
__constant__ double c_q4_deta[16] = {-QD, -QE, -QE, -QD, -QE, -QD, -QD, -QE,
                                     QE,  QD,  QD,  QE,  QD,  QE,  QE,  QD};
__constant__ double c_t3_N[3] = {1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0};
__constant__ double c_t3_dpsi[3] = {-1.0, 1.0, 0.0};
__constant__ double c_t3_deta[3] = {-1.0, 0.0, 1.0};

template <int NN> struct Tab;
template <> struct Tab<4> {
    static constexpr int NGP = 4;
    __device__ static double N(int i, int g) { return c_q4_N[i * 4 + g]; }
    __device__ static double dpsi(int i, int g) { return c_q4_dpsi[i * 4 + g]; }
    __device__ static double deta(int i, int g) { return c_q4_deta[i * 4 + g]; }
    __device__ static double w(int) { return 1.0; }
};
template <> struct Tab<3> {
    static constexpr int NGP = 1;
    __device__ static double N(int i, int g) { return c_t3_N[i]; }
    __device__ static double dpsi(int i, int g) { return c_t3_dpsi[i]; }
    __device__ static double deta(int i, int g) { return c_t3_deta[i]; }
    __device__ static double w(int) { return 0.5; }
};

// nb_fem_get_jacobian + nb_fem_get_derivatives (utils.c:9-60)
template <int NN>
__device__ __forceinline__ double shape_derivs(const double (&x)[NN], const double (&y)[NN],
                                               int gp, double (&dx)[NN], double (&dy)[NN]) {
    double dx_dpsi = 0.0, dy_dpsi = 0.0, dx_deta = 0.0, dy_deta = 0.0;
#pragma unroll
    for (int i = 0; i < NN; i++) {
        double dp = Tab<NN>::dpsi(i, gp), de = Tab<NN>::deta(i, gp);
        dx_dpsi = add(dx_dpsi, mul(dp, x[i]));
        dx_deta = add(dx_deta, mul(de, x[i]));
        dy_dpsi = add(dy_dpsi, mul(dp, y[i]));
        dy_deta = add(dy_deta, mul(de, y[i]));
    }
    double detJ = sub(mul(dx_dpsi, dy_deta), mul(dy_dpsi, dx_deta));
    double j0 = dvd(dy_deta, detJ), j1 = dvd(-dy_dpsi, detJ);
    double j2 = dvd(-dx_deta, detJ), j3 = dvd(dx_dpsi, detJ);
#pragma unroll
    for (int i = 0; i < NN; i++) {
        double dp = Tab<NN>::dpsi(i, gp), de = Tab<NN>::deta(i, gp);
        dx[i] = add(mul(j0, dp), mul(j1, de));
        dy[i] = add(mul(j2, dp), mul(j3, de));
    }
    return detJ;
}

// One entry of B^T D B at a Gauss point before the detJ*t*w scaling
// (pipeline_sum_gauss_point, pipeline.c:197-212).
template <int NN>
__device__ __forceinline__ double bdb(int a, int b, const double (&dx)[NN], const double (&dy)[NN],
                                      double D0, double D1, double D2, double D3) {
    const int i = a >> 1, j = b >> 1;
    if (!(a & 1) && !(b & 1)) return add(mul(mul(dx[i], dx[j]), D0), mul(mul(dy[i], dy[j]), D3));
    if (!(a & 1) && (b & 1)) return add(mul(mul(dx[i], dy[j]), D1), mul(mul(dy[i], dx[j]), D3));
    if ((a & 1) && !(b & 1)) return add(mul(mul(dy[i], dx[j]), D1), mul(mul(dx[i], dy[j]), D3));
    return add(mul(mul(dy[i], dy[j]), D2), mul(mul(dx[i], dx[j]), D3));
}

// Ke is exactly symmetric in nbots' arithmetic (the mirrored entry multiplies
// the same factors), so only the upper triangle is integrated.  Output
// layout is entry-major: Ke[(a * 2NN + b) * N_elem + e], Fe[a * N_elem + e].
template <int NN>
__global__ void __launch_bounds__(128) k_element(uint32_t N_elem, const double* __restrict__ nod,
                                                 const uint32_t* __restrict__ conn,
                                                 const double* __restrict__ E, double nu, double th,
                                                 double density, int self_weight, double gx,
                                                 double gy, const uint8_t* __restrict__ enabled,
                                                 const double* __restrict__ dmg,
                                                 double* __restrict__ Ke, double* __restrict__ Fe,
                                                 uint32_t* distorted) {
    constexpr int ND = 2 * NN;
    constexpr int NGP = Tab<NN>::NGP;
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= N_elem) return;
    double x[NN], y[NN];
#pragma unroll
    for (int i = 0; i < NN; i++) {
        uint32_t n = conn[(size_t)e * NN + i];
        x[i] = nod[2 * (size_t)n];
        y[i] = nod[2 * (size_t)n + 1];
    }
    // assemble_element (pipeline.c:93-98) and set_plane_stress (formulas.c:48-54)
    double D0 = 1e-6, D1 = 1e-6, D2 = 1e-6, D3 = 1e-6, dens = 1e-6;
    if (enabled == nullptr || enabled[e]) {
        double Ee = E[e];
        D0 = dvd(Ee, sub(1.0, mul(nu, nu)));
        D1 = mul(nu, D0);
        D2 = D0;
        D3 = dvd(Ee, mul(2.0, add(1.0, nu)));
        dens = density;
    }
    double fx = 0.0, fy = 0.0;
    if (self_weight) {
        fx = mul(gx, dens);
        fy = mul(gy, dens);
    }
    double k[ND * (ND + 1) / 2];
    double f[ND];
#pragma unroll
    for (int i = 0; i < ND * (ND + 1) / 2; i++) k[i] = 0.0;
#pragma unroll
    for (int i = 0; i < ND; i++) f[i] = 0.0;
#pragma unroll
    for (int gp = 0; gp < NGP; gp++) {
        double dx[NN], dy[NN];
        double detJ = shape_derivs<NN>(x, y, gp, dx, dy);
        if (detJ < 0) {
            atomicMin(distorted, e);
            return;
        }
        const double wp = Tab<NN>::w(gp);
        // DMG_pipeline_assemble_system (static_damage2D.c:527-534): each
        // Gauss point scales D by (1 - damage) first
        double G0 = D0, G1 = D1, G2 = D2, G3 = D3;
        if (dmg != nullptr) {
            const double keep = sub(1.0, dmg[(size_t)e * NGP + gp]);
            G0 = mul(D0, keep);
            G1 = mul(D1, keep);
            G2 = mul(D2, keep);
            G3 = mul(D3, keep);
        }
        int o = 0;
#pragma unroll
        for (int a = 0; a < ND; a++) {
#pragma unroll
            for (int b = a; b < ND; b++) {
                double s = bdb<NN>(a, b, dx, dy, G0, G1, G2, G3);
                k[o] = add(k[o], mul(mul(mul(s, detJ), th), wp));
                o++;
            }
        }
#pragma unroll
        for (int i = 0; i < NN; i++) {
            double integral = mul(mul(mul(Tab<NN>::N(i, gp), detJ), th), wp);
            f[2 * i] = add(f[2 * i], mul(integral, fx));
            f[2 * i + 1] = add(f[2 * i + 1], mul(integral, fy));
        }
    }
    int o = 0;
#pragma unroll
    for (int a = 0; a < ND; a++) {
#pragma unroll
        for (int b = a; b < ND; b++) {
            Ke[(size_t)(a * ND + b) * N_elem + e] = k[o];
            if (b != a) Ke[(size_t)(b * ND + a) * N_elem + e] = k[o];
            o++;
        }
    }
#pragma unroll
    for (int i = 0; i < ND; i++) Fe[(size_t)i * N_elem + e] = f[i];
}

// One thread per node v: its two CSR rows share one sorted column list made
// of (2w, 2w+1) pairs (sparse.c:36-52), so each pair is one 2x2 block.
template <int NN>
__global__ void __launch_bounds__(128) k_gather(uint32_t N_nod, uint32_t N_elem,
                                                const uint32_t* __restrict__ inc_ptr,
                                                const uint32_t* __restrict__ inc_elem,
                                                const uint8_t* __restrict__ inc_local,
                                                const uint32_t* __restrict__ rp,
                                                const uint32_t* __restrict__ ci,
                                                const double* __restrict__ Ke,
                                                const double* __restrict__ Fe,
                                                double* __restrict__ K, double* __restrict__ F,
                                                unsigned long long* matched) {
    constexpr int ND = 2 * NN;
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= N_nod) return;
    const uint32_t a0 = inc_ptr[v], a1 = inc_ptr[v + 1];
    const uint32_t r0 = rp[2 * v], len = rp[2 * v + 1] - r0, r1 = rp[2 * v + 1];
    unsigned long long cnt = 0;
    for (uint32_t kk = 0; kk < len; kk += 2) {
        const uint32_t c = ci[r0 + kk];
        const uint32_t w = c >> 1;
        const bool paired = !(c & 1) && kk + 1 < len && ci[r0 + kk + 1] == c + 1;
        double s00 = 0.0, s01 = 0.0, s10 = 0.0, s11 = 0.0;
        uint32_t ia = a0, ib = inc_ptr[w];
        const uint32_t ib1 = inc_ptr[w + 1];
        while (paired && ia < a1 && ib < ib1) {
            const uint32_t ea = inc_elem[ia], eb = inc_elem[ib];
            if (ea < eb) { ia++; continue; }
            if (eb < ea) { ib++; continue; }
            const int i = inc_local[ia], j = inc_local[ib];
            const size_t P = N_elem;
            s00 = add(s00, Ke[(size_t)((2 * i) * ND + 2 * j) * P + ea]);
            s01 = add(s01, Ke[(size_t)((2 * i) * ND + 2 * j + 1) * P + ea]);
            s10 = add(s10, Ke[(size_t)((2 * i + 1) * ND + 2 * j) * P + ea]);
            s11 = add(s11, Ke[(size_t)((2 * i + 1) * ND + 2 * j + 1) * P + ea]);
            cnt++;
            ia++;
            ib++;
        }
        if (!paired) {
            // not a node block: nbots' pattern never makes one; leave the
            // slot at zero and make the pair count disagree
            K[r0 + kk] = 0.0;
            K[r1 + kk] = 0.0;
            cnt += 1ull << 40;
            kk -= 1;  // advance by one column only
            continue;
        }
        K[r0 + kk] = s00;
        K[r0 + kk + 1] = s01;
        K[r1 + kk] = s10;
        K[r1 + kk + 1] = s11;
    }
    double f0 = 0.0, f1 = 0.0;
    for (uint32_t ia = a0; ia < a1; ia++) {
        const uint32_t e = inc_elem[ia];
        const int i = inc_local[ia];
        f0 = add(f0, Fe[(size_t)(2 * i) * N_elem + e]);
        f1 = add(f1, Fe[(size_t)(2 * i + 1) * N_elem + e]);
    }
    F[2 * v] = f0;
    F[2 * v + 1] = f1;
    if (cnt) atomicAdd(matched, cnt);
}

__global__ void k_increments(uint32_t n_groups, const uint32_t* __restrict__ idx,
                             const uint32_t* __restrict__ gptr, const double* __restrict__ inc,
                             double* __restrict__ F) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_groups) return;
    double f = F[idx[g]];
    for (uint32_t k = gptr[g]; k < gptr[g + 1]; k++) f = add(f, inc[k]);
    F[idx[g]] = f;
}

constexpr int kMaxRowEvents = 96;

// Thread per row j: replay, in global event order, every Dirichlet event
// that touches row j: its own (row reset to the identity, F[j] = value) and
// those of the dofs in its columns (K[j][d] = 0, F[j] -= K[j][d] * value).
__global__ void __launch_bounds__(128) k_dirichlet(uint32_t N, const uint32_t* __restrict__ rp,
                                                   const uint32_t* __restrict__ ci,
                                                   double* __restrict__ K, double* __restrict__ F,
                                                   const uint32_t* __restrict__ ev_ptr,
                                                   const uint32_t* __restrict__ ev_of,
                                                   const double* __restrict__ ev_val, int* status) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    uint32_t evn[kMaxRowEvents];
    uint32_t pos[kMaxRowEvents];  // CSR slot of the column, or UINT32_MAX for the row's own event
    int n = 0;
    const uint32_t b = rp[j], e = rp[j + 1];
    for (uint32_t k = b; k < e; k++) {
        const uint32_t c = ci[k];
        for (uint32_t t = ev_ptr[c]; t < ev_ptr[c + 1]; t++) {
            if (n == kMaxRowEvents) {
                atomicCAS(status, 0, NBG_ERR_ARG);
                return;
            }
            evn[n] = ev_of[t];
            pos[n] = c == j ? 0xffffffffu : k;
            n++;
        }
    }
    if (n == 0) return;
    for (int a = 1; a < n; a++) {  // insertion sort by event number
        uint32_t ke = evn[a], kp = pos[a];
        int q = a - 1;
        while (q >= 0 && evn[q] > ke) {
            evn[q + 1] = evn[q];
            pos[q + 1] = pos[q];
            q--;
        }
        evn[q + 1] = ke;
        pos[q + 1] = kp;
    }
    double f = F[j];
    for (int a = 0; a < n; a++) {
        const double val = ev_val[evn[a]];
        if (pos[a] == 0xffffffffu) {
            for (uint32_t k = b; k < e; k++) K[k] = ci[k] == j ? 1.0 : 0.0;
            f = val;
        } else {
            const double var = K[pos[a]];
            K[pos[a]] = 0.0;
            f = sub(f, mul(var, val));
        }
    }
    F[j] = f;
}

template <int NN>
__global__ void __launch_bounds__(128) k_strain(uint32_t N_elem, const double* __restrict__ nod,
                                                const uint32_t* __restrict__ conn,
                                                const double* __restrict__ u,
                                                double* __restrict__ strain) {
    constexpr int NGP = Tab<NN>::NGP;
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= N_elem) return;
    double x[NN], y[NN], ux[NN], uy[NN];
#pragma unroll
    for (int i = 0; i < NN; i++) {
        uint32_t n = conn[(size_t)e * NN + i];
        x[i] = nod[2 * (size_t)n];
        y[i] = nod[2 * (size_t)n + 1];
        ux[i] = u[2 * (size_t)n];
        uy[i] = u[2 * (size_t)n + 1];
    }
    bool stop = false;
#pragma unroll
    for (int gp = 0; gp < NGP; gp++) {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        if (!stop) {
            double dx[NN], dy[NN];
            double detJ = shape_derivs<NN>(x, y, gp, dx, dy);
            if (detJ < 0) {
                stop = true;  // get_element_strain leaves the remaining points at zero
            } else {
#pragma unroll
                for (int i = 0; i < NN; i++) {
                    s0 = add(s0, mul(dx[i], ux[i]));
                    s1 = add(s1, mul(dy[i], uy[i]));
                    s2 = add(s2, add(mul(dy[i], ux[i]), mul(dx[i], uy[i])));
                }
            }
        }
        const size_t id = (size_t)e * NGP + gp;
        strain[id * 3] = s0;
        strain[id * 3 + 1] = s1;
        strain[id * 3 + 2] = s2;
    }
}

__global__ void k_stress(uint32_t N_elem, int ngp, const double* __restrict__ E, double nu,
                         const uint8_t* __restrict__ enabled, const double* __restrict__ strain,
                         double* __restrict__ stress) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= N_elem) return;
    double D0 = 1e-6, D1 = 1e-6, D2 = 1e-6, D3 = 1e-6;
    if (enabled == nullptr || enabled[e]) {
        D0 = dvd(E[e], sub(1.0, mul(nu, nu)));
        D1 = mul(nu, D0);
        D2 = D0;
        D3 = dvd(E[e], mul(2.0, add(1.0, nu)));
    }
    for (int g = 0; g < ngp; g++) {
        const size_t id = (size_t)e * ngp + g;
        const double e0 = strain[id * 3], e1 = strain[id * 3 + 1], e2 = strain[id * 3 + 2];
        stress[id * 3] = add(mul(e0, D0), mul(e1, D1));
        stress[id * 3 + 1] = add(mul(e0, D1), mul(e1, D2));
        stress[id * 3 + 2] = mul(e2, D3);
    }
}

// Principal stresses per Gauss point (pipeline.c:321-340): the mean of the
// normal stresses plus and minus the radius of Mohr's circle, nbots'
// operation order without contraction and a correctly rounded square root.
__global__ void k_main_stress(uint32_t n, const double* __restrict__ stress,
                              double* __restrict__ main_stress) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double sx = stress[(size_t)i * 3], sy = stress[(size_t)i * 3 + 1];
    const double txy = stress[(size_t)i * 3 + 2];
    const double avg = mul(0.5, add(sx, sy));
    const double d = sub(sx, sy);
    const double R = __dsqrt_rn(add(mul(0.25, mul(d, d)), mul(txy, txy)));
    main_stress[(size_t)i * 2] = add(avg, R);
    main_stress[(size_t)i * 2 + 1] = sub(avg, R);
}

inline unsigned nblk(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

extern "C" int nbg_main_stress_f64(uint32_t nen, uint32_t N_elem, const double* stress,
                                   double* main_stress, void* stream) {
    if (nen != 3 && nen != 4) return NBG_ERR_ARG;
    const uint64_t n = (uint64_t)N_elem * (nen == 4 ? 4 : 1);
    if (n == 0) return NBG_OK;
    if (n > UINT32_MAX) return NBG_ERR_ARG;
    k_main_stress<<<nblk(n, 256), 256, 0, (cudaStream_t)stream>>>((uint32_t)n, stress,
                                                                  main_stress);
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}

extern "C" int nbg_element_stiffness_damage_f64(uint32_t nen, uint32_t N_elem, const double* nod,
                                                const uint32_t* conn, const double* E, double nu,
                                                double thickness, double density,
                                                int self_weight, double gx, double gy,
                                                const uint8_t* enabled, const double* damage,
                                                double* Ke, double* Fe, uint32_t* distorted,
                                                void* stream) {
    if (N_elem == 0) return NBG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (nen == 4)
        k_element<4><<<nblk(N_elem, 128), 128, 0, s>>>(N_elem, nod, conn, E, nu, thickness, density,
                                                       self_weight, gx, gy, enabled, damage, Ke,
                                                       Fe, distorted);
    else if (nen == 3)
        k_element<3><<<nblk(N_elem, 128), 128, 0, s>>>(N_elem, nod, conn, E, nu, thickness, density,
                                                       self_weight, gx, gy, enabled, damage, Ke,
                                                       Fe, distorted);
    else
        return NBG_ERR_ARG;
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}

extern "C" int nbg_element_stiffness_f64(uint32_t nen, uint32_t N_elem, const double* nod,
                                         const uint32_t* conn, const double* E, double nu,
                                         double thickness, double density, int self_weight,
                                         double gx, double gy, const uint8_t* enabled, double* Ke,
                                         double* Fe, uint32_t* distorted, void* stream) {
    return nbg_element_stiffness_damage_f64(nen, N_elem, nod, conn, E, nu, thickness, density,
                                            self_weight, gx, gy, enabled, nullptr, Ke, Fe,
                                            distorted, stream);
}

extern "C" int nbg_gather_assemble_f64(uint32_t nen, uint32_t N_nod, uint32_t N_elem,
                                       const uint32_t* inc_ptr, const uint32_t* inc_elem,
                                       const uint8_t* inc_local, const uint32_t* row_ptr,
                                       const uint32_t* col_idx, const double* Ke, const double* Fe,
                                       double* K, double* F, unsigned long long* matched,
                                       void* stream) {
    if (N_nod == 0) return NBG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (nen == 4)
        k_gather<4><<<nblk(N_nod, 128), 128, 0, s>>>(N_nod, N_elem, inc_ptr, inc_elem, inc_local,
                                                     row_ptr, col_idx, Ke, Fe, K, F, matched);
    else if (nen == 3)
        k_gather<3><<<nblk(N_nod, 128), 128, 0, s>>>(N_nod, N_elem, inc_ptr, inc_elem, inc_local,
                                                     row_ptr, col_idx, Ke, Fe, K, F, matched);
    else
        return NBG_ERR_ARG;
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}

extern "C" int nbg_apply_increments_f64(uint32_t n_groups, const uint32_t* idx_of_group,
                                        const uint32_t* group_ptr, const double* inc, double* F,
                                        void* stream) {
    if (n_groups == 0) return NBG_OK;
    k_increments<<<nblk(n_groups, 128), 128, 0, (cudaStream_t)stream>>>(n_groups, idx_of_group,
                                                                       group_ptr, inc, F);
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}

extern "C" int nbg_dirichlet_f64(uint32_t N, const uint32_t* row_ptr, const uint32_t* col_idx,
                                 double* K, double* F, const uint32_t* ev_ptr,
                                 const uint32_t* ev_of, const double* ev_val, int* status,
                                 void* stream) {
    if (N == 0) return NBG_OK;
    k_dirichlet<<<nblk(N, 128), 128, 0, (cudaStream_t)stream>>>(N, row_ptr, col_idx, K, F, ev_ptr,
                                                               ev_of, ev_val, status);
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}

extern "C" int nbg_strain_f64(uint32_t nen, uint32_t N_elem, const double* nod,
                              const uint32_t* conn, const double* u, double* strain,
                              void* stream) {
    if (N_elem == 0) return NBG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (nen == 4)
        k_strain<4><<<nblk(N_elem, 128), 128, 0, s>>>(N_elem, nod, conn, u, strain);
    else if (nen == 3)
        k_strain<3><<<nblk(N_elem, 128), 128, 0, s>>>(N_elem, nod, conn, u, strain);
    else
        return NBG_ERR_ARG;
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}

extern "C" int nbg_stress_f64(uint32_t nen, uint32_t N_elem, const double* E, double nu,
                              const uint8_t* enabled, const double* strain, double* stress,
                              void* stream) {
    if (N_elem == 0) return NBG_OK;
    if (nen != 3 && nen != 4) return NBG_ERR_ARG;
    k_stress<<<nblk(N_elem, 128), 128, 0, (cudaStream_t)stream>>>(N_elem, nen == 4 ? 4 : 1, E, nu,
                                                                 enabled, strain, stress);
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}
