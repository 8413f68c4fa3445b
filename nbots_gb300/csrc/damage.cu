// Kernels of nbots' quasi-static damage solve
// (pde_bot/finite_element/solid_mechanics/static_damage2D.c:239-470):
//   - strain and tension damage per Gauss point (DMG_pipeline_compute_strain,
//     :571-631, with tension_damage, :134-182, and get_clfd, :633-647);
//   - the residual F - K u and its squared norm (:343-351);
//   - Gauss-Seidel (solver_bot/sparse/solvers/gauss_seidel.c:14-58, with
//     nb_sparse_forward_solve, triangular.c:14-32), the fallback when the
//     conjugate gradient does not converge.
// The damaged element stiffness is the assembly kernel's (assemble.cu) with
// a per-Gauss-point damage array.
//
// Per-element and per-row arithmetic repeats nbots' operation order with
// explicitly rounded operations.  The exponential is CUDA's exp (within one
// ulp of the C library's), and the sums over all rows use a fixed tree
// instead of nbots' left-to-right loop, so damage and norms agree with nbots'
// to rounding, not bit for bit.
//
// Gauss-Seidel runs as one block that keeps the whole solve on the device.
// The forward substitution x_i = (c_i - sum_{j<i} K_ij x_j) / K_ii is
// level-scheduled: the host groups the rows so that every row of a level
// depends only on rows of earlier levels (nbg_host_lower_levels), and the
// block solves one level between two barriers.  Each row still subtracts its
// terms in nbots' order, so the iterates are nbots' own.
#include <cstdint>

#include "persist.cuh"

using namespace nbg;

namespace {

// Q4 and T3 tables of nbots' element.c:54-121 (node-major, 12 significant
// digits for Q4), repeated from assemble.cu so that this unit stands alone.
#define QD 0.394337567297
#define QE 0.105662432703
__constant__ double c_q4_dpsi[16] = {-QD, -QD, -QE, -QE, QD, QD, QE, QE,
                                     QE,  QE,  QD,  QD,  -QE, -QE, -QD, -QD};
__constant__ double c_q4_deta[16] = {-QD, -QE, -QE, -QD, -QE, -QD, -QD, -QE,
                                     QE,  QD,  QD,  QE,  QD,  QE,  QE,  QD};
__constant__ double c_t3_dpsi[3] = {-1.0, 1.0, 0.0};
__constant__ double c_t3_deta[3] = {-1.0, 0.0, 1.0};

template <int NN> struct Tab;
template <> struct Tab<4> {
    static constexpr int NGP = 4;
    __device__ static double dpsi(int i, int g) { return c_q4_dpsi[i * 4 + g]; }
    __device__ static double deta(int i, int g) { return c_q4_deta[i * 4 + g]; }
};
template <> struct Tab<3> {
    static constexpr int NGP = 1;
    __device__ static double dpsi(int i, int) { return c_t3_dpsi[i]; }
    __device__ static double deta(int i, int) { return c_t3_deta[i]; }
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

// nbots' MAX(a, b) = ((a) > (b)) ? (a) : (b); unlike fmax it passes a NaN
// in b through.
__device__ __forceinline__ double cmax(double a, double b) { return a > b ? a : b; }

struct DamageLaw {
    double D0, D1, D2, D3;  // plane-stress constitutive matrix
    double E, ft, gf, r0;
};

// set_plane_stress (formulas.c:48-54) and tension_damage_r0
// (static_damage2D.c:128-132), rounded as nbots rounds them.
__device__ __forceinline__ DamageLaw make_law(double E, double nu, double ft, double gf) {
    DamageLaw m;
    m.D0 = dvd(E, sub(1.0, mul(nu, nu)));
    m.D1 = mul(nu, m.D0);
    m.D2 = m.D0;
    m.D3 = dvd(E, mul(2.0, add(1.0, nu)));
    m.E = E;
    m.ft = ft;
    m.gf = gf;
    m.r0 = dvd(ft, __dsqrt_rn(E));
    return m;
}

// tension_damage (static_damage2D.c:134-182) at one Gauss point.
__device__ __forceinline__ double tension_damage(const DamageLaw& m, double s0, double s1,
                                                 double s2, double r_prev, double& r,
                                                 double clfd) {
    const double es0 = add(mul(m.D0, s0), mul(m.D1, s1));
    const double es1 = add(mul(m.D1, s0), mul(m.D2, s1));
    const double es2 = mul(m.D3, s2);
    const double avg = mul(0.5, add(es0, es1));
    const double d = sub(es0, es1);
    const double R = __dsqrt_rn(add(mul(0.25, mul(d, d)), mul(es2, es2)));
    const double p1 = cmax(0.0, add(avg, R));
    const double p2 = cmax(0.0, sub(avg, R));
    const double det = sub(mul(m.D0, m.D2), mul(m.D1, m.D1));
    const double id11 = dvd(m.D2, det), id12 = dvd(-m.D1, det), id22 = dvd(m.D0, det);
    const double sTs =
        add(add(mul(id11, mul(p1, p1)), mul(mul(mul(2.0, id12), p1), p2)), mul(id22, mul(p2, p2)));
    const double tau = __dsqrt_rn(sTs);
    r = cmax(r_prev, tau);
    const double div = mul(dvd(m.gf, clfd), dvd(m.E, mul(m.ft, m.ft)));
    const double A = dvd(1.0, sub(div, 0.5));
    return sub(1.0, mul(dvd(m.r0, r), exp(mul(A, sub(1.0, dvd(r, m.r0))))));
}

// One thread per element: strain at each Gauss point, then its damage and
// damage threshold r.  A distorted element records its id and leaves its
// points untouched.
template <int NN>
__global__ void __launch_bounds__(128)
    k_strain_damage(uint32_t N_elem, const double* __restrict__ nod,
                    const uint32_t* __restrict__ conn, const double* __restrict__ u, double E,
                    double nu, double ft, double gf, const double* __restrict__ r_prev,
                    double* __restrict__ r, double* __restrict__ dmg, double* __restrict__ strain, uint32_t* distorted) {
    constexpr int NGP = Tab<NN>::NGP;
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= N_elem) return;
    const DamageLaw m = make_law(E, nu, ft, gf);
    double x[NN], y[NN], ux[NN], uy[NN];
#pragma unroll
    for (int i = 0; i < NN; i++) {
        const uint32_t n = conn[(size_t)e * NN + i];
        x[i] = nod[2 * (size_t)n];
        y[i] = nod[2 * (size_t)n + 1];
        ux[i] = u[2 * (size_t)n];
        uy[i] = u[2 * (size_t)n + 1];
    }
    // get_clfd: the first three nodes
    const double clfd = __dsqrt_rn(
        sub(mul(sub(x[1], x[0]), sub(y[2], y[0])), mul(sub(y[1], y[0]), sub(x[2], x[0]))));
#pragma unroll
    for (int gp = 0; gp < NGP; gp++) {
        double dx[NN], dy[NN];
        const double detJ = shape_derivs<NN>(x, y, gp, dx, dy);
        if (detJ < 0) {
            atomicMin(distorted, e);
            return;
        }
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
#pragma unroll
        for (int i = 0; i < NN; i++) {
            s0 = add(s0, mul(dx[i], ux[i]));
            s1 = add(s1, mul(dy[i], uy[i]));
            s2 = add(s2, add(mul(dy[i], ux[i]), mul(dx[i], uy[i])));
        }
        const size_t id = (size_t)e * NGP + gp;
        strain[id * 3] = s0;
        strain[id * 3 + 1] = s1;
        strain[id * 3 + 2] = s2;
        double rn;
        dmg[id] = tension_damage(m, s0, s1, s2, r_prev[id], rn, clfd);
        r[id] = rn;
    }
}

constexpr int kResThreads = 256;

// res = F - K u with nbots' left-to-right row sums (the P of
// nb_sparse_multiply_vector, bit for bit), and per-block sums of res^2.
__global__ void __launch_bounds__(kResThreads)
    k_residual(uint32_t N, const uint32_t* __restrict__ rp, const uint32_t* __restrict__ ci,
               const double* __restrict__ K, const double* __restrict__ F,
               const double* __restrict__ u, double* __restrict__ res, double* __restrict__ part) {
    __shared__ double buf[kResThreads];
    const uint32_t i = blockIdx.x * kResThreads + threadIdx.x;
    double v[1] = {0.0};
    if (i < N) {
        double s = 0.0;
        for (uint32_t k = rp[i]; k < rp[i + 1]; k++) s = add(s, mul(K[k], u[ci[k]]));
        const double ri = sub(F[i], s);
        res[i] = ri;
        v[0] = mul(ri, ri);
    }
    double t[1];
    block_sum_f64<1>(v, buf, t);
    if (threadIdx.x == 0) part[blockIdx.x] = t[0];
}

// One block: out[0] = sum of the per-block partials in a fixed order.
__global__ void __launch_bounds__(kResThreads)
    k_sum_parts(uint32_t n, const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double buf[kResThreads];
    double v[1] = {0.0};
    for (uint32_t k = threadIdx.x; k < n; k += kResThreads) v[0] = add(v[0], part[k]);
    double t[1];
    block_sum_f64<1>(v, buf, t);
    if (threadIdx.x == 0) out[0] = t[0];
}

__global__ void k_add_to(uint32_t N, double* __restrict__ x, const double* __restrict__ dx) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) x[i] = add(x[i], dx[i]);
}

constexpr int kGsThreads = 1024;

struct GsArgs {
    uint32_t N;
    const uint32_t* rp;
    const uint32_t* ci;
    const double* K;
    const double* b;
    double* x;
    double* c;
    double* diag;
    const uint32_t* lev_ptr;
    const uint32_t* lev_rows;
    uint32_t n_levels;
    uint32_t max_iter;
    double tol;
    unsigned long long time_limit_ns;
    nbg_gs_result_t* out;
};

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__global__ void __launch_bounds__(kGsThreads) k_gauss_seidel(GsArgs a) {
    __shared__ double buf[kGsThreads];
    __shared__ double s_err;
    __shared__ int s_stop;
    const uint32_t N = a.N;
    const unsigned long long t0 = gtimer();
    // diagonal of each row (nb_sparse_get(A, i, i): 0 when absent)
    for (uint32_t i = threadIdx.x; i < N; i += kGsThreads) {
        double d = 0.0;
        for (uint32_t k = a.rp[i]; k < a.rp[i + 1]; k++)
            if (a.ci[k] == i) d = a.K[k];
        a.diag[i] = d;
    }
    if (threadIdx.x == 0) {
        s_err = 1e10;
        s_stop = 0;
    }
    const double tol2 = a.tol * a.tol;
    uint32_t k = 0;
    int status = NBG_OK;
    __syncthreads();
    while (k < a.max_iter) {
        // c = b - (strict upper part) x, error = |b - A x|^2
        double v[1] = {0.0};
        for (uint32_t i = threadIdx.x; i < N; i += kGsThreads) {
            double ci_ = a.b[i], ei = a.b[i];
            for (uint32_t q = a.rp[i]; q < a.rp[i + 1]; q++) {
                const uint32_t col = a.ci[q];
                const double t = mul(a.K[q], a.x[col]);
                ei = sub(ei, t);
                if (col > i) ci_ = sub(ci_, t);
            }
            a.c[i] = ci_;
            v[0] = add(v[0], mul(ei, ei));
        }
        double t[1];
        block_sum_f64<1>(v, buf, t);
        if (threadIdx.x == 0) {
            s_err = t[0];
            s_stop = t[0] <= tol2;  // as nbots: a NaN error keeps sweeping
            if (!s_stop && a.time_limit_ns && gtimer() - t0 > a.time_limit_ns) s_stop = 2;
        }
        __syncthreads();
        if (s_stop) {
            if (s_stop == 2) status = NBG_ERR_TIMEOUT;
            break;
        }
        // forward substitution, one level at a time
        for (uint32_t L = 0; L < a.n_levels; L++) {
            const uint32_t l0 = a.lev_ptr[L], l1 = a.lev_ptr[L + 1];
            for (uint32_t j = l0 + threadIdx.x; j < l1; j += kGsThreads) {
                const uint32_t i = a.lev_rows[j];
                double xi = a.c[i];
                for (uint32_t q = a.rp[i]; q < a.rp[i + 1] && a.ci[q] < i; q++)
                    xi = sub(xi, mul(a.K[q], a.x[a.ci[q]]));
                a.x[i] = dvd(xi, a.diag[i]);
            }
            __syncthreads();
        }
        k++;
    }
    if (threadIdx.x == 0) {
        a.out->niter = k;
        a.out->error = __dsqrt_rn(s_err);
        a.out->status = status != NBG_OK ? status : (s_err > tol2 ? 1 : NBG_OK);
    }
}

inline unsigned nblk(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

extern "C" int nbg_strain_damage_f64(uint32_t nen, uint32_t N_elem, const double* nod,
                                     const uint32_t* conn, const double* u, double E, double nu,
                                     double ft, double gf, const double* r_prev, double* r,
                                     double* damage, double* strain, uint32_t* distorted,
                                     void* stream) {
    if (N_elem == 0) return NBG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (nen == 4)
        k_strain_damage<4><<<nblk(N_elem, 128), 128, 0, s>>>(N_elem, nod, conn, u, E, nu, ft, gf,
                                                             r_prev, r,
                                                             damage, strain, distorted);
    else if (nen == 3)
        k_strain_damage<3><<<nblk(N_elem, 128), 128, 0, s>>>(N_elem, nod, conn, u, E, nu, ft, gf,
                                                             r_prev, r,
                                                             damage, strain, distorted);
    else
        return NBG_ERR_ARG;
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}

extern "C" size_t nbg_residual_workspace_bytes(uint32_t N) {
    return 8 * ((size_t)nblk(N ? N : 1, kResThreads) + 1);
}

extern "C" int nbg_residual_f64(uint32_t N, const uint32_t* row_ptr, const uint32_t* col_idx,
                                const double* K, const double* F, const double* u, double* res,
                                double* norm2, void* ws, void* stream) {
    if (N == 0) return NBG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned nb = nblk(N, kResThreads);
    double* part = (double*)ws;
    k_residual<<<nb, kResThreads, 0, s>>>(N, row_ptr, col_idx, K, F, u, res, part);
    NBG_CHECK(cudaGetLastError());
    k_sum_parts<<<1, kResThreads, 0, s>>>(nb, part, norm2);
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}

extern "C" int nbg_add_to_f64(uint32_t N, double* x, const double* dx, void* stream) {
    if (N == 0) return NBG_OK;
    k_add_to<<<nblk(N, 256), 256, 0, (cudaStream_t)stream>>>(N, x, dx);
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}

extern "C" size_t nbg_gauss_seidel_workspace_bytes(uint32_t N) {
    return align256(16 * (size_t)(N ? N : 1)) + 256;
}

extern "C" int nbg_gauss_seidel_f64(uint32_t N, const uint32_t* row_ptr, const uint32_t* col_idx,
                                    const double* K, const double* b, double* x,
                                    const uint32_t* lev_ptr, const uint32_t* lev_rows,
                                    uint32_t n_levels, uint32_t max_iter, double tol,
                                    double time_limit_s, nbg_gs_result_t* result, void* ws,
                                    void* stream) {
    if (!result || !ws) return NBG_ERR_ARG;
    result->niter = 0;
    result->status = NBG_OK;
    result->error = 0.0;
    if (N == 0) return NBG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    char* base = (char*)ws;
    GsArgs a;
    a.N = N;
    a.rp = row_ptr;
    a.ci = col_idx;
    a.K = K;
    a.b = b;
    a.x = x;
    a.c = (double*)base;
    a.diag = (double*)base + N;
    a.out = (nbg_gs_result_t*)(base + align256(16 * (size_t)N));
    a.lev_ptr = lev_ptr;
    a.lev_rows = lev_rows;
    a.n_levels = n_levels;
    a.max_iter = max_iter;
    a.tol = tol;
    a.time_limit_ns = time_limit_s > 0 ? (unsigned long long)(time_limit_s * 1e9) : 0ull;
    k_gauss_seidel<<<1, kGsThreads, 0, s>>>(a);
    NBG_CHECK(cudaGetLastError());
    NBG_CHECK(cudaMemcpyAsync(result, a.out, sizeof(nbg_gs_result_t), cudaMemcpyDeviceToHost, s));
    NBG_CHECK(cudaStreamSynchronize(s));
    return NBG_OK;
}
