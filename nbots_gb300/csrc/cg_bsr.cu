// Fast persistent FP64 (Jacobi-preconditioned) CG on the 2x2-block SELL
// layout (bsr.cu): one cooperative launch per solve, one thread per node
// row, convergence decided on the device, every spin bounded.
//
// GB300 issues FP64 at a small fraction of its FP32 rate, so this kernel
// keeps the FP64 instruction count at one FMA per stored value plus seven
// per dof (q = g / Aii becomes a multiply by the stored reciprocal, and
// dot_gq of the next L1 reuses dot_gkqk of L2), leaves the scalar
// recurrences to thread 0 and the cross-thread sums to warp 0, and uses
// three barriers per iteration, one after each of L1 | L2 | L3 of
// cg_precond_jacobi.c:50-74.
//
// Two stop rules (template LAGGED):
//  * nbots' (cg_precond_jacobi.c:45, 80-89; conjugate_gradient.c:40, 70-76):
//    after iteration k the loop tests ||g_{k-1}||, the norm from before the
//    iteration's update, against an absolute tolerance, so it runs one
//    iteration past the first ||g|| <= tol, and reports that lagged norm.
//    The drop-in nb_sparse_solve_* entries use it; with FMAs and the
//    reciprocal diagonal the iterates differ from nbots' in the last bits
//    only.
//  * the fast rule: stop on the current ||g||, but only after confirming it
//    on the true residual.  When the recurrence says converged, one extra
//    pass recomputes g = A x - b (and q, g.q, g.g) from x; if the true norm
//    is still above the target, g replaces the recurrence's residual and the
//    iteration continues with beta from the true g.q (residual replacement),
//    so the reported norm is always a true FP64 residual.  A target below
//    what FP64 can reach on the system shows either as a second failed check
//    with a true residual not even halved since the first, or as a
//    recurrence that does not meet the target again within twice the
//    iterations its rate so far needs (plus 100): the solve then stops, not
//    converged (status 1), reporting the last true residual, that floor.
// JAC = false is the unpreconditioned CG (q = g).
#include <cstdint>

#include "perm.cuh"
#include "persist.cuh"

using namespace nbg;

namespace {

struct CgBsrArgs {
    nbg_bsr_t A;
    const double* b;
    double* x;
    double *g, *q, *p, *w;
    double* part;  // 6 * kMaxBlocks doubles: L1 [0,K), L2 [K,3K), init and check [3K,6K)
    unsigned* bar;
    int* status;
    double* res;  // niter, status, reported gg, bb, true-residual checks
    uint32_t max_iter;
    double tol;
    unsigned flags;
};

template <bool JAC>
__device__ __forceinline__ double2 precond(double2 g, double2 di) {
    return JAC ? make_double2(g.x * di.x, g.y * di.y) : g;
}

template <bool JAC, bool LAGGED>
__global__ void __launch_bounds__(kPersistThreads, kPersistMinBlocks) k_cg_bsr_f64(CgBsrArgs a) {
    __shared__ double buf[3 * kPersistThreads];
    __shared__ double s_coef;  // alpha, then beta
    __shared__ int s_stop;     // 0 iterate, 1 stop, 2 confirm on the true residual first
    __shared__ struct {
        double gq, gq_old, gg, bb, target2, report, gg_check, gg0, k_limit;
        uint32_t k, checks;
    } sc;  // scalar state, thread 0 only
    const unsigned G = gridDim.x;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nw = kPersistThreads / 32;
    uint32_t s0, s1;
    slice_range(a.A.n_slices, s0, s1);
    const uint32_t Nn = a.A.Nn;
    double2* __restrict__ x = reinterpret_cast<double2*>(a.x);
    double2* __restrict__ g = reinterpret_cast<double2*>(a.g);
    double2* __restrict__ q = reinterpret_cast<double2*>(a.q);
    double2* __restrict__ p = reinterpret_cast<double2*>(a.p);
    double2* __restrict__ w = reinterpret_cast<double2*>(a.w);
    const double2* __restrict__ b = reinterpret_cast<const double2*>(a.b);
    const double2* __restrict__ dinv = reinterpret_cast<const double2*>(a.A.dinv64);
    const double2 one = make_double2(1.0, 1.0);
    double* const part0 = a.part;
    double* const part1 = a.part + kMaxBlocks;
    // own slot: L1 may overwrite [0, G) early; the check runs between the L2
    // barrier and L3, when no block can be writing part0 or part1's readers
    // still need them
    double* const part2 = a.part + 3 * kMaxBlocks;

    if (threadIdx.x == 0) {
        sc.gq = sc.gq_old = sc.gg = sc.bb = sc.target2 = sc.report = sc.gg_check = 0.0;
        sc.gg0 = sc.k_limit = 0.0;
        sc.k = sc.checks = 0;
    }
    {   // init: g = A x - b, q = g / Aii, p = -q
        double v[3] = {0.0, 0.0, 0.0};  // gq, gg, bb
        for (uint32_t s = s0 + warp; s < s1; s += nw) {
            const uint32_t i = s * 32 + lane;
            if (i >= Nn) continue;
            const double2 ax = spmv_row_f64(a.A, s, lane, x);
            const double2 bi = b[i];
            const double2 gi = make_double2(ax.x - bi.x, ax.y - bi.y);
            const double2 qi = precond<JAC>(gi, JAC ? dinv[i] : one);
            g[i] = gi;
            q[i] = qi;
            p[i] = make_double2(-qi.x, -qi.y);
            v[0] = fma(gi.x, qi.x, fma(gi.y, qi.y, v[0]));
            v[1] = fma(gi.x, gi.x, fma(gi.y, gi.y, v[1]));
            v[2] = fma(bi.x, bi.x, fma(bi.y, bi.y, v[2]));
        }
        double t[3];
        block_sum_f64<3>(v, buf, t);
        if (threadIdx.x == 0)
            for (int j = 0; j < 3; j++) part2[blockIdx.x * 3 + j] = t[j];
    }
    if (grid_barrier(a.bar, G, blockIdx.x, a.status)) goto done;
    {
        double t[3];
        group_reduce0<3>(part2, G, t);
        if (threadIdx.x == 0) {
            sc.gq = t[0];
            sc.gg = sc.report = sc.gg0 = t[1];
            sc.bb = t[2];
            sc.target2 = (a.flags & NBG_CG_RELATIVE) ? a.tol * a.tol * sc.bb : a.tol * a.tol;
            s_stop = !(sc.gg > sc.target2) || a.max_iter == 0;
        }
        __syncthreads();
    }
    while (!s_stop) {
        {   // L1: w = A p, p.w
            double v[1] = {0.0};
            for (uint32_t s = s0 + warp; s < s1; s += nw) {
                const uint32_t i = s * 32 + lane;
                if (i >= Nn) continue;
                const double2 wi = spmv_row_f64(a.A, s, lane, p);
                w[i] = wi;
                const double2 pi = p[i];
                v[0] = fma(pi.x, wi.x, fma(pi.y, wi.y, v[0]));
            }
            double t[1];
            block_sum_f64<1>(v, buf, t);
            if (threadIdx.x == 0) part0[blockIdx.x] = t[0];
        }
        if (grid_barrier(a.bar, G, blockIdx.x, a.status)) goto done;
        {
            double pw[1];
            group_reduce0<1>(part0, G, pw);
            if (threadIdx.x == 0) s_coef = sc.gq / pw[0];
            __syncthreads();
        }
        {   // L2: x += alpha p, g += alpha w, q = g / Aii
            const double alpha = s_coef;
            double v[2] = {0.0, 0.0};
            for (uint32_t s = s0 + warp; s < s1; s += nw) {
                const uint32_t i = s * 32 + lane;
                if (i >= Nn) continue;
                const double2 pi = p[i], wi = w[i];
                double2 xi = x[i], gi = g[i];
                xi.x = fma(alpha, pi.x, xi.x);
                xi.y = fma(alpha, pi.y, xi.y);
                gi.x = fma(alpha, wi.x, gi.x);
                gi.y = fma(alpha, wi.y, gi.y);
                const double2 qi = precond<JAC>(gi, JAC ? dinv[i] : one);
                x[i] = xi;
                g[i] = gi;
                q[i] = qi;
                v[0] = fma(gi.x, qi.x, fma(gi.y, qi.y, v[0]));
                v[1] = fma(gi.x, gi.x, fma(gi.y, gi.y, v[1]));
            }
            double t[2];
            block_sum_f64<2>(v, buf, t);
            if (threadIdx.x == 0) {
                part1[blockIdx.x * 2] = t[0];
                part1[blockIdx.x * 2 + 1] = t[1];
            }
        }
        if (grid_barrier(a.bar, G, blockIdx.x, a.status)) goto done;
        {
            double t2[2];
            group_reduce0<2>(part1, G, t2);
            if (threadIdx.x == 0) {
                sc.gq_old = sc.gq;
                sc.gq = t2[0];
                s_coef = t2[0] / sc.gq_old;  // beta
                sc.k++;
                if (LAGGED) {
                    const double lag = sc.gg;  // ||g_{k-1}||^2, as nbots tests it
                    sc.gg = t2[1];
                    sc.report = lag;
                    s_stop = !(lag > sc.target2) || sc.k >= a.max_iter;
                } else {
                    sc.gg = sc.report = t2[1];
                    s_stop = !(sc.gg > sc.target2) ? 2 : (sc.k >= a.max_iter ? 1 : 0);
                    // after a failed check the recurrence gets twice the
                    // iterations its rate so far needs to meet the target
                    // again; when it hovers above it instead, the true
                    // residual of that check is the FP64 floor
                    if (s_stop == 0 && sc.checks > 0 && (double)sc.k > sc.k_limit) {
                        s_stop = 1;
                        sc.report = sc.gg_check;
                    }
                }
            }
            __syncthreads();
        }
        if (!LAGGED && s_stop == 2) {
            // confirm on the true residual: x is complete (written before the
            // L2 barrier) and nobody writes it again before the next L2
            double v[2] = {0.0, 0.0};
            for (uint32_t s = s0 + warp; s < s1; s += nw) {
                const uint32_t i = s * 32 + lane;
                if (i >= Nn) continue;
                const double2 ax = spmv_row_f64(a.A, s, lane, x);
                const double2 bi = b[i];
                const double2 gi = make_double2(ax.x - bi.x, ax.y - bi.y);
                const double2 qi = precond<JAC>(gi, JAC ? dinv[i] : one);
                g[i] = gi;
                q[i] = qi;
                v[0] = fma(gi.x, qi.x, fma(gi.y, qi.y, v[0]));
                v[1] = fma(gi.x, gi.x, fma(gi.y, gi.y, v[1]));
            }
            double t[2];
            block_sum_f64<2>(v, buf, t);
            if (threadIdx.x == 0) {
                part2[blockIdx.x * 2] = t[0];
                part2[blockIdx.x * 2 + 1] = t[1];
            }
            if (grid_barrier(a.bar, G, blockIdx.x, a.status)) goto done;
            double t2[2];
            group_reduce0<2>(part2, G, t2);
            if (threadIdx.x == 0) {
                sc.checks++;
                sc.gq = t2[0];
                sc.gg = sc.report = t2[1];
                s_coef = t2[0] / sc.gq_old;  // beta from the replaced residual
                // the recurrence fell below the target again but the true
                // residual did not follow (not even halved since the last
                // check): it sits at its FP64 floor above the target
                const bool stalled = sc.checks > 1 && !(sc.gg < 0.25 * sc.gg_check);
                sc.gg_check = sc.gg;
                // iterations to go from this residual to the target at the
                // rate of the k so far (from gg0 to the target)
                const double need = (double)sc.k * log(sc.gg / sc.target2) /
                                    log(sc.gg0 / sc.target2);
                sc.k_limit = (double)sc.k + 2.0 * need + 100.0;
                s_stop = !(sc.gg > sc.target2) || stalled || sc.k >= a.max_iter ||
                         sc.checks >= 64;
            }
            __syncthreads();
        }
        if (s_stop) break;
        {   // L3: p = -q + beta p
            const double beta = s_coef;
            for (uint32_t s = s0 + warp; s < s1; s += nw) {
                const uint32_t i = s * 32 + lane;
                if (i >= Nn) continue;
                const double2 qi = q[i], pi = p[i];
                p[i] = make_double2(fma(beta, pi.x, -qi.x), fma(beta, pi.y, -qi.y));
            }
        }
        if (grid_barrier(a.bar, G, blockIdx.x, a.status)) goto done;
    }
done:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.res[0] = (double)sc.k;
        int st = ld_volatile(a.status);
        a.res[1] = st != 0 ? (double)st : (sc.report > sc.target2 ? 1.0 : 0.0);
        a.res[2] = sc.report;
        a.res[3] = sc.bb;
        a.res[4] = (double)sc.checks;
    }
}

size_t cg_bsr_core_bytes(uint32_t N) {
    return 4 * align256((size_t)N * 8) + align256(kMaxBlocks * 3 * 8) * 2 + 3 * 256;
}

// plus the permuted copies of b and x for a layout with a node order
size_t cg_bsr_bytes(uint32_t N) { return cg_bsr_core_bytes(N) + perm_tail_bytes(N); }

}  // namespace

extern "C" size_t nbg_cg_bsr_workspace_bytes(uint32_t N) { return cg_bsr_bytes(N); }

extern "C" int nbg_cg_bsr_f64(const nbg_bsr_t* A, const double* b, double* x, uint32_t max_iter,
                              double tol, unsigned flags, nbg_cg_result_t* result, void* ws,
                              size_t ws_bytes, void* stream) {
    if (!result || !A) return NBG_ERR_ARG;
    *result = nbg_cg_result_t{0, 0, 0.0, 0.0};
    if (A->Nn == 0) return NBG_OK;
    if (!A->b64 || ((flags & NBG_CG_JACOBI) && !A->dinv64)) return NBG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t need = cg_bsr_bytes(A->N);
    void* own = nullptr;
    if (!ws) {
        NBG_CHECK(cudaMalloc(&own, need));
        ws = own;
    } else if (ws_bytes < need) {
        return NBG_ERR_ARG;
    }
    char* base = (char*)ws;
    const size_t v = align256((size_t)A->N * 8);
    CgBsrArgs a;
    a.A = *A;
    a.b = b;
    a.x = x;
    a.g = (double*)(base);
    a.q = (double*)(base + v);
    a.p = (double*)(base + 2 * v);
    a.w = (double*)(base + 3 * v);
    a.part = (double*)(base + 4 * v);
    char* tail = base + 4 * v + 2 * align256(kMaxBlocks * 3 * 8);
    a.bar = (unsigned*)tail;
    a.status = (int*)(tail + 256);
    a.res = (double*)(tail + 512);
    a.max_iter = max_iter;
    a.tol = tol;
    a.flags = flags;
    int rc = NBG_OK;
    unsigned G = 1;
    double hr[5] = {0, 0, 0, 0, 0};
    cudaError_t e = cudaMemsetAsync(tail, 0, 3 * 256, s);
    if (A->perm) {  // solve in the layout's node order
        double* bp = (double*)(base + cg_bsr_core_bytes(A->N));
        double* xp = bp + align256((size_t)A->N * 8) / 8;
        if (e == cudaSuccess) e = perm_gather(A->Nn, A->perm, b, bp, s);
        if (e == cudaSuccess) e = perm_gather(A->Nn, A->perm, (const double*)x, xp, s);
        a.b = bp;
        a.x = xp;
    }
    const bool jac = (flags & NBG_CG_JACOBI) != 0, lagged = (flags & NBG_CG_NBOTS_STOP) != 0;
    const void* fn = jac ? (lagged ? (const void*)k_cg_bsr_f64<true, true>
                                   : (const void*)k_cg_bsr_f64<true, false>)
                         : (lagged ? (const void*)k_cg_bsr_f64<false, true>
                                   : (const void*)k_cg_bsr_f64<false, false>);
    if (e == cudaSuccess) rc = coop_grid(fn, A->n_slices, &G);
    if (e == cudaSuccess && rc == NBG_OK) {
        void* args[] = {&a};
        e = cudaLaunchCooperativeKernel(fn, dim3(G), dim3(kPersistThreads), args, 0, s);
        if (e == cudaSuccess && A->perm) e = perm_scatter(A->Nn, A->perm, (const double*)a.x, x, s);
    }
    if (e == cudaSuccess && rc == NBG_OK)
        e = cudaMemcpyAsync(hr, a.res, sizeof(hr), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && rc == NBG_OK) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = nbg_cuda_error(e);
    if (rc == NBG_OK) {
        result->niter = (uint32_t)hr[0];
        result->status = (int)hr[1];
        result->tol_reached = sqrt(hr[2]);
        result->bnorm = sqrt(hr[3]);
        rc = result->status;
    }
    if (own) cudaFree(own);
    return rc;
}
