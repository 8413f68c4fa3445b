// Persistent FP64 (Jacobi-preconditioned) CG: one cooperative launch runs
// the whole solve with device-side convergence checks.
//
// Iteration (nbots' cg_precond_jacobi.c:45-76), three grid barriers:
//   L1: w = A p; dot_pw, dot_gg (old g), dot_gq
//   L2: alpha = gq/pw; x += alpha p; g += alpha w; q = g / Aii; dot_gkqk
//   L3: beta = gkqk/gq; p = -q + beta p
// Per-row work repeats nbots' arithmetic (rounded products, left-to-right
// row sums, division by the diagonal).  GB300 issues FP64 at about two
// operations per SM per clock, so the SpMV's two FP64 operations per nonzero
// bound the iteration: folding L3 into the next SpMV (recomputing -q + beta p
// for every gathered column) saves a barrier but costs five per nonzero; on
// the 1M-dof cantilever the folded form took 1.58 s for 7,017 iterations,
// this one 1.11 s.  The SpMV of L1 is warp-staged (warp_rows_exact): a warp
// loads the values and columns of 32 rows with coalesced loads, gathers p for
// all their products at once, then each lane adds its own row's products in
// nbots' order; with one row per thread this took the 16,770-dof cantilever
// from 43 to 21 us per iteration (a thread walking its row alone waits on
// each dependent column load in turn).  It is used up to two rows per thread
// of the grid; on the 1M-dof cantilever (14 rows per thread) it took 230 us
// per iteration against 158 for the plain thread-per-row loop, which keeps
// the FP64 pipe fed from many independent rows.  The scalar recurrences run in thread
// 0; the dot products are summed by warp 0 in a fixed order, identical from
// run to run.
#include <cstdint>
#include <cstdio>

#include "persist.cuh"

using namespace nbg;

namespace {

constexpr int kThreads = 256;
constexpr int kStage = 576;  // products staged per warp and pass: 32 rows of 18

struct CgDevResult {
    uint32_t niter;
    int status;
    double dot_gg;
    double bb;
};

struct CgArgs {
    uint32_t N;
    const uint32_t* rp;
    const uint32_t* ci;
    const double* val;
    const double* b;
    double* x;
    double* g;
    double* q;
    double* P0;
    double* P1;
    double* w;
    double* Aii;
    double* partA;  // 3 per block
    double* partB;  // 1 per block
    double* partC;  // 2 per block
    unsigned* bar;
    int* status;
    CgDevResult* res;
    uint32_t max_iter;
    double tol;
    unsigned flags;
};

template <bool JAC, bool STAGED>
__global__ void __launch_bounds__(kThreads) k_cg_f64(CgArgs a) {
    __shared__ double buf[3 * kThreads];
    __shared__ double prod[STAGED ? kThreads / 32 : 1][STAGED ? kStage : 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ double s_coef;  // alpha, then beta
    __shared__ int s_stop;
    __shared__ struct {
        double gg, bb, gq, tol2;
        uint32_t k;
    } sc;  // scalar state, thread 0 only
    const unsigned G = gridDim.x;
    const uint32_t per = (a.N + G - 1) / G;
    const uint32_t r0 = min(blockIdx.x * per, a.N), r1 = min(r0 + per, a.N);
    const uint32_t* __restrict__ rp = a.rp;
    const uint32_t* __restrict__ ci = a.ci;
    const double* __restrict__ val = a.val;
    double* __restrict__ p = a.P0;
    if (threadIdx.x == 0) {
        sc.gg = sc.bb = sc.gq = sc.tol2 = 0.0;
        sc.k = 0;
    }

    // init (cg_precond_jacobi.c:33-43)
    {
        double v[2] = {0.0, 0.0};
        for (uint32_t r = r0 + threadIdx.x; r < r1; r += kThreads) {
            double sum = 0.0, d = 0.0;
            for (uint32_t k = rp[r]; k < rp[r + 1]; k++) {
                const uint32_t c = ci[k];
                sum = add(sum, mul(val[k], a.x[c]));
                if (c == r) d = val[k];
            }
            const double gi = sub(sum, a.b[r]);
            const double qi = JAC ? dvd(gi, d) : gi;
            a.g[r] = gi;
            a.Aii[r] = d;
            a.q[r] = qi;
            p[r] = -qi;
            v[0] = add(v[0], mul(gi, gi));
            v[1] = add(v[1], mul(a.b[r], a.b[r]));
        }
        double t[2];
        block_sum_f64<2>(v, buf, t);
        if (threadIdx.x == 0) {
            a.partC[blockIdx.x * 2] = t[0];
            a.partC[blockIdx.x * 2 + 1] = t[1];
        }
    }
    if (grid_barrier(a.bar, G, blockIdx.x, a.status)) goto done;
    {
        double t[2];
        group_reduce0<2>(a.partC, G, t);
        if (threadIdx.x == 0) {
            sc.gg = t[0];
            sc.bb = t[1];
            const double tolb = (a.flags & NBG_CG_RELATIVE) ? a.tol * sqrt(sc.bb) : a.tol;
            sc.tol2 = tolb * tolb;
            s_stop = !(sc.gg > sc.tol2) || a.max_iter == 0;
        }
        __syncthreads();
    }
    while (!s_stop) {
        {   // L1: w = A p; p.w, g.g (the lagged norm nbots tests), g.q
            double v3[3] = {0.0, 0.0, 0.0};
            if constexpr (STAGED) {
                for (uint32_t g0 = r0 + warp * 32; g0 < r1; g0 += kThreads) {
                    const uint32_t nrows = min(32u, r1 - g0);
                    const double s = warp_rows_exact<kStage>(rp, ci, val, p, g0, nrows,
                                                             prod[warp], lane);
                    if ((uint32_t)lane < nrows) {
                        const uint32_t r = g0 + lane;
                        a.w[r] = s;
                        const double gi = a.g[r], qi = a.q[r];
                        v3[0] = add(v3[0], mul(p[r], s));
                        v3[1] = add(v3[1], mul(gi, gi));
                        v3[2] = add(v3[2], mul(gi, qi));
                    }
                }
            } else {
                for (uint32_t r = r0 + threadIdx.x; r < r1; r += kThreads) {
                    // four columns, values and gathers in flight, then the
                    // four ordered adds
                    const uint32_t ke = rp[r + 1];
                    uint32_t kk = rp[r];
                    double s = 0.0;
                    for (; kk + 4 <= ke; kk += 4) {
                        const uint32_t c0 = ci[kk], c1 = ci[kk + 1], c2 = ci[kk + 2],
                                       c3 = ci[kk + 3];
                        const double v0 = val[kk], v1 = val[kk + 1], v2 = val[kk + 2],
                                     v3 = val[kk + 3];
                        const double x0 = p[c0], x1 = p[c1], x2 = p[c2], x3 = p[c3];
                        s = add(s, mul(v0, x0));
                        s = add(s, mul(v1, x1));
                        s = add(s, mul(v2, x2));
                        s = add(s, mul(v3, x3));
                    }
                    for (; kk < ke; kk++) s = add(s, mul(val[kk], p[ci[kk]]));
                    a.w[r] = s;
                    const double gi = a.g[r], qi = a.q[r];
                    v3[0] = add(v3[0], mul(p[r], s));
                    v3[1] = add(v3[1], mul(gi, gi));
                    v3[2] = add(v3[2], mul(gi, qi));
                }
            }
            double t[3];
            block_sum_f64<3>(v3, buf, t);
            if (threadIdx.x == 0)
                for (int j = 0; j < 3; j++) a.partA[blockIdx.x * 3 + j] = t[j];
        }
        if (grid_barrier(a.bar, G, blockIdx.x, a.status)) goto done;
        {
            double t3[3];
            group_reduce0<3>(a.partA, G, t3);
            if (threadIdx.x == 0) {
                sc.gg = t3[1];
                sc.gq = t3[2];
                s_coef = dvd(t3[2], t3[0]);  // alpha = gq / pw
            }
            __syncthreads();
        }
        {   // L2: x += alpha p; g += alpha w; q = g / Aii; g.q
            const double alpha = s_coef;
            double v1[1] = {0.0};
            for (uint32_t r = r0 + threadIdx.x; r < r1; r += kThreads) {
                a.x[r] = add(a.x[r], mul(alpha, p[r]));
                const double gi = add(a.g[r], mul(alpha, a.w[r]));
                a.g[r] = gi;
                const double qi = JAC ? dvd(gi, a.Aii[r]) : gi;
                a.q[r] = qi;
                v1[0] = add(v1[0], mul(gi, qi));
            }
            double t[1];
            block_sum_f64<1>(v1, buf, t);
            if (threadIdx.x == 0) a.partB[blockIdx.x] = t[0];
        }
        if (grid_barrier(a.bar, G, blockIdx.x, a.status)) goto done;
        {
            double t1[1];
            group_reduce0<1>(a.partB, G, t1);
            if (threadIdx.x == 0) {
                s_coef = dvd(t1[0], sc.gq);  // beta
                sc.k++;
                s_stop = !(sc.gg > sc.tol2) || sc.k >= a.max_iter;
            }
            __syncthreads();
        }
        if (s_stop) break;
        {   // L3: p = -q + beta p
            const double beta = s_coef;
            for (uint32_t r = r0 + threadIdx.x; r < r1; r += kThreads)
                p[r] = add(-a.q[r], mul(beta, p[r]));
        }
        if (grid_barrier(a.bar, G, blockIdx.x, a.status)) goto done;
    }
done:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.res->niter = sc.k;
        a.res->dot_gg = sc.gg;
        a.res->bb = sc.bb;
        int st = ld_volatile(a.status);
        a.res->status = st != 0 ? st : (sc.gg > sc.tol2 ? NBG_NOT_CONVERGED : NBG_OK);
    }
}

struct Layout {
    size_t g, q, P0, P1, w, Aii, partA, partB, partC, bar, status, res, total;
};

Layout layout(uint32_t N) {
    Layout L;
    size_t o = 0;
    const size_t v = align256((size_t)N * 8);
    L.g = o; o += v;
    L.q = o; o += v;
    L.P0 = o; o += v;
    L.P1 = o; o += v;
    L.w = o; o += v;
    L.Aii = o; o += v;
    L.partA = o; o += align256(kMaxBlocks * 3 * 8);
    L.partB = o; o += align256(kMaxBlocks * 8);
    L.partC = o; o += align256(kMaxBlocks * 2 * 8);
    L.bar = o; o += 256;
    L.status = o; o += 256;
    L.res = o; o += 256;
    L.total = o;
    return L;
}

}  // namespace

extern "C" size_t nbg_cg_workspace_bytes(uint32_t N) { return layout(N).total; }

extern "C" int nbg_cg_f64(uint32_t N, const uint32_t* row_ptr, const uint32_t* col_idx,
                          const double* val, const double* b, double* x, uint32_t max_iter,
                          double tol, unsigned flags, nbg_cg_result_t* result, void* ws,
                          size_t ws_bytes, void* stream) {
    if (!result) return NBG_ERR_ARG;
    result->niter = 0;
    result->status = NBG_OK;
    result->tol_reached = 0.0;
    result->bnorm = 0.0;
    if (N == 0) return NBG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const Layout L = layout(N);
    void* own = nullptr;
    if (ws == nullptr) {
        NBG_CHECK(cudaMalloc(&own, L.total));
        ws = own;
    } else if (ws_bytes < L.total) {
        return NBG_ERR_ARG;
    }
    char* base = (char*)ws;
    CgArgs a;
    a.N = N;
    a.rp = row_ptr;
    a.ci = col_idx;
    a.val = val;
    a.b = b;
    a.x = x;
    a.g = (double*)(base + L.g);
    a.q = (double*)(base + L.q);
    a.P0 = (double*)(base + L.P0);
    a.P1 = (double*)(base + L.P1);
    a.w = (double*)(base + L.w);
    a.Aii = (double*)(base + L.Aii);
    a.partA = (double*)(base + L.partA);
    a.partB = (double*)(base + L.partB);
    a.partC = (double*)(base + L.partC);
    a.bar = (unsigned*)(base + L.bar);
    a.status = (int*)(base + L.status);
    a.res = (CgDevResult*)(base + L.res);
    a.max_iter = max_iter;
    a.tol = tol;
    a.flags = flags;

    int rc = NBG_OK;
    cudaError_t e = cudaMemsetAsync(base + L.bar, 0, 3 * 256, s);
    int dev = 0, nsm = 0, occ = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    // at most two rows per thread of the grid: warp-staged SpMV (latency);
    // more: one row per thread, the FP64 pipe busy with many rows in flight
    const bool staged = (uint64_t)N <= 2ull * 2 * (uint64_t)nsm * kThreads;
    const bool jac = (flags & NBG_CG_JACOBI) != 0;
    const void* fn = jac ? (staged ? (const void*)k_cg_f64<true, true>
                                   : (const void*)k_cg_f64<true, false>)
                         : (staged ? (const void*)k_cg_f64<false, true>
                                   : (const void*)k_cg_f64<false, false>);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kThreads, 0);
    CgDevResult hr{};
    if (e == cudaSuccess) {
        unsigned G = (unsigned)(nsm * (occ < 2 ? occ : 2));
        const unsigned want = staged ? (N + kThreads - 1) / kThreads
                                     : (N + kThreads * 4 - 1) / (kThreads * 4);
        if (want < G) G = want;
        if (G < 1) G = 1;
        if (G > kMaxBlocks) G = kMaxBlocks;
        void* args[] = {&a};
        e = cudaLaunchCooperativeKernel(fn, dim3(G), dim3(kThreads), args, 0, s);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hr, a.res, sizeof(hr), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        rc = nbg_cuda_error(e);
    } else {
        result->niter = hr.niter;
        result->status = hr.status;
        result->tol_reached = sqrt(hr.dot_gg);
        result->bnorm = sqrt(hr.bb);
        rc = hr.status;
    }
    if (own) cudaFree(own);
    return rc;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of nbg_cg_f64.
//
// Some callers cannot allocate device memory when they solve: a host
// application that reserves the GPU's memory in its own pool and forbids
// libraries to call cudaMalloc, or a loop that cannot take the device-wide
// synchronisation cudaMalloc / cudaFree imply.  This entry point runs the
// same kernel with its scratch (work vectors, partial sums, barrier and
// status words) in a file-scope device array instead of a workspace.
//
// Limits and sharing:
//  * the array holds kNoAllocScratchBytes (16 MiB) on every GPU that loads
//    this library, until the process exits; a system fits when
//    nbg_cg_workspace_bytes(N) is at most that, i.e. N <= 345,408 dofs;
//    larger N is rejected with NBG_ERR_ARG and a message in nbg_last_error;
//  * in host code g_cg_scratch names a host-side shadow, not device memory,
//    so every call looks up the array's device address on the current
//    device (cudaGetSymbolAddress, which allocates nothing) and passes that
//    to the kernel.  Looking it up per call rather than once per device keeps
//    the address right after the host application resets the device
//    (cudaDeviceReset), which gives the array a new address.  The first call
//    on a device also loads this library's kernels there; make it before any
//    stream capture;
//  * every call shares the array and it keeps the last call's contents: each
//    call clears the barrier, status and result words it needs at zero, and
//    the work vectors are written before they are read;
//  * calls that overlap on the GPU (two streams, or two host threads on one
//    device) race on the array and must be serialised by the caller.
namespace {
constexpr size_t kNoAllocScratchBytes = 16u << 20;
static __device__ __align__(256) unsigned char g_cg_scratch[kNoAllocScratchBytes];
}  // namespace

extern "C" int nbg_cg_f64_noalloc(uint32_t N, const uint32_t* row_ptr, const uint32_t* col_idx,
                                  const double* val, const double* b, double* x,
                                  uint32_t max_iter, double tol, unsigned flags,
                                  nbg_cg_result_t* result, void* stream) {
    const size_t need = layout(N).total;
    if (need > kNoAllocScratchBytes) {
        char msg[200];
        std::snprintf(msg, sizeof(msg),
                      "nbg_cg_f64_noalloc: N = %u needs %zu bytes of scratch; the static "
                      "array holds %zu (N <= 345408)",
                      N, need, kNoAllocScratchBytes);
        return nbg_error_text(NBG_ERR_ARG, msg);
    }
    void* ptr = nullptr;
    NBG_CHECK(cudaGetSymbolAddress(&ptr, g_cg_scratch));
    if (ptr == nullptr) return nbg_error_text(NBG_ERR_CUDA, "nbg_cg_f64_noalloc: no address");
    return nbg_cg_f64(N, row_ptr, col_idx, val, b, x, max_iter, tol, flags, result, ptr,
                      kNoAllocScratchBytes, stream);
}
