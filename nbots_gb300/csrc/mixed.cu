// Mixed-precision Jacobi-PCG with reliable updates, one cooperative launch.
//
// GB300 runs FP32 at many times its FP64 rate, and the stiffness matrices
// here have condition numbers near 1e8, where plain FP32 CG needs several
// times more iterations than FP64.  Measured on the lognormal cantilever
// (1M dof), the inflation comes from three places: the precision of the
// matrix values (even 32 significant bits cost 1.33x the iterations: the
// inner operator must match the FP64 one behind the residual), FP32 search
// directions p and FP32 products A p, and an FP32 correction x.  The FP32
// residual r is harmless.  So the inner iteration runs on the FP32 pipes
// with:
//   matrix      FP32 hi + a 16-bit remainder in units of 2^-16 ulp(hi)
//               (about 40 significant bits in 6 B/value instead of 8),
//   p, A p      FP32 hi + bfloat16 lo per dof,
//   x           float-float (FP32 hi + FP32 lo),
//   r           FP32,
// products and sums by error-free transformations (TwoProduct with FMA,
// TwoSum), dot products with compensated FP32 sums per thread and FP64
// across threads.  A reliable update (Sleijpen & van der Vorst 1996) adds x
// to the FP64 solution and recomputes r = b - A u in FP64 with the FP64
// values whenever |r| has fallen by `delta` since the last one; p is kept,
// so the Krylov progress survives.  Convergence is judged on the FP64
// residual only.  Three grid barriers per iteration (L1 | L2 | L3 of
// cg_precond_jacobi.c:50-74): folding L3 into the next SpMV (each block
// rebuilding z + beta p for the columns it reads) measured slower, 77 vs
// 66 us per iteration at 1M dof, because the float-float rebuild per column
// costs more issue slots and gather bytes than the barrier it saves.
#include <cstdint>

#include "persist.cuh"

using namespace nbg;

// Keep each block's own-row vectors in shared memory when they fit
// (overridable at build time for tuning).
#ifndef NBG_MIXED_RESIDENT
#define NBG_MIXED_RESIDENT 1
#endif

namespace {

struct MixArgs {
    nbg_bsr_t A;
    const double* b;
    double* u;
    float* ph;               // search direction, global (gathered by neighbours)
    __nv_bfloat16* pl;
    float *r, *wh, *xh, *xl;  // own-row vectors when they do not fit in shared memory
    __nv_bfloat16* wl;
    double* part;  // L1 [0,K), L2 [K,3K), init/update [3K,6K)
    unsigned* bar;
    int* status;
    double* res;  // niter, updates, status, rr64, bb
    uint32_t max_iter;
    double tol, delta;
    unsigned flags;
    int resident;  // own-row vectors live in shared memory
};

__device__ __forceinline__ float bf_round(float x) {
    return __bfloat162float(__float2bfloat16_rn(x));
}

// w = A p for node row (s, lane), split-precision operands, float-float sum
__device__ __forceinline__ void spmv_row_split(const MixArgs& a, uint32_t s, uint32_t lane,
                                               FF& y0, FF& y1) {
    const float4* __restrict__ bh = reinterpret_cast<const float4*>(a.A.b32);
    const uint2* __restrict__ bl = reinterpret_cast<const uint2*>(a.A.blo);
    const float2* __restrict__ ph = reinterpret_cast<const float2*>(a.ph);
    const __nv_bfloat162* __restrict__ pl = reinterpret_cast<const __nv_bfloat162*>(a.pl);
    FFAcc c0{0.f, 0.f}, c1{0.f, 0.f};
    const uint32_t k0 = a.A.slice_off[s], k1 = a.A.slice_off[s + 1];
#pragma unroll 3
    for (uint32_t k = k0; k < k1; k++) {
        const size_t e = (size_t)k * 32 + lane;
        const uint32_t c = a.A.bcol[e];
        const float4 m = bh[e];
        const float4 ml = ulp16_decode4(bl[e], m);
        const float2 pc = ph[c];
        const float2 pcl = __bfloat1622float2(pl[c]);
        c0.fma2(m.x, ml.x, pc.x, pcl.x);
        c0.fma2(m.y, ml.y, pc.y, pcl.y);
        c1.fma2(m.z, ml.z, pc.x, pcl.x);
        c1.fma2(m.w, ml.w, pc.y, pcl.y);
    }
    y0 = c0.result();
    y1 = c1.result();
}

// Own-row vectors of this block, indexed by local node row
// (i - 32 * s0): shared memory when they fit, else the global workspace.
struct Own {
    float2 *xh, *xl, *r, *dv, *wh, *ph;
    __nv_bfloat162 *wl, *pl;
};

__device__ __forceinline__ size_t own_smem_bytes(uint32_t nrows) { return (size_t)nrows * 56; }

__device__ __forceinline__ Own own_vectors(const MixArgs& a, unsigned char* smem, uint32_t s0,
                                           uint32_t nrows) {
    Own o;
    const size_t base = (size_t)s0 * 32;
    if (a.resident) {
        float2* f = reinterpret_cast<float2*>(smem);
        o.xh = f;
        o.xl = f + nrows;
        o.r = f + 2 * nrows;
        o.dv = f + 3 * nrows;
        o.wh = f + 4 * nrows;
        o.ph = f + 5 * nrows;
        __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(f + 6 * nrows);
        o.wl = h;
        o.pl = h + nrows;
    } else {
        o.xh = reinterpret_cast<float2*>(a.xh) + base;
        o.xl = reinterpret_cast<float2*>(a.xl) + base;
        o.r = reinterpret_cast<float2*>(a.r) + base;
        o.dv = const_cast<float2*>(reinterpret_cast<const float2*>(a.A.dinv32)) + base;
        o.wh = reinterpret_cast<float2*>(a.wh) + base;
        o.ph = reinterpret_cast<float2*>(a.ph) + base;
        o.wl = reinterpret_cast<__nv_bfloat162*>(a.wl) + base;
        o.pl = reinterpret_cast<__nv_bfloat162*>(a.pl) + base;
    }
    return o;
}

// r = b - A u in FP64 for the own rows, stored as FP32; z = r / Aii
// (float-float); accumulates |r|^2 (FP64), r.z and optionally |b|^2; with
// set_p, p = z (own copy and the global one).
__device__ __forceinline__ void true_residual(const MixArgs& a, const Own& o, uint32_t s0,
                                              uint32_t s1, double& rr, FFAcc& rz, double* bb,
                                              bool set_p) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nw = kPersistThreads / 32;
    const double2* __restrict__ u = reinterpret_cast<const double2*>(a.u);
    const double2* __restrict__ b = reinterpret_cast<const double2*>(a.b);
    for (uint32_t s = s0 + warp; s < s1; s += nw) {
        const uint32_t i = s * 32 + lane, li = i - s0 * 32;
        if (i >= a.A.Nn) continue;
        const double2 au = spmv_row_f64(a.A, s, lane, u);
        const double2 bi = b[i];
        const double r0 = bi.x - au.x, r1 = bi.y - au.y;
        rr = fma(r0, r0, fma(r1, r1, rr));
        if (bb) *bb = fma(bi.x, bi.x, fma(bi.y, bi.y, *bb));
        const float f0 = (float)r0, f1 = (float)r1;
        o.r[li] = make_float2(f0, f1);
        const float2 di = o.dv[li];
        const FF z0 = two_prod(f0, di.x), z1 = two_prod(f1, di.y);
        rz.fma2(f0, 0.f, z0.hi, z0.lo);
        rz.fma2(f1, 0.f, z1.hi, z1.lo);
        if (set_p) {
            const float2 hi = make_float2(z0.hi, z1.hi);
            const __nv_bfloat162 lo = __floats2bfloat162_rn(z0.lo, z1.lo);
            o.ph[li] = hi;
            o.pl[li] = lo;
            reinterpret_cast<float2*>(a.ph)[i] = hi;
            reinterpret_cast<__nv_bfloat162*>(a.pl)[i] = lo;
        }
    }
}

__global__ void __launch_bounds__(kPersistThreads, kPersistMinBlocks) k_cg_mixed(MixArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double red[3 * 32];
    __shared__ double bc[3];
    const unsigned G = gridDim.x;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nw = kPersistThreads / 32;
    uint32_t s0, s1;
    slice_range(a.A.n_slices, s0, s1);
    const uint32_t Nn = a.A.Nn;
    const Own o = own_vectors(a, smem, s0, (s1 - s0) * 32);
    float2* __restrict__ gph = reinterpret_cast<float2*>(a.ph);
    __nv_bfloat162* __restrict__ gpl = reinterpret_cast<__nv_bfloat162*>(a.pl);
    double* const part0 = a.part;
    double* const part1 = a.part + kMaxBlocks;
    double* const part2 = a.part + 3 * kMaxBlocks;

    uint32_t k = 0, nupd = 0;
    double rr64 = 0.0, bb = 0.0, target2 = 0.0, rz = 0.0, rr = 0.0, rmax2 = 0.0;
    int converged = 0;
    {   // init: own copy of 1/Aii, x = 0, r = b - A u (FP64), p = z
        const float2* __restrict__ gdv = reinterpret_cast<const float2*>(a.A.dinv32);
        for (uint32_t s = s0 + warp; s < s1; s += nw) {
            const uint32_t i = s * 32 + lane, li = i - s0 * 32;
            if (i >= Nn) continue;
            if (a.resident) o.dv[li] = gdv[i];
            o.xh[li] = make_float2(0.f, 0.f);
            o.xl[li] = make_float2(0.f, 0.f);
        }
        __syncwarp();
        double rrl = 0.0, bbl = 0.0;
        FFAcc rzk{0.f, 0.f};
        true_residual(a, o, s0, s1, rrl, rzk, &bbl, true);
        const FF t = rzk.result();
        double v[3] = {rrl, bbl, (double)t.hi + (double)t.lo};
        publish<3>(v, red, part2);
    }
    if (grid_barrier(a.bar, G, a.status)) goto done;
    {
        double t[3];
        grid_reduce<3>(part2, t, bc);
        rr64 = t[0];
        bb = t[1];
        rz = t[2];
    }
    target2 = (a.flags & NBG_CG_RELATIVE) ? a.tol * a.tol * bb : a.tol * a.tol;
    rr = rmax2 = rr64;
    converged = !(rr64 > target2);
    {
        const double d2 = a.delta * a.delta;
        while (!converged && k < a.max_iter) {
            {   // L1: w = A p, p.w
                FFAcc pw{0.f, 0.f};
                for (uint32_t s = s0 + warp; s < s1; s += nw) {
                    const uint32_t i = s * 32 + lane, li = i - s0 * 32;
                    if (i >= Nn) continue;
                    FF y0, y1;
                    spmv_row_split(a, s, lane, y0, y1);
                    const float l0 = bf_round(y0.lo), l1 = bf_round(y1.lo);
                    o.wh[li] = make_float2(y0.hi, y1.hi);
                    o.wl[li] = __floats2bfloat162_rn(l0, l1);
                    const float2 p = o.ph[li];
                    const float2 plo = __bfloat1622float2(o.pl[li]);
                    pw.fma2(p.x, plo.x, y0.hi, l0);
                    pw.fma2(p.y, plo.y, y1.hi, l1);
                }
                const FF t = pw.result();
                double v[1] = {(double)t.hi + (double)t.lo};
                publish<1>(v, red, part0);
            }
            if (grid_barrier(a.bar, G, a.status)) goto done;
            double pwd;
            grid_reduce<1>(part0, &pwd, bc);
            const FF alpha = ff_from_double(rz / pwd);
            {   // L2: x += alpha p, r -= alpha w, z = r / Aii (own rows only)
                FFAcc rzk{0.f, 0.f}, rrk{0.f, 0.f};
                for (uint32_t s = s0 + warp; s < s1; s += nw) {
                    const uint32_t i = s * 32 + lane, li = i - s0 * 32;
                    if (i >= Nn) continue;
                    const float2 p = o.ph[li], plo = __bfloat1622float2(o.pl[li]);
                    const float2 w = o.wh[li], wlo = __bfloat1622float2(o.wl[li]);
                    const float2 xhi = o.xh[li], xlo = o.xl[li];
                    const float2 ri = o.r[li], di = o.dv[li];
                    const FF x0 = ff_add({xhi.x, xlo.x}, ff_mul(alpha, {p.x, plo.x}));
                    const FF x1 = ff_add({xhi.y, xlo.y}, ff_mul(alpha, {p.y, plo.y}));
                    o.xh[li] = make_float2(x0.hi, x1.hi);
                    o.xl[li] = make_float2(x0.lo, x1.lo);
                    const FF aw0 = ff_mul(alpha, {w.x, wlo.x}), aw1 = ff_mul(alpha, {w.y, wlo.y});
                    const FF t0 = two_sum(ri.x, -aw0.hi), t1 = two_sum(ri.y, -aw1.hi);
                    const float r0 = __fadd_rn(t0.hi, __fsub_rn(t0.lo, aw0.lo));
                    const float r1 = __fadd_rn(t1.hi, __fsub_rn(t1.lo, aw1.lo));
                    o.r[li] = make_float2(r0, r1);
                    const FF z0 = two_prod(r0, di.x), z1 = two_prod(r1, di.y);
                    rzk.fma2(r0, 0.f, z0.hi, z0.lo);
                    rzk.fma2(r1, 0.f, z1.hi, z1.lo);
                    rrk.fma2(r0, 0.f, r0, 0.f);
                    rrk.fma2(r1, 0.f, r1, 0.f);
                }
                const FF t1 = rzk.result(), t2 = rrk.result();
                double v[2] = {(double)t1.hi + (double)t1.lo, (double)t2.hi + (double)t2.lo};
                publish<2>(v, red, part1);
            }
            if (grid_barrier(a.bar, G, a.status)) goto done;
            double t2[2];
            grid_reduce<2>(part1, t2, bc);
            double rz_new = t2[0];
            rr = t2[1];
            if (rr > rmax2) rmax2 = rr;
            k++;
            if (rr <= d2 * rmax2 || rr <= target2 || k >= a.max_iter) {
                // reliable update: u += x in FP64, then r = b - A u in FP64
                double2* __restrict__ u = reinterpret_cast<double2*>(a.u);
                for (uint32_t s = s0 + warp; s < s1; s += nw) {
                    const uint32_t i = s * 32 + lane, li = i - s0 * 32;
                    if (i >= Nn) continue;
                    const float2 xhi = o.xh[li], xlo = o.xl[li];
                    double2 ui = u[i];
                    ui.x += (double)xhi.x + (double)xlo.x;
                    ui.y += (double)xhi.y + (double)xlo.y;
                    u[i] = ui;
                    o.xh[li] = make_float2(0.f, 0.f);
                    o.xl[li] = make_float2(0.f, 0.f);
                }
                if (grid_barrier(a.bar, G, a.status)) goto done;
                double rrl = 0.0;
                FFAcc rzk{0.f, 0.f};
                true_residual(a, o, s0, s1, rrl, rzk, nullptr, false);
                const FF t = rzk.result();
                double v[2] = {rrl, (double)t.hi + (double)t.lo};
                publish<2>(v, red, part2);
                if (grid_barrier(a.bar, G, a.status)) goto done;
                double tt[2];
                grid_reduce<2>(part2, tt, bc);
                rr64 = tt[0];
                rz_new = tt[1];
                rr = rmax2 = rr64;
                nupd++;
                converged = !(rr64 > target2);
                if (converged || k >= a.max_iter) break;
            }
            const FF beta = ff_from_double(rz_new / rz);
            rz = rz_new;
            // L3: p = z + beta p (own copy and the global one)
            for (uint32_t s = s0 + warp; s < s1; s += nw) {
                const uint32_t i = s * 32 + lane, li = i - s0 * 32;
                if (i >= Nn) continue;
                const float2 ri = o.r[li], di = o.dv[li];
                const float2 p = o.ph[li], plo = __bfloat1622float2(o.pl[li]);
                const FF n0 = ff_add(two_prod(ri.x, di.x), ff_mul(beta, {p.x, plo.x}));
                const FF n1 = ff_add(two_prod(ri.y, di.y), ff_mul(beta, {p.y, plo.y}));
                const float2 hi = make_float2(n0.hi, n1.hi);
                const __nv_bfloat162 lo = __floats2bfloat162_rn(n0.lo, n1.lo);
                if (a.resident) {
                    o.ph[li] = hi;
                    o.pl[li] = lo;
                }
                gph[i] = hi;
                gpl[i] = lo;
            }
            if (grid_barrier(a.bar, G, a.status)) goto done;
        }
    }
done:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.res[0] = (double)k;
        a.res[1] = (double)nupd;
        int st = ld_volatile(a.status);
        a.res[2] = st != 0 ? (double)st : (converged ? 0.0 : 1.0);
        a.res[3] = rr64;
        a.res[4] = bb;
    }
}

size_t mixed_bytes(uint32_t N) {
    const size_t f = align256((size_t)N * 4), h = align256((size_t)N * 2);
    return 5 * f + 2 * h + align256(kMaxBlocks * 6 * 8) + 3 * 256;
}

}  // namespace

extern "C" size_t nbg_cg_mixed_workspace_bytes(uint32_t N) { return mixed_bytes(N); }

extern "C" int nbg_cg_mixed(const nbg_bsr_t* A, const double* b, double* x, uint32_t max_iter,
                            double tol, double delta, unsigned flags, nbg_mixed_result_t* result,
                            void* ws, size_t ws_bytes, void* stream) {
    if (!result || !A) return NBG_ERR_ARG;
    *result = nbg_mixed_result_t{0, 0, 0, 0.0, 0.0};
    if (A->Nn == 0) return NBG_OK;
    if (!A->b64 || !A->b32 || !A->blo || !A->dinv32 || !(delta > 0.0 && delta < 1.0))
        return NBG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t need = mixed_bytes(A->N);
    void* own = nullptr;
    if (!ws) {
        NBG_CHECK(cudaMalloc(&own, need));
        ws = own;
    } else if (ws_bytes < need) {
        return NBG_ERR_ARG;
    }
    char* base = (char*)ws;
    const size_t f = align256((size_t)A->N * 4), h = align256((size_t)A->N * 2);
    MixArgs a;
    a.A = *A;
    a.b = b;
    a.u = x;
    a.r = (float*)base;
    a.ph = (float*)(base + f);
    a.wh = (float*)(base + 2 * f);
    a.xh = (float*)(base + 3 * f);
    a.xl = (float*)(base + 4 * f);
    a.pl = (__nv_bfloat16*)(base + 5 * f);
    a.wl = (__nv_bfloat16*)(base + 5 * f + h);
    a.part = (double*)(base + 5 * f + 2 * h);
    char* tail = base + 5 * f + 2 * h + align256(kMaxBlocks * 6 * 8);
    a.bar = (unsigned*)tail;
    a.status = (int*)(tail + 256);
    a.res = (double*)(tail + 512);
    a.max_iter = max_iter;
    a.tol = tol;
    a.delta = delta;
    a.flags = flags;
    int rc = NBG_OK;
    unsigned G = 1;
    size_t dyn = 0;
    double hr[5] = {0, 0, 0, 0, 0};
    cudaError_t e = cudaMemsetAsync(tail, 0, 3 * 256, s);
    if (e == cudaSuccess)
        rc = coop_grid_resident((const void*)k_cg_mixed, A->n_slices,
                                NBG_MIXED_RESIDENT ? 56 * 32 : 0, &G, &dyn);
    a.resident = dyn > 0;
    if (e == cudaSuccess && rc == NBG_OK) {
        void* args[] = {&a};
        e = cudaLaunchCooperativeKernel((const void*)k_cg_mixed, dim3(G), dim3(kPersistThreads),
                                        args, dyn, s);
    }
    if (e == cudaSuccess && rc == NBG_OK)
        e = cudaMemcpyAsync(hr, a.res, sizeof(hr), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && rc == NBG_OK) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = nbg_cuda_error(e);
    if (rc == NBG_OK) {
        result->niter = (uint32_t)hr[0];
        result->n_updates = (uint32_t)hr[1];
        result->status = (int)hr[2];
        result->bnorm = sqrt(hr[4]);
        result->relres = hr[4] > 0 ? sqrt(hr[3] / hr[4]) : sqrt(hr[3]);
        rc = result->status;
    }
    if (own) cudaFree(own);
    return rc;
}
