// Mixed-precision Jacobi-PCG with reliable updates, one cooperative launch.
//
// GB300 runs FP32 at many times its FP64 rate, and the stiffness matrices
// here have condition numbers near 1e8, where plain FP32 CG needs several
// times more iterations than FP64.  Measured on the lognormal cantilever
// (1M dof), the inflation comes from three places: the precision of the
// matrix values (even 32 significant bits cost 1.33x the iterations: the
// inner operator must match the FP64 one behind the residual), FP32 search
// directions p and FP32 products A p, and an FP32 correction x.  The
// iteration count alone is not the whole story: with about 40-bit matrix
// values and an FP32 residual the counts match FP64, yet the solution
// keeps an error of 1e-8 to 1e-7 (varying with rounding details) in the
// smooth modes, whose share of the residual is too small for the stopping
// test to see.  A CPU emulation of this solver on the cantilever traced it
// to the FP32 residual (its rounding each iteration feeds those modes) and
// to the matrix precision; with both raised the error matches FP64's.  So
// the inner iteration runs on the FP32 pipes with:
//   matrix      FP32 hi + a 23-bit remainder in units of 2^-46 hi
//               (about 47 significant bits in 7 B/value instead of 8),
//   p, A p      FP32 hi + FP32 lo per dof (float-float),
//   x, r        float-float,
// products and sums by error-free transformations (TwoProduct with FMA,
// TwoSum), dot products with compensated FP32 sums per thread and
// float-float sums across threads and blocks.  A reliable update (Sleijpen
// & van der Vorst 1996) adds x to the FP64 solution and recomputes
// r = b - A u in FP64 with the FP64 values whenever |r| has fallen by
// `delta` since the last one; p is kept, so the Krylov progress survives.
// Convergence is judged on the FP64 residual only.  Three grid barriers per
// iteration in the global-gather form (L1 | L2 | L3 of
// cg_precond_jacobi.c:50-74), two in the ghost-node form below: folding L3
// into the next SpMV (each block rebuilding z + beta p for the columns it
// reads) measured slower, 77 vs 66 us per iteration at 1M dof, because the
// float-float rebuild per column costs more issue slots and gather bytes
// than the barrier it saves.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "perm.cuh"
#include "persist.cuh"

using namespace nbg;

// Keep each block's own-row vectors in shared memory when they fit
// (overridable at build time for tuning).
#ifndef NBG_MIXED_RESIDENT
#define NBG_MIXED_RESIDENT 1
#endif
// The vectors p, A p, x and r are float-float, stored as float4 {hi of both
// dofs, lo of both} per node row: one 16-byte load or store per row and
// vector, one gather per block entry.  (With bfloat16 low parts for p and
// A p the 4M-dof unstructured T3 case needed 26,067 iterations against
// FP64's 22,323; with FP32 ones 22,563.)
#ifndef NBG_MIXED_UNROLL
#define NBG_MIXED_UNROLL 4  // entries in flight per lane in the SpMV
#endif
// One 1024-thread block per SM: with two 512-thread blocks the SM serves one
// block's warps first and the other block's SpMV ends several microseconds
// later, which the next barrier then waits for.
#ifndef NBG_MIXED_THREADS
#define NBG_MIXED_THREADS 1024
#endif
#ifndef NBG_MIXED_MIN_BLOCKS
#define NBG_MIXED_MIN_BLOCKS 1
#endif
constexpr int kMixThreads = NBG_MIXED_THREADS;
constexpr int kMixMinBlocks = NBG_MIXED_MIN_BLOCKS;
// Batched launches give every system at least one block, so they use
// smaller blocks (more of them per SM) than the single-system launch.
#ifndef NBG_BATCH_THREADS
#define NBG_BATCH_THREADS 256
#endif
#ifndef NBG_BATCH_MIN_BLOCKS
#define NBG_BATCH_MIN_BLOCKS 4
#endif
constexpr int kBatThreads = NBG_BATCH_THREADS;
constexpr int kBatMinBlocks = NBG_BATCH_MIN_BLOCKS;
constexpr int kUnroll = NBG_MIXED_UNROLL;
// The ghost-node form's grid barriers by counting (grid_barrier_count),
// whose arrival is a reduction with no return value: 0.2422 against 0.2443
// s per 1M-dof solve with the arrival that returns the old word
// (grid_barrier).
#ifndef NBG_BARRIER_COUNT
#define NBG_BARRIER_COUNT 1
#endif
#ifndef NBG_L2_KEEP
// percent of L2 for the matrix part kept between iterations (1M-dof ghost
// form: 0.2500 s at 40, 0.2560 at 50, 0.2644 at 60, 0.251-0.253 at 10-30:
// the rest of L2 holds the vectors)
#define NBG_L2_KEEP 40
#endif

namespace {

// 1/Aii in shared memory too, or read from global memory (L2) when the
// shared memory is better left to the L1 cache of the SpMV's gathers
#ifndef NBG_MIXED_DV_SHARED
#define NBG_MIXED_DV_SHARED 0
#endif
constexpr bool kDvShared = NBG_MIXED_DV_SHARED;
// own-row bytes per node: p, x, r, A p (16 B each) and 1/Aii (8 B, when
// shared)
constexpr size_t kOwnNodeBytes = 64 + (kDvShared ? 8 : 0);

struct MixArgs {
    nbg_bsr_t A;
    const double* b;
    double* u;
    float4* p;             // search direction, global (gathered by neighbours)
    float4 *x4, *r4, *w4;  // x, r, A p of the rows: own rows when they do not fit in
                           // shared memory (the ghost form keeps x and r there)
    const float *ph, *pl;  // the standalone operator's input, hi and lo apart
    uint32_t max_iter;
    double tol, delta;
    unsigned flags;
    int resident;      // own-row vectors live in shared memory
    uint32_t keep_pm;  // per mille of each block's matrix stream kept in L2
};

// One system of a launch: its slices, its blocks and its synchronisation.
struct Group {
    double* part;  // L1 [0,K), L2 [K,3K), init/update [3K,6K), K = pstride
    unsigned* bar;
    int* status;
    double* res;              // niter, updates, status, rr64, bb, b.u
    uint32_t s_begin, s_end;  // slices
    uint32_t g_base, g_size;  // blocks [g_base, g_base + g_size) of the launch
    uint32_t pstride;
};



// Scalar state of one solve, kept by thread 0 of every block of the group
// (each block derives the same values from the same partial sums).  Per
// iteration it runs on the FP32 pipes: p.w, r.z and |r|^2 arrive as
// float-float sums, the step lengths are float-float quotients (ff_div) and
// the update test compares FP32 leading parts.  GB300 issues FP64 at a small
// fraction of its FP32 rate: one FP64 division on thread 0 held its block
// for about half a microsecond, twice per iteration.  FP64 stays where the
// result is judged, on the true residual at the start and at each reliable
// update.
struct MixScalars {
    FF rz;                          // r.z of the current residual
    double rr64, bb, target2;       // true |r|^2, |b|^2, stopping threshold
    float rmax2, target2f, delta2;  // update test
    uint32_t k, nupd;
    int converged;

    __device__ __forceinline__ void clear() {
        rz = FF{0.f, 0.f};
        rr64 = bb = target2 = 0.0;
        rmax2 = target2f = delta2 = 0.f;
        k = nupd = 0;
        converged = 0;
    }
    // The start's sums {|r|^2, |b|^2, r.z} (FP64): 2 stop, 0 iterate.
    __device__ __forceinline__ int start(const double (&t)[3], const MixArgs& a) {
        rr64 = t[0];
        bb = t[1];
        rz = ff_from_double(t[2]);
        target2 = (a.flags & NBG_CG_RELATIVE) ? a.tol * a.tol * bb : a.tol * a.tol;
        target2f = (float)target2;
        delta2 = (float)(a.delta * a.delta);
        rmax2 = (float)rr64;
        converged = !(rr64 > target2);
        return (converged || a.max_iter == 0) ? 2 : 0;
    }
    __device__ __forceinline__ FF alpha(FF pw) const { return ff_div(rz, pw); }
    // The recursive residual's {r.z, |r|^2}: 1 when a reliable update is
    // due, else 0 with beta.
    __device__ __forceinline__ int step(FF rz_new, FF rr, uint32_t max_iter, FF& beta) {
        if (rr.hi > rmax2) rmax2 = rr.hi;
        k++;
        const int upd = rr.hi <= delta2 * rmax2 || rr.hi <= target2f || k >= max_iter;
        if (!upd) {
            beta = ff_div(rz_new, rz);
            rz = rz_new;
        }
        return upd;
    }
    // A reliable update's {|r|^2, r.z} (FP64): 2 stop, else 0 with beta.
    __device__ __forceinline__ int replaced(const double (&t)[2], uint32_t max_iter, FF& beta) {
        rr64 = t[0];
        rmax2 = (float)rr64;
        nupd++;
        converged = !(rr64 > target2);
        const int stop = converged || k >= max_iter;
        if (!stop) {
            const FF rzn = ff_from_double(t[1]);
            beta = ff_div(rzn, rz);
            rz = rzn;
        }
        return stop ? 2 : 0;
    }
};

// Half of w = A p for node row (s, r): lanes l and l + 16 share row
// r = 16 h + (l & 15) of slice s, taking alternate entries, so a warp works on
// half a slice at a time (the block's 2 (s1 - s0) half slices spread evenly
// over its warps) and each load still covers two 16-entry runs.  The two
// partial float-float sums are combined with one exchange; TwoSum is
// symmetric, so both lanes hold the same bits.  Every lane of the warp must
// call it (the exchange is warp-wide).
// kSplit: p from the separate hi and lo arrays (the standalone operator),
// else from the solver's interleaved copy.
template <bool kSplit = false>
__device__ __forceinline__ void spmv_half_split(const MixArgs& a, uint32_t s, uint32_t r,
                                                uint32_t par, bool live, uint64_t pol, FF& y0,
                                                FF& y1) {
    const float4* __restrict__ bh = reinterpret_cast<const float4*>(a.A.b32);
    const uint2* __restrict__ bl = reinterpret_cast<const uint2*>(a.A.blo);
    const uint32_t* __restrict__ bx = reinterpret_cast<const uint32_t*>(a.A.bxt);
    const float2* __restrict__ ph = reinterpret_cast<const float2*>(a.ph);
    const float2* __restrict__ pl = reinterpret_cast<const float2*>(a.pl);
    const float4* __restrict__ p4 = a.p;
    // scalar accumulators: with p gathered from global memory the packed
    // FP32x2 form of spmv_half_local measured 5 % slower here (4M-dof T3:
    // 192 against 183 us per iteration); the roundings are the same
    FFAcc c0{0.f, 0.f}, c1{0.f, 0.f};
    // rows past Nn in the last slice hold no entries: such lanes only
    // take part in the exchange
    const uint32_t k0 = a.A.slice_off[s] + par, k1 = live ? a.A.slice_off[s + 1] : 0;
#pragma unroll(kUnroll)
    for (uint32_t k = k0; k < k1; k += 2) {
        const size_t e = (size_t)k * 32 + r;
        const uint32_t c = ld_hint(a.A.bcol + e, pol);
        const float4 m = ld_hint(bh + e, pol);  // a00 a10 a01 a11
        const float4 sc = rem23_scale4(ld_hint(bl + e, pol), ld_hint(bx + e, pol));
        float4 pv;
        if (kSplit) {
            const float2 h = ph[c], l = pl[c];
            pv = make_float4(h.x, h.y, l.x, l.y);
        } else {
            pv = p4[c];
        }
        c0.fma2s(m.x, sc.x, pv.x, pv.z);
        c0.fma2s(m.z, sc.z, pv.y, pv.w);
        c1.fma2s(m.y, sc.y, pv.x, pv.z);
        c1.fma2s(m.w, sc.w, pv.y, pv.w);
    }
    FF t[2] = {c0.result(), c1.result()};
#pragma unroll
    for (int j = 0; j < 2; j++) {
        const float h = __shfl_xor_sync(0xffffffffu, t[j].hi, 16);
        const float l = __shfl_xor_sync(0xffffffffu, t[j].lo, 16);
        t[j] = ff_add(t[j], FF{h, l});
    }
    y0 = t[0];
    y1 = t[1];
}

// Own-row vectors of this block, indexed by local node row
// (i - 32 * s0): shared memory when they fit, else the global workspace.
struct Own {
    float4 *p, *x, *r, *w;  // {hi, hi, lo, lo}
    float2* dv;
};

template <bool kRes>
__device__ __forceinline__ Own own_vectors(const MixArgs& a, unsigned char* smem, uint32_t s0,
                                           uint32_t nrows) {
    Own o;
    const size_t base = (size_t)s0 * 32;
    if (kRes) {
        o.p = reinterpret_cast<float4*>(smem);
        o.x = o.p + nrows;
        o.r = o.p + 2 * nrows;
        o.w = o.p + 3 * nrows;
        o.dv = kDvShared ? reinterpret_cast<float2*>(o.p + 4 * nrows)
                         : const_cast<float2*>(reinterpret_cast<const float2*>(a.A.dinv32)) +
                               base;
    } else {
        o.p = a.p + base;
        o.x = a.x4 + base;
        o.r = a.r4 + base;
        o.w = a.w4 + base;
        o.dv = const_cast<float2*>(reinterpret_cast<const float2*>(a.A.dinv32)) + base;
    }
    return o;
}

// r = b - A u in FP64 for the own rows, stored as float-float; z = r / Aii
// (float-float); accumulates |r|^2 (FP64), r.z and optionally |b|^2; with
// set_p, p = z (own copy and the global one).
template <int kThreads>
__device__ __forceinline__ void true_residual(const MixArgs& a, const Own& o, uint32_t s0,
                                              uint32_t s1, double& rr, FFAcc& rz, double* bb,
                                              bool set_p) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nw = kThreads / 32;
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
        const FF f0 = ff_from_double(r0), f1 = ff_from_double(r1);
        o.r[li] = make_float4(f0.hi, f1.hi, f0.lo, f1.lo);
        const float2 di = o.dv[li];
        const FF z0 = ff_mulf(f0, di.x), z1 = ff_mulf(f1, di.y);
        rz.fma2(f0.hi, f0.lo, z0.hi, z0.lo);
        rz.fma2(f1.hi, f1.lo, z1.hi, z1.lo);
        if (set_p) {
            const float4 p = make_float4(z0.hi, z1.hi, z0.lo, z1.lo);
            o.p[li] = p;
            a.p[i] = p;  // the same slot when the own rows are in global memory
        }
    }
}

// The solver of one system on the blocks [g_base, g_base + g_size) of the
// launch: its own slices, group barrier, partial sums and result.  The
// scalar recurrences (step lengths, residual norms, stopping and update
// decisions) run in thread 0 (MixScalars) and reach the block through
// shared memory as FP32 pairs and flags.
template <bool kRes, int kThreads>
__device__ __forceinline__ void mixed_solve(const MixArgs& a, const Group& g, unsigned char* smem) {
    // batched launches give each system at most a few dozen blocks
    constexpr int kRB = kThreads == kMixThreads ? kReduceBatch : 1;
    __shared__ double red[3 * 32];
    float2* const ffred = reinterpret_cast<float2*>(red);
    __shared__ float s_alpha[2], s_beta[2];
    __shared__ int s_flag;  // 0 iterate, 1 reliable update, 2 stop
    __shared__ MixScalars sc;  // thread 0 only
    const unsigned G = g.g_size;
    const uint32_t rank = blockIdx.x - g.g_base;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nw = kThreads / 32;
    uint32_t s0, s1;
    group_slice_range(g.s_begin, g.s_end, rank, G, s0, s1);
    const uint32_t Nn = a.A.Nn;
    const Own o = own_vectors<kRes>(a, smem, s0, (s1 - s0) * 32);
    float4* __restrict__ gp = a.p;
    double* const part0 = g.part;
    double* const part1 = g.part + g.pstride;
    double* const part2 = g.part + 3 * g.pstride;
    // the arrival that returns the old word: with the counting barrier the
    // global-gather and batched launches ran slower (4M-dof T3: 4.19 against
    // 4.07 s; the 96-system batch: 1.43 against 1.36 s)
    auto sync = [&]() { return grid_barrier(g.bar, G, rank, g.status); };

    if (threadIdx.x == 0) sc.clear();
    {   // init: own copy of 1/Aii, x = 0, r = b - A u (FP64), p = z
        const float2* __restrict__ gdv = reinterpret_cast<const float2*>(a.A.dinv32);
        for (uint32_t s = s0 + warp; s < s1; s += nw) {
            const uint32_t i = s * 32 + lane, li = i - s0 * 32;
            if (i >= Nn) continue;
            if (kRes && kDvShared) o.dv[li] = gdv[i];
            o.x[li] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncwarp();
        double rrl = 0.0, bbl = 0.0;
        FFAcc rzk{0.f, 0.f};
        true_residual<kThreads>(a, o, s0, s1, rrl, rzk, &bbl, true);
        const FF t = rzk.result();
        double v[3] = {rrl, bbl, (double)t.hi + (double)t.lo};
        group_publish<3>(v, red, part2, rank);
    }
    if (sync()) goto done;
    {
        double t[3];
        group_reduce0<3>(part2, G, t);
        if (threadIdx.x == 0) s_flag = sc.start(t, a);
        __syncthreads();
    }
    while (s_flag != 2) {
        {   // L1: w = A p, p.w (two lanes per node row)
            FFAcc pw{0.f, 0.f};
            const uint32_t par = lane >> 4, nh = 2 * (s1 - s0);
            // warp w takes half slices w, w + nw, ...
            for (uint32_t h = warp; h < nh; h += nw) {
                const uint32_t s = s0 + (h >> 1), r = ((h & 1) << 4) | (lane & 15);
                const uint32_t i = s * 32 + r, li = i - s0 * 32;
                // a slice's rows past Nn are padding: skip them whole (both lanes)
                if (s * 32 + ((h & 1) << 4) >= Nn) continue;
                FF y0, y1;
                // the first keep_pm / 1000 of this block's slices stay in L2
                const uint64_t pol = l2_policy((s - s0) * 1000u < a.keep_pm * (s1 - s0));
                spmv_half_split(a, s, r, par, i < Nn, pol, y0, y1);
                if (par || i >= Nn) continue;
                o.w[li] = make_float4(y0.hi, y1.hi, y0.lo, y1.lo);
                const float4 p = o.p[li];
                pw.fma2(p.x, p.z, y0.hi, y0.lo);
                pw.fma2(p.y, p.w, y1.hi, y1.lo);
            }
            FF v[1] = {pw.result()};
            group_publish_ff<1>(v, ffred, reinterpret_cast<float2*>(part0), rank);
        }
        if (sync()) goto done;
        {
            FF pw[1];
            group_reduce0_ff<1, kRB>(reinterpret_cast<const float2*>(part0), G, pw);
            if (threadIdx.x == 0) {
                const FF al = sc.alpha(pw[0]);
                s_alpha[0] = al.hi;
                s_alpha[1] = al.lo;
            }
            __syncthreads();
        }
        {   // L2: x += alpha p, r -= alpha w, z = r / Aii (own rows only)
            const FF alpha = {s_alpha[0], s_alpha[1]};
            FFAcc rzk{0.f, 0.f}, rrk{0.f, 0.f};
            for (uint32_t s = s0 + warp; s < s1; s += nw) {
                const uint32_t i = s * 32 + lane, li = i - s0 * 32;
                if (i >= Nn) continue;
                const float4 p = o.p[li], w = o.w[li], xo = o.x[li], ri = o.r[li];
                const float2 di = o.dv[li];
                const FF x0 = ff_add({xo.x, xo.z}, ff_mul(alpha, {p.x, p.z}));
                const FF x1 = ff_add({xo.y, xo.w}, ff_mul(alpha, {p.y, p.w}));
                o.x[li] = make_float4(x0.hi, x1.hi, x0.lo, x1.lo);
                const FF aw0 = ff_mul(alpha, {w.x, w.z}), aw1 = ff_mul(alpha, {w.y, w.w});
                const FF r0 = ff_add({ri.x, ri.z}, {-aw0.hi, -aw0.lo});
                const FF r1 = ff_add({ri.y, ri.w}, {-aw1.hi, -aw1.lo});
                o.r[li] = make_float4(r0.hi, r1.hi, r0.lo, r1.lo);
                const FF z0 = ff_mulf(r0, di.x), z1 = ff_mulf(r1, di.y);
                rzk.fma2(r0.hi, r0.lo, z0.hi, z0.lo);
                rzk.fma2(r1.hi, r1.lo, z1.hi, z1.lo);
                rrk.fma2(r0.hi, r0.lo, r0.hi, r0.lo);
                rrk.fma2(r1.hi, r1.lo, r1.hi, r1.lo);
            }
            FF v[2] = {rzk.result(), rrk.result()};
            group_publish_ff<2>(v, ffred, reinterpret_cast<float2*>(part1), rank);
        }
        if (sync()) goto done;
        {
            FF t2[2];
            group_reduce0_ff<2, kRB>(reinterpret_cast<const float2*>(part1), G, t2);
            if (threadIdx.x == 0) {
                FF be;
                s_flag = sc.step(t2[0], t2[1], a.max_iter, be);
                if (!s_flag) {
                    s_beta[0] = be.hi;
                    s_beta[1] = be.lo;
                }
            }
            __syncthreads();
        }
        if (s_flag) {
            // reliable update: u += x in FP64, then r = b - A u in FP64
            double2* __restrict__ u = reinterpret_cast<double2*>(a.u);
            for (uint32_t s = s0 + warp; s < s1; s += nw) {
                const uint32_t i = s * 32 + lane, li = i - s0 * 32;
                if (i >= Nn) continue;
                const float4 xo = o.x[li];
                double2 ui = u[i];
                ui.x += (double)xo.x + (double)xo.z;
                ui.y += (double)xo.y + (double)xo.w;
                u[i] = ui;
                o.x[li] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            if (sync()) goto done;
            double rrl = 0.0;
            FFAcc rzk{0.f, 0.f};
            true_residual<kThreads>(a, o, s0, s1, rrl, rzk, nullptr, false);
            const FF t = rzk.result();
            double v[2] = {rrl, (double)t.hi + (double)t.lo};
            group_publish<2>(v, red, part2, rank);
            if (sync()) goto done;
            double tt[2];
            group_reduce0<2>(part2, G, tt);
            if (threadIdx.x == 0) {
                FF be;
                s_flag = sc.replaced(tt, a.max_iter, be);
                if (!s_flag) {
                    s_beta[0] = be.hi;
                    s_beta[1] = be.lo;
                }
            }
            __syncthreads();
            if (s_flag == 2) break;
        }
        {   // L3: p = z + beta p (own copy and the global one)
            const FF beta = {s_beta[0], s_beta[1]};
            for (uint32_t s = s0 + warp; s < s1; s += nw) {
                const uint32_t i = s * 32 + lane, li = i - s0 * 32;
                if (i >= Nn) continue;
                const float4 ri = o.r[li], p = o.p[li];
                const float2 di = o.dv[li];
                const FF n0 = ff_add(ff_mulf({ri.x, ri.z}, di.x), ff_mul(beta, {p.x, p.z}));
                const FF n1 = ff_add(ff_mulf({ri.y, ri.w}, di.y), ff_mul(beta, {p.y, p.w}));
                const float4 pn = make_float4(n0.hi, n1.hi, n0.lo, n1.lo);
                if (kRes) o.p[li] = pn;
                gp[i] = pn;
            }
        }
        if (sync()) goto done;
    }
    {   // b.u in FP64 (the compliance F^T u when b is the load vector).  part0
        // was last read before the L2 barrier of the last iteration.
        const double2* __restrict__ u = reinterpret_cast<const double2*>(a.u);
        const double2* __restrict__ b = reinterpret_cast<const double2*>(a.b);
        double bu = 0.0;
        for (uint32_t s = s0 + warp; s < s1; s += nw) {
            const uint32_t i = s * 32 + lane;
            if (i >= Nn) continue;
            const double2 ui = u[i], bi = b[i];
            bu = fma(bi.x, ui.x, fma(bi.y, ui.y, bu));
        }
        double v[1] = {bu};
        group_publish<1>(v, red, part0, rank);
        if (sync()) goto done;
        double J[1];
        group_reduce0<1>(part0, G, J);
        if (rank == 0 && threadIdx.x == 0) g.res[5] = J[0];
    }
done:
    if (rank == 0 && threadIdx.x == 0) {
        g.res[0] = (double)sc.k;
        g.res[1] = (double)sc.nupd;
        int st = ld_volatile(g.status);
        g.res[2] = st != 0 ? (double)st : (sc.converged ? 0.0 : 1.0);
        g.res[3] = sc.rr64;
        g.res[4] = sc.bb;
    }
}

// kRes: the block's own-row vectors live in dynamic shared memory (known at
// compile time, so their addresses are 32-bit shared ones).
template <bool kRes>
__global__ void __launch_bounds__(kMixThreads, kMixMinBlocks) k_cg_mixed(MixArgs a,
                                                                                Group g) {
    extern __shared__ __align__(16) unsigned char smem[];
    mixed_solve<kRes, kMixThreads>(a, g, smem);
}

// Many independent systems stored in one block-diagonal layout, in one
// launch: block b works for system groups[block_of[b]].
template <bool kRes>
__global__ void __launch_bounds__(kBatThreads, kBatMinBlocks)
    k_cg_mixed_many(MixArgs a, const Group* __restrict__ groups,
                    const uint32_t* __restrict__ block_of) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ Group sg;
    if (threadIdx.x == 0) sg = groups[block_of[blockIdx.x]];
    __syncthreads();
    mixed_solve<kRes, kBatThreads>(a, sg, smem);
}

// Share of the SpMV's matrix stream (FP32 values, remainders, columns:
// 32 B per block entry) marked evict_last: what fits in NBG_L2_KEEP percent
// of this device's L2, the rest of L2 being left to the gathered vector and
// the other data.
uint32_t keep_permille(const nbg_bsr_t& A, double bytes_per_entry = 32.0) {
    int dev = 0, l2 = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess)
        return 0;
    const double stream = bytes_per_entry * (double)A.n_entries;
    const double budget = l2 * (NBG_L2_KEEP / 100.0);
    if (stream <= 0.0 || budget >= stream) return 1000;
    return (uint32_t)(1000.0 * budget / stream);
}

size_t mixed_core_bytes(uint32_t N) {
    const size_t f = align256((size_t)N * 4), h = align256((size_t)N * 4);
    return 6 * f + 2 * h + align256(kMaxBlocks * 6 * 8) + 3 * 256;
}

// The vector slots at the start of a workspace (indexed by node row, a
// float4 each): p, x, r, A p.
void carve_vectors(MixArgs& a, char* base, uint32_t N) {
    const size_t f = align256((size_t)N * 4);
    a.p = (float4*)base;
    a.x4 = (float4*)(base + 2 * f);
    a.r4 = (float4*)(base + 4 * f);
    a.w4 = (float4*)(base + 6 * f);
    a.ph = a.pl = nullptr;
}

// plus the permuted copies of b and x for a layout with a node order
size_t mixed_bytes(uint32_t N) { return mixed_core_bytes(N) + perm_tail_bytes(N); }

// The mixed solver's SpMV operator as its own launch: w = A p with the split
// matrix and float-float p, two lanes per node row, the solver's L2 policy
// (the first keep_pm / 1000 of each block's slices evict_last).  One block per
// SM, slices split evenly, as in the solver.
__global__ void __launch_bounds__(kMixThreads, kMixMinBlocks)
    k_spmv_mixed(MixArgs a, float2* __restrict__ wh, float2* __restrict__ wl) {
    uint32_t s0, s1;
    slice_range(a.A.n_slices, s0, s1);
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nw = kMixThreads / 32, par = lane >> 4, nh = 2 * (s1 - s0);
    for (uint32_t h = warp; h < nh; h += nw) {
        const uint32_t s = s0 + (h >> 1), r = ((h & 1) << 4) | (lane & 15);
        const uint32_t i = s * 32 + r;
        if (s * 32 + ((h & 1) << 4) >= a.A.Nn) continue;
        FF y0, y1;
        const uint64_t pol = l2_policy((s - s0) * 1000u < a.keep_pm * (s1 - s0));
        spmv_half_split<true>(a, s, r, par, i < a.A.Nn, pol, y0, y1);
        if (par || i >= a.A.Nn) continue;
        wh[i] = make_float2(y0.hi, y1.hi);
        wl[i] = make_float2(y0.lo, y1.lo);
    }
}

// ---------------------------------------------------------------------------
// Ghost-node form of the single-system solver.
//
// A block's SpMV reads p at its own rows and at the rows of other blocks that
// its rows couple to, its ghosts (on the 1M-dof cantilever, a block's strip of
// about 3.4 grid rows has the two neighbouring grid rows as ghosts, 0.6 times
// its own row count).  This form keeps p for the block's own rows and for
// its ghosts in shared memory, with the layout's columns renumbered locally
// in 16 bits (own row slots first, then the ghosts in ascending node order),
// so the SpMV gathers from shared memory, not L2, and the matrix stream is
// 30 B per block entry instead of 32.  Owners publish their residual r
// (after L2 and after each reliable update); after the barrier that ends L2
// every block computes its ghosts' new p itself, with the owner's arithmetic
// on the owner's r and on its own copy of the ghost's previous p (the same
// bits, by induction from p = z at the start), so the third barrier of each
// iteration (the exchange of p) goes away.  The iterates equal those of the
// global-gather form bit for bit.  x moves to global memory to leave shared
// memory to the ghosts.
//
// The plan (ghost lists, local columns) depends on the launch's block
// partition and is rebuilt by a short kernel at the start of every solve.
#ifndef NBG_MIXED_SO_SMEM
#define NBG_MIXED_SO_SMEM 1  // the block's slice offsets in shared memory
#endif
constexpr uint32_t kGhostMax = 16384;   // ghosts per block
constexpr uint32_t kGhostKeys = 32768;  // outside-column references per block the plan sorts

struct GhostArgs {
    const uint16_t* lcol;   // local column of every layout entry
    const uint32_t* ids;    // kGhostMax ghost node ids per block, ascending
    const uint32_t* count;  // ghosts per block
    uint32_t scap;          // own row slots of the largest block
    uint32_t pcap;          // row slots + ghosts, largest over the blocks
    uint32_t gcap;          // ghosts, largest over the blocks
};

// One block per group of the solver's partition: its ghosts (the columns of
// its live rows outside its row slots, sorted and made unique in shared
// memory) and the local column of each of its entries.  *fail is set when a
// block has more outside references than kGhostKeys, more ghosts than
// kGhostMax, or more than 65535 local columns; the solver then keeps the
// global-gather form.
__global__ void __launch_bounds__(1024, 1) k_ghost_plan(nbg_bsr_t A, uint16_t* lcol,
                                                      uint32_t* ids, uint32_t* count,
                                                      int* fail) {
    extern __shared__ __align__(16) uint32_t keys[];  // kGhostKeys
    __shared__ uint32_t s_n;
    __shared__ uint32_t s_scan[32];
    const uint32_t tid = threadIdx.x, bd = blockDim.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t nw = bd >> 5;
    uint32_t s0, s1;
    slice_range(A.n_slices, s0, s1);
    const uint32_t n0 = s0 * 32, nslot = (s1 - s0) * 32;
    if (tid == 0) s_n = 0;
    __syncthreads();
    for (uint32_t s = s0 + warp; s < s1; s += nw) {
        const uint32_t i = s * 32 + lane;
        if (i >= A.Nn) continue;
        for (uint32_t k = A.slice_off[s]; k < A.slice_off[s + 1]; k++) {
            const uint32_t c = A.bcol[(size_t)k * 32 + lane];
            if (c - n0 >= nslot) {
                const uint32_t pos = atomicAdd(&s_n, 1u);
                if (pos < kGhostKeys) keys[pos] = c;
            }
        }
    }
    __syncthreads();
    const uint32_t n = s_n;
    if (n > kGhostKeys) {  // the same n in every thread
        if (tid == 0) atomicExch(fail, 1);
        return;
    }
    uint32_t P2 = 1;
    while (P2 < n) P2 <<= 1;
    for (uint32_t j = n + tid; j < P2; j += bd) keys[j] = 0xffffffffu;
    __syncthreads();
    // bitonic sort of keys[0, P2)
    for (uint32_t size = 2; size <= P2; size <<= 1)
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t t = tid; t < P2 / 2; t += bd) {
                const uint32_t lo = 2 * stride * (t / stride) + (t % stride), hi = lo + stride;
                const uint32_t x = keys[lo], y = keys[hi];
                if ((x > y) == ((lo & size) == 0)) {
                    keys[lo] = y;
                    keys[hi] = x;
                }
            }
            __syncthreads();
        }
    // unique: each thread counts the first occurrences in its chunk, an
    // exclusive block scan places them
    const uint32_t chunk = (n + bd - 1) / bd;
    const uint32_t j0 = min(tid * chunk, n), j1 = min(j0 + chunk, n);
    uint32_t cnt = 0;
    for (uint32_t j = j0; j < j1; j++) cnt += (j == 0 || keys[j] != keys[j - 1]);
    uint32_t v = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= (uint32_t)o) v += t;
    }
    if (lane == 31) s_scan[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nw ? s_scan[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (uint32_t)o) w += t;
        }
        s_scan[lane] = w;
    }
    __syncthreads();
    const uint32_t u = s_scan[nw - 1];
    if (u > kGhostMax || nslot + u > 65535u) {  // the same u in every thread
        if (tid == 0) atomicExch(fail, 1);
        return;
    }
    uint32_t* const my = ids + (size_t)blockIdx.x * kGhostMax;
    uint32_t pos = v - cnt + (warp ? s_scan[warp - 1] : 0);
    for (uint32_t j = j0; j < j1; j++)
        if (j == 0 || keys[j] != keys[j - 1]) my[pos++] = keys[j];
    __syncthreads();
    for (uint32_t j = tid; j < u; j += bd) keys[j] = my[j];
    if (tid == 0) count[blockIdx.x] = u;
    __syncthreads();
    for (uint32_t s = s0 + warp; s < s1; s += nw) {
        const uint32_t i = s * 32 + lane;
        for (uint32_t k = A.slice_off[s]; k < A.slice_off[s + 1]; k++) {
            const size_t e = (size_t)k * 32 + lane;
            uint32_t lc = i - n0;  // rows past Nn (never read): their own slot
            if (i < A.Nn) {
                const uint32_t c = A.bcol[e];
                if (c - n0 < nslot) {
                    lc = c - n0;
                } else {
                    uint32_t lo = 0, hi = u;  // first ghost >= c (it is there)
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (keys[mid] < c) lo = mid + 1; else hi = mid;
                    }
                    lc = nslot + lo;
                }
            }
            lcol[e] = (uint16_t)lc;
        }
    }
}

// spmv_half_split with local columns and p (own rows and ghosts) in shared
// memory as float4 {hi of both dofs, lo of both dofs}; the same products and
// sums in the same order.
__device__ __forceinline__ void spmv_half_local(const MixArgs& a, const uint16_t* __restrict__ lcol,
                                                const float4* P, const uint32_t* so,
                                                uint32_t s, uint32_t r, uint32_t par, bool live,
                                                uint64_t pol, FF& y0, FF& y1) {
    const float4* __restrict__ bh = reinterpret_cast<const float4*>(a.A.b32);
    const uint2* __restrict__ bl = reinterpret_cast<const uint2*>(a.A.blo);
    const uint32_t* __restrict__ bx = reinterpret_cast<const uint32_t*>(a.A.bxt);
    FFAcc2 acc{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};  // rows 0 and 1
    // so: this block's slice offsets, so[0] that of its first slice
    const uint32_t k0 = so[s] + par, k1 = live ? so[s + 1] : 0;
#pragma unroll(kUnroll)
    for (uint32_t k = k0; k < k1; k += 2) {
        const size_t e = (size_t)k * 32 + r;
        const uint32_t c = ld_hint(lcol + e, pol);
        const float4 m = ld_hint(bh + e, pol);  // a00 a10 a01 a11
        const float4 sc = rem23_scale4(ld_hint(bl + e, pol), ld_hint(bx + e, pol));
        const float4 pv = P[c];
        acc.fma2s(make_float2(m.x, m.y), make_float2(sc.x, sc.y), pv.x, pv.z);
        acc.fma2s(make_float2(m.z, m.w), make_float2(sc.z, sc.w), pv.y, pv.w);
    }
    FF t[2] = {FFAcc{acc.s.x, acc.c.x}.result(), FFAcc{acc.s.y, acc.c.y}.result()};
#pragma unroll
    for (int j = 0; j < 2; j++) {
        const float h = __shfl_xor_sync(0xffffffffu, t[j].hi, 16);
        const float l = __shfl_xor_sync(0xffffffffu, t[j].lo, 16);
        t[j] = ff_add(t[j], FF{h, l});
    }
    y0 = t[0];
    y1 = t[1];
}

// The ghost form keeps r and x in global memory (the workspace's r and x
// rows).
__device__ __forceinline__ float4* ghost_r(const MixArgs& a) { return a.r4; }
__device__ __forceinline__ float4* ghost_x(const MixArgs& a) { return a.x4; }

// true_residual for the ghost form: r (float-float) to global memory, where
// the owner keeps it and the blocks that hold this row as a ghost read it.
template <int kThreads>
__device__ __forceinline__ void true_residual_ghost(const MixArgs& a, float4* P,
                                                    uint32_t s0, uint32_t s1, double& rr,
                                                    FFAcc& rz, double* bb, bool set_p) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nw = kThreads / 32;
    const double2* __restrict__ u = reinterpret_cast<const double2*>(a.u);
    const double2* __restrict__ b = reinterpret_cast<const double2*>(a.b);
    const float2* __restrict__ dinv = reinterpret_cast<const float2*>(a.A.dinv32);
    float4* __restrict__ r4 = ghost_r(a);
    for (uint32_t s = s0 + warp; s < s1; s += nw) {
        const uint32_t i = s * 32 + lane, li = i - s0 * 32;
        if (i >= a.A.Nn) continue;
        const double2 au = spmv_row_f64(a.A, s, lane, u);
        const double2 bi = b[i];
        const double r0 = bi.x - au.x, r1 = bi.y - au.y;
        rr = fma(r0, r0, fma(r1, r1, rr));
        if (bb) *bb = fma(bi.x, bi.x, fma(bi.y, bi.y, *bb));
        const FF f0 = ff_from_double(r0), f1 = ff_from_double(r1);
        r4[i] = make_float4(f0.hi, f1.hi, f0.lo, f1.lo);
        const float2 di = dinv[i];
        const FF z0 = ff_mulf(f0, di.x), z1 = ff_mulf(f1, di.y);
        rz.fma2(f0.hi, f0.lo, z0.hi, z0.lo);
        rz.fma2(f1.hi, f1.lo, z1.hi, z1.lo);
        if (set_p) P[li] = make_float4(z0.hi, z1.hi, z0.lo, z1.lo);
    }
}

template <int kThreads>
__device__ __forceinline__ void mixed_solve_ghost(const MixArgs& a, const Group& g,
                                                  const GhostArgs& gh, unsigned char* smem) {
    __shared__ double red[3 * 32];
    float2* const ffred = reinterpret_cast<float2*>(red);
    __shared__ float s_alpha[2], s_beta[2];
    __shared__ int s_flag;  // 0 iterate, 1 reliable update, 2 stop
    __shared__ MixScalars sc;  // thread 0 only
    const unsigned G = g.g_size;
    const uint32_t rank = blockIdx.x - g.g_base;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t nw = kThreads / 32;
    uint32_t s0, s1;
    group_slice_range(g.s_begin, g.s_end, rank, G, s0, s1);
    const uint32_t Nn = a.A.Nn, nslot = (s1 - s0) * 32;
    const uint32_t ng = gh.count[rank];
    float4* const P = reinterpret_cast<float4*>(smem);
    float4* const W = P + gh.pcap;  // A p of the own rows {hi, hi, lo, lo}
    uint32_t* const GID = reinterpret_cast<uint32_t*>(W + gh.scap);
    // slice offsets of this block, indexed by s - s0
    uint32_t* const SO = NBG_MIXED_SO_SMEM ? GID + gh.gcap
                                           : const_cast<uint32_t*>(a.A.slice_off) + s0;
    float4* __restrict__ r4 = ghost_r(a);
    float4* __restrict__ x4 = ghost_x(a);
    const float2* __restrict__ dinv = reinterpret_cast<const float2*>(a.A.dinv32);
    double* const part0 = g.part;
    double* const part1 = g.part + g.pstride;
    double* const part2 = g.part + 3 * g.pstride;
#if NBG_BARRIER_COUNT
    unsigned bar_target = 0;
    auto sync = [&]() { return grid_barrier_count(g.bar, G, bar_target, g.status); };
#else
    auto sync = [&]() { return grid_barrier(g.bar, G, rank, g.status); };
#endif

    if (tid == 0) sc.clear();
    for (uint32_t j = tid; j < ng; j += kThreads) GID[j] = gh.ids[(size_t)rank * kGhostMax + j];
    if (NBG_MIXED_SO_SMEM)
        for (uint32_t j = tid; j <= s1 - s0; j += kThreads) SO[j] = a.A.slice_off[s0 + j];
    {   // init: x = 0, r = b - A u (FP64), own p = z, r published
        for (uint32_t s = s0 + warp; s < s1; s += nw) {
            const uint32_t i = s * 32 + lane;
            if (i >= Nn) continue;
            x4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        double rrl = 0.0, bbl = 0.0;
        FFAcc rzk{0.f, 0.f};
        true_residual_ghost<kThreads>(a, P, s0, s1, rrl, rzk, &bbl, true);
        const FF t = rzk.result();
        double v[3] = {rrl, bbl, (double)t.hi + (double)t.lo};
        group_publish<3>(v, red, part2, rank);
    }
    if (sync()) goto done;
    {
        double t[3];
        group_reduce0<3>(part2, G, t);
        if (tid == 0) s_flag = sc.start(t, a);
        // ghosts start as their owners' p = z
        for (uint32_t j = tid; j < ng; j += kThreads) {
            const uint32_t c = GID[j];
            const float4 rc = r4[c];
            const float2 dc = dinv[c];
            const FF z0 = ff_mulf({rc.x, rc.z}, dc.x), z1 = ff_mulf({rc.y, rc.w}, dc.y);
            P[nslot + j] = make_float4(z0.hi, z1.hi, z0.lo, z1.lo);
        }
        __syncthreads();
    }
    while (s_flag != 2) {
        {   // L1: w = A p from shared memory, p.w (two lanes per node row)
            FFAcc pw{0.f, 0.f};
            const uint32_t par = lane >> 4, nh = 2 * (s1 - s0);
            for (uint32_t h = warp; h < nh; h += nw) {
                const uint32_t s = s0 + (h >> 1), r = ((h & 1) << 4) | (lane & 15);
                const uint32_t i = s * 32 + r, li = i - s0 * 32;
                if (s * 32 + ((h & 1) << 4) >= Nn) continue;
                FF y0, y1;
                const uint64_t pol = l2_policy((s - s0) * 1000u < a.keep_pm * (s1 - s0));
                spmv_half_local(a, gh.lcol, P, SO, s - s0, r, par, i < Nn, pol, y0, y1);
                if (par || i >= Nn) continue;
                W[li] = make_float4(y0.hi, y1.hi, y0.lo, y1.lo);
                const float4 p = P[li];
                pw.fma2(p.x, p.z, y0.hi, y0.lo);
                pw.fma2(p.y, p.w, y1.hi, y1.lo);
            }
            FF v[1] = {pw.result()};
            group_publish_ff<1>(v, ffred, reinterpret_cast<float2*>(part0), rank);
        }
        if (sync()) goto done;
        {
            FF pw[1];
            group_reduce0_ff<1>(reinterpret_cast<const float2*>(part0), G, pw);
            if (tid == 0) {
                const FF al = sc.alpha(pw[0]);
                s_alpha[0] = al.hi;
                s_alpha[1] = al.lo;
            }
            __syncthreads();
        }
        {   // L2: x += alpha p, r -= alpha w, z = r / Aii; r published
            const FF alpha = {s_alpha[0], s_alpha[1]};
            FFAcc rzk{0.f, 0.f}, rrk{0.f, 0.f};
            // both dofs of a row at once on the packed FP32x2 instructions
            // (the same roundings as the global-gather form's scalar code)
            const FF2 alpha2 = ff2_bcast(alpha);
            auto lohi = [](float4 v) -> FF2 {
                return {make_float2(v.x, v.y), make_float2(v.z, v.w)};
            };
            auto row = [&](uint32_t i, float4 xo, float4 ro, float2 di) {
                const uint32_t li = i - s0 * 32;
                const FF2 x = ff2_add(lohi(xo), ff2_mul(alpha2, lohi(P[li])));
                x4[i] = make_float4(x.hi.x, x.hi.y, x.lo.x, x.lo.y);
                const FF2 aw = ff2_mul(alpha2, lohi(W[li]));
                const FF2 r = ff2_add(lohi(ro), {f2neg(aw.hi), f2neg(aw.lo)});
                r4[i] = make_float4(r.hi.x, r.hi.y, r.lo.x, r.lo.y);
                const FF2 z = ff2_mulf(r, di);
                rzk.fma2(r.hi.x, r.lo.x, z.hi.x, z.lo.x);
                rzk.fma2(r.hi.y, r.lo.y, z.hi.y, z.lo.y);
                rrk.fma2(r.hi.x, r.lo.x, r.hi.x, r.lo.x);
                rrk.fma2(r.hi.y, r.lo.y, r.hi.y, r.lo.y);
            };
            // two slices per step, their global loads issued together (one
            // memory round trip for both); rows in the same order as one
            // slice per step, so the sums are unchanged
            for (uint32_t s = s0 + warp; s < s1; s += 2 * nw) {
                const uint32_t iA = s * 32 + lane, iB = iA + 32 * nw;
                if (iA >= Nn) continue;
                const bool vB = s + nw < s1 && iB < Nn;
                const float4 xA = x4[iA], rA = r4[iA];
                const float2 dA = dinv[iA];
                float4 xB{}, rB{};
                float2 dB{};
                if (vB) {
                    xB = x4[iB];
                    rB = r4[iB];
                    dB = dinv[iB];
                }
                row(iA, xA, rA, dA);
                if (vB) row(iB, xB, rB, dB);
            }
            FF v[2] = {rzk.result(), rrk.result()};
            group_publish_ff<2>(v, ffred, reinterpret_cast<float2*>(part1), rank);
        }
        if (sync()) goto done;
        {
            FF t2[2];
            group_reduce0_ff<2>(reinterpret_cast<const float2*>(part1), G, t2);
            if (tid == 0) {
                FF be;
                s_flag = sc.step(t2[0], t2[1], a.max_iter, be);
                if (!s_flag) {
                    s_beta[0] = be.hi;
                    s_beta[1] = be.lo;
                }
            }
            __syncthreads();
        }
        if (s_flag) {
            // reliable update: u += x in FP64, then r = b - A u in FP64
            double2* __restrict__ u = reinterpret_cast<double2*>(a.u);
            for (uint32_t s = s0 + warp; s < s1; s += nw) {
                const uint32_t i = s * 32 + lane;
                if (i >= Nn) continue;
                const float4 xo = x4[i];
                double2 ui = u[i];
                ui.x += (double)xo.x + (double)xo.z;
                ui.y += (double)xo.y + (double)xo.w;
                u[i] = ui;
                x4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            if (sync()) goto done;
            double rrl = 0.0;
            FFAcc rzk{0.f, 0.f};
            true_residual_ghost<kThreads>(a, P, s0, s1, rrl, rzk, nullptr, false);
            const FF t = rzk.result();
            double v[2] = {rrl, (double)t.hi + (double)t.lo};
            group_publish<2>(v, red, part2, rank);
            if (sync()) goto done;
            double tt[2];
            group_reduce0<2>(part2, G, tt);
            if (tid == 0) {
                FF be;
                s_flag = sc.replaced(tt, a.max_iter, be);
                if (!s_flag) {
                    s_beta[0] = be.hi;
                    s_beta[1] = be.lo;
                }
            }
            __syncthreads();
            if (s_flag == 2) break;
        }
        {   // L3: p = z + beta p for the own rows and the ghosts (no barrier:
            // every p this block's next SpMV reads is in its shared memory)
            const FF beta = {s_beta[0], s_beta[1]};
            // p slot l from the row's r (hi, lo) and 1/Aii
            const FF2 beta2 = ff2_bcast(beta);
            auto pnew = [&](uint32_t l, float4 rv, float2 di) {
                const float4 p = P[l];
                const FF2 n = ff2_add(ff2_mulf({make_float2(rv.x, rv.y), make_float2(rv.z, rv.w)}, di),
                                      ff2_mul(beta2, {make_float2(p.x, p.y), make_float2(p.z, p.w)}));
                P[l] = make_float4(n.hi.x, n.hi.y, n.lo.x, n.lo.y);
            };
            // two slices (two ghosts) per step, their loads issued together
            for (uint32_t s = s0 + warp; s < s1; s += 2 * nw) {
                const uint32_t iA = s * 32 + lane, iB = iA + 32 * nw;
                if (iA >= Nn) continue;
                const bool vB = s + nw < s1 && iB < Nn;
                const float4 rA = r4[iA];
                const float2 dA = dinv[iA];
                float4 rB{};
                float2 dB{};
                if (vB) {
                    rB = r4[iB];
                    dB = dinv[iB];
                }
                pnew(iA - s0 * 32, rA, dA);
                if (vB) pnew(iB - s0 * 32, rB, dB);
            }
            for (uint32_t j = tid; j < ng; j += 2 * kThreads) {
                const uint32_t jB = j + kThreads;
                const uint32_t cA = GID[j], cB = jB < ng ? GID[jB] : cA;
                const float4 rA = r4[cA], rB = r4[cB];
                const float2 dA = dinv[cA], dB = dinv[cB];
                pnew(nslot + j, rA, dA);
                if (jB < ng) pnew(nslot + jB, rB, dB);
            }
            __syncthreads();
        }
    }
    {   // b.u in FP64 (the compliance F^T u when b is the load vector).  part0
        // was last read before the L2 barrier of the last iteration.
        const double2* __restrict__ u = reinterpret_cast<const double2*>(a.u);
        const double2* __restrict__ b = reinterpret_cast<const double2*>(a.b);
        double bu = 0.0;
        for (uint32_t s = s0 + warp; s < s1; s += nw) {
            const uint32_t i = s * 32 + lane;
            if (i >= Nn) continue;
            const double2 ui = u[i], bi = b[i];
            bu = fma(bi.x, ui.x, fma(bi.y, ui.y, bu));
        }
        double v[1] = {bu};
        group_publish<1>(v, red, part0, rank);
        if (sync()) goto done;
        double J[1];
        group_reduce0<1>(part0, G, J);
        if (rank == 0 && tid == 0) g.res[5] = J[0];
    }
done:
    if (rank == 0 && tid == 0) {
        g.res[0] = (double)sc.k;
        g.res[1] = (double)sc.nupd;
        int st = ld_volatile(g.status);
        g.res[2] = st != 0 ? (double)st : (sc.converged ? 0.0 : 1.0);
        g.res[3] = sc.rr64;
        g.res[4] = sc.bb;
    }
}

__global__ void __launch_bounds__(kMixThreads, kMixMinBlocks)
    k_cg_mixed_ghost(MixArgs a, Group g, GhostArgs gh) {
    extern __shared__ __align__(16) unsigned char smem[];
    mixed_solve_ghost<kMixThreads>(a, g, gh, smem);
}

// Workspace of the ghost plan for layout A on this device: local columns,
// ghost lists of up to one block per SM, counts, the failure flag.
size_t ghost_plan_bytes(const nbg_bsr_t& A) {
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0;
    const size_t G = (size_t)nsm * kMixMinBlocks;
    return align256(2 * (size_t)A.n_entries) + align256(G * kGhostMax * 4) + align256(G * 4) + 256;
}

}  // namespace

extern "C" int nbg_spmv_bsr_mixed(const nbg_bsr_t* A, const float* ph, const float* pl,
                                  float* wh, float* wl, void* stream) {
    if (!A || !A->b32 || !A->blo || !A->bxt || !ph || !pl || !wh || !wl) return NBG_ERR_ARG;
    if (A->perm) return NBG_ERR_ARG;  // the operator alone is for layouts in mesh order
    if (A->Nn == 0) return NBG_OK;
    MixArgs a;
    memset(&a, 0, sizeof(a));
    a.A = *A;
    a.ph = ph;
    a.pl = pl;
    a.keep_pm = keep_permille(*A);
    unsigned G = 0;
    const int rc = coop_grid((const void*)k_spmv_mixed, A->n_slices, &G, kMixThreads);
    if (rc != NBG_OK) return rc;
    k_spmv_mixed<<<G, kMixThreads, 0, (cudaStream_t)stream>>>(
        a, reinterpret_cast<float2*>(wh), reinterpret_cast<float2*>(wl));
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}



extern "C" size_t nbg_cg_mixed_workspace_bytes(uint32_t N) { return mixed_bytes(N); }

namespace {
thread_local int g_mixed_form = 0;  // form of this thread's last nbg_cg_mixed launch
}  // namespace

extern "C" int nbg_cg_mixed_last_form(void) { return g_mixed_form; }

extern "C" size_t nbg_cg_mixed_layout_workspace_bytes(const nbg_bsr_t* A) {
    return A ? mixed_bytes(A->N) + ghost_plan_bytes(*A) : 0;
}

namespace {
// The ghost plan for a G-block partition of A, and the launch data of the
// ghost form when its vectors fit in shared memory at one block per SM:
// returns 1 and fills gh and *dyn, or 0 (the caller keeps the global-gather
// form).  plan: the workspace region of ghost_plan_bytes(A).
int ghost_setup(const nbg_bsr_t& A, unsigned G, char* plan, cudaStream_t s, GhostArgs* gh,
                size_t* dyn) {
    if (!NBG_MIXED_RESIDENT) return 0;
    uint16_t* lcol = (uint16_t*)plan;
    uint32_t* ids = (uint32_t*)(plan + align256(2 * (size_t)A.n_entries));
    uint32_t* count = ids + (size_t)G * kGhostMax;
    int* fail = (int*)((char*)count + align256((size_t)G * 4));
    int dev = 0, nsm = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess)
        return 0;
    if (G > (unsigned)nsm * kMixMinBlocks) return 0;  // beyond the plan's space
    if (cudaFuncSetAttribute((const void*)k_ghost_plan,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(kGhostKeys * 4)) != cudaSuccess)
        return 0;
    if (cudaMemsetAsync(fail, 0, sizeof(int), s) != cudaSuccess) return 0;
    k_ghost_plan<<<G, 1024, kGhostKeys * 4, s>>>(A, lcol, ids, count, fail);
    if (cudaGetLastError() != cudaSuccess) return 0;
    std::vector<uint32_t> cnt(G);
    int hfail = 1;
    if (cudaMemcpyAsync(cnt.data(), count, 4 * (size_t)G, cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaMemcpyAsync(&hfail, fail, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess || hfail)
        return 0;
    uint32_t scap = 0, pcap = 0, gcap = 0;
    for (unsigned b = 0; b < G; b++) {
        const uint32_t s0 = (uint32_t)(((uint64_t)A.n_slices * b) / G);
        const uint32_t s1 = (uint32_t)(((uint64_t)A.n_slices * (b + 1)) / G);
        scap = std::max(scap, 32 * (s1 - s0));
        pcap = std::max(pcap, 32 * (s1 - s0) + cnt[b]);
        gcap = std::max(gcap, cnt[b]);
    }
    const size_t bytes = 16 * (size_t)pcap + 16 * (size_t)scap + 4 * (size_t)gcap +
                         (NBG_MIXED_SO_SMEM ? 4 * ((size_t)scap / 32 + 1) : 0);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, (const void*)k_cg_mixed_ghost) != cudaSuccess ||
        bytes + fa.sharedSizeBytes > (size_t)optin)
        return 0;
    if (cudaFuncSetAttribute((const void*)k_cg_mixed_ghost,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
        cudaSuccess)
        return 0;
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void*)k_cg_mixed_ghost,
                                                      kMixThreads, bytes) != cudaSuccess ||
        (unsigned)occ * (unsigned)nsm < G)
        return 0;
    gh->lcol = lcol;
    gh->ids = ids;
    gh->count = count;
    gh->scap = scap;
    gh->pcap = pcap;
    gh->gcap = gcap;
    *dyn = bytes;
    return 1;
}
}  // namespace

extern "C" int nbg_cg_mixed(const nbg_bsr_t* A, const double* b, double* x, uint32_t max_iter,
                            double tol, double delta, unsigned flags, nbg_mixed_result_t* result,
                            void* ws, size_t ws_bytes, void* stream) {
    if (!result || !A) return NBG_ERR_ARG;
    *result = nbg_mixed_result_t{0, 0, 0, 0.0, 0.0};
    if (A->Nn == 0) return NBG_OK;
    if (!A->b64 || !A->b32 || !A->blo || !A->bxt || !A->dinv32 || !(delta > 0.0 && delta < 1.0))
        return NBG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t need = mixed_bytes(A->N), plan_bytes = ghost_plan_bytes(*A);
    void* own = nullptr;
    if (!ws) {
        NBG_CHECK(cudaMalloc(&own, need + plan_bytes));
        ws = own;
        ws_bytes = need + plan_bytes;
    } else if (ws_bytes < need) {
        return NBG_ERR_ARG;
    }
    char* base = (char*)ws;
    // the ghost form when the workspace holds its plan
    char* const plan = plan_bytes && ws_bytes >= need + plan_bytes ? base + need : nullptr;
    const size_t f = align256((size_t)A->N * 4), h = align256((size_t)A->N * 4);
    MixArgs a;
    a.A = *A;
    a.b = b;
    a.u = x;
    carve_vectors(a, base, A->N);
    Group g;
    g.part = (double*)(base + 6 * f + 2 * h);
    char* tail = base + 6 * f + 2 * h + align256(kMaxBlocks * 6 * 8);
    g.bar = (unsigned*)tail;
    g.status = (int*)(tail + 256);
    g.res = (double*)(tail + 512);
    a.max_iter = max_iter;
    a.tol = tol;
    a.delta = delta;
    a.flags = flags;
    a.keep_pm = keep_permille(*A);
    int rc = NBG_OK;
    unsigned G = 1;
    size_t dyn = 0;
    double hr[5] = {0, 0, 0, 0, 0};
    cudaError_t e = cudaMemsetAsync(tail, 0, 3 * 256, s);
    if (A->perm) {  // solve in the layout's node order
        double* bp = (double*)(base + mixed_core_bytes(A->N));
        double* xp = bp + align256((size_t)A->N * 8) / 8;
        if (e == cudaSuccess) e = perm_gather(A->Nn, A->perm, b, bp, s);
        if (e == cudaSuccess) e = perm_gather(A->Nn, A->perm, (const double*)x, xp, s);
        a.b = bp;
        a.u = xp;
    }
    GhostArgs gh;
    memset(&gh, 0, sizeof(gh));
    bool ghost = false;
    if (e == cudaSuccess && plan) {
        // one block per SM, as the resident global-gather form's first choice
        int dev = 0, nsm = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess) {
            const unsigned want = (A->n_slices + kMixThreads / 32 - 1) / (kMixThreads / 32);
            G = std::max(1u, std::min((unsigned)nsm * kMixMinBlocks, want));
            ghost = ghost_setup(*A, G, plan, s, &gh, &dyn) == 1;
        }
        (void)cudaGetLastError();  // a plan that could not run leaves the global-gather form
    }
    if (e == cudaSuccess && !ghost)
        rc = coop_grid_resident((const void*)k_cg_mixed<true>, A->n_slices,
                                NBG_MIXED_RESIDENT ? kOwnNodeBytes * 32 : 0, &G, &dyn, kMixThreads,
                                kMixMinBlocks);
    if (e == cudaSuccess && rc == NBG_OK && !ghost && dyn == 0)
        rc = coop_grid((const void*)k_cg_mixed<false>, A->n_slices, &G, kMixThreads);
    a.resident = dyn > 0;
    const void* fn = ghost ? (const void*)k_cg_mixed_ghost
                           : a.resident ? (const void*)k_cg_mixed<true>
                                        : (const void*)k_cg_mixed<false>;
    g.s_begin = 0;
    g.s_end = A->n_slices;
    g.g_base = 0;
    g.g_size = G;
    g.pstride = kMaxBlocks;
    if (ghost) a.keep_pm = keep_permille(*A, 30.0);
    g_mixed_form = ghost ? NBG_MIXED_GHOST : a.resident ? NBG_MIXED_RESIDENT_ROWS
                                                       : NBG_MIXED_GLOBAL_ROWS;
    if (e == cudaSuccess && rc == NBG_OK) {
        void* args[] = {&a, &g, &gh};
        e = cudaLaunchCooperativeKernel(fn, dim3(G), dim3(kMixThreads),
                                        args, dyn, s);
        if (e == cudaSuccess && A->perm) e = perm_scatter(A->Nn, A->perm, (const double*)a.u, x, s);
    }
    if (e == cudaSuccess && rc == NBG_OK)
        e = cudaMemcpyAsync(hr, g.res, sizeof(hr), cudaMemcpyDeviceToHost, s);
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

// ------------------------------------------------------------------ batch
// Many independent systems stored as one block-diagonal layout (each
// system's node rows start on a slice boundary) and solved by one
// cooperative launch of k_cg_mixed_many, replayed as a CUDA graph together
// with zeroing x and, optionally, the SIMP compliance sensitivities.

struct nbg_mixed_batch {
    nbg_bsr_t A;
    const double* b;
    double* x;
    uint32_t n_sys;
    std::vector<uint32_t> slice_ptr, blocks;
    uint32_t max_iter;
    double tol, delta, gamma;
    unsigned flags;
    cudaStream_t stream;
    void* ws;
    MixArgs args;  // settings shared by every system
    Group* d_groups;
    uint32_t* d_map;
    double* d_res;
    unsigned char* d_state;
    unsigned G;
    size_t dyn;
    // compliance sensitivities after the solve (a = b = x)
    bool sens;
    uint32_t nen, N_elem;
    const double* nod;
    const uint32_t* conn;
    const double* rho;
    double* dJ;
    double nu, thickness, penal, E0, Emin;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
};

namespace {

constexpr size_t kStateStride = 256;  // per system: barrier at +0, status at +128
constexpr size_t kResStride = 8;      // doubles of result per system

size_t batch_bytes(uint32_t N, uint32_t n_sys) {
    return mixed_bytes(N) + align256((size_t)n_sys * kStateStride) +
           align256((size_t)n_sys * kResStride * 8) + align256((size_t)n_sys * sizeof(Group)) +
           align256((size_t)kMaxBlocks * 4);
}

// Vector slots of the workspace shared by every system (indexed by the
// global node row).
void bind_vectors(MixArgs& a, char* base, uint32_t N) { carve_vectors(a, base, N); }

double* part_slots(char* base, uint32_t N) {
    const size_t f = align256((size_t)N * 4), h = align256((size_t)N * 4);
    return (double*)(base + 6 * f + 2 * h);
}

// Blocks per system: one each, then one at a time to the system with the
// largest weight per block (weight = slices^gamma), never more blocks than
// warps of slices.  Minimises the largest weight per block.
void share_blocks(const std::vector<uint32_t>& sp, double gamma, unsigned total,
                  std::vector<uint32_t>& out) {
    const size_t n = sp.size() - 1;
    const uint32_t nw = kBatThreads / 32;
    std::vector<double> w(n);
    std::vector<uint32_t> cap(n);
    out.assign(n, 1);
    for (size_t i = 0; i < n; i++) {
        const uint32_t S = sp[i + 1] - sp[i];
        w[i] = std::pow((double)std::max<uint32_t>(S, 1), gamma);
        cap[i] = std::max<uint32_t>(1, (S + nw - 1) / nw);
    }
    for (unsigned left = total - (unsigned)n; left > 0; --left) {
        size_t best = n;
        double bw = -1.0;
        for (size_t i = 0; i < n; i++)
            if (out[i] < cap[i] && w[i] / out[i] > bw) {
                bw = w[i] / out[i];
                best = i;
            }
        if (best == n) break;
        out[best]++;
    }
}

uint32_t max_slices_per_block(const std::vector<uint32_t>& sp, const std::vector<uint32_t>& bl) {
    uint32_t m = 0;
    for (size_t i = 0; i + 1 < sp.size(); i++)
        m = std::max(m, (sp[i + 1] - sp[i] + bl[i] - 1) / bl[i]);
    return m;
}

inline int cu(cudaError_t e) { return e == cudaSuccess ? NBG_OK : nbg_cuda_error(e); }

void drop_graph(nbg_mixed_batch* m) {
    if (m->exec) cudaGraphExecDestroy(m->exec);
    if (m->graph) cudaGraphDestroy(m->graph);
    m->exec = nullptr;
    m->graph = nullptr;
}

// Block shares, launch size and the per-system argument table for `gamma`.
int batch_plan(nbg_mixed_batch* m, double gamma) {
    const void* fn = (const void*)k_cg_mixed_many<true>;
    int dev = 0, nsm = 0, optin = 0;
    NBG_CHECK(cudaGetDevice(&dev));
    NBG_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    NBG_CHECK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    NBG_CHECK(cudaFuncGetAttributes(&fa, fn));
    const uint32_t n = m->n_sys;
    std::vector<uint32_t> bl;
    unsigned G = 0;
    size_t dyn = 0;
    // own rows in shared memory when every block's rows fit
    for (int per_sm = kBatMinBlocks; NBG_MIXED_RESIDENT && per_sm >= 1 && !G; --per_sm) {
        const unsigned total = std::min<unsigned>((unsigned)nsm * per_sm, kMaxBlocks);
        if (n > total) break;
        share_blocks(m->slice_ptr, gamma, total, bl);
        const size_t bytes = (size_t)max_slices_per_block(m->slice_ptr, bl) * kOwnNodeBytes * 32;
        if (bytes + fa.sharedSizeBytes > (size_t)optin) continue;
        NBG_CHECK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        int occ = 0;
        NBG_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kBatThreads, bytes));
        unsigned used = 0;
        for (uint32_t v : bl) used += v;
        if ((unsigned)occ * (unsigned)nsm >= used) {
            G = used;
            dyn = bytes;
        }
    }
    if (!G) {
        fn = (const void*)k_cg_mixed_many<false>;
        int occ = 0;
        NBG_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kBatThreads, 0));
        const unsigned total = std::min<unsigned>((unsigned)nsm * (unsigned)std::max(occ, 1), kMaxBlocks);
        if (n > total) return NBG_ERR_ARG;  // every system needs a co-resident block
        share_blocks(m->slice_ptr, gamma, total, bl);
        for (uint32_t v : bl) G += v;
        dyn = 0;
    }
    // shared settings, group table and block -> system map
    char* base = (char*)m->ws;
    MixArgs& a = m->args;
    memset(&a, 0, sizeof(a));
    a.A = m->A;
    a.b = m->b;
    a.u = m->x;
    bind_vectors(a, base, m->A.N);
    a.max_iter = m->max_iter;
    a.tol = m->tol;
    a.delta = m->delta;
    a.flags = m->flags;
    a.keep_pm = keep_permille(m->A);
    a.resident = dyn > 0;
    std::vector<Group> groups(n);
    std::vector<uint32_t> map(G);
    double* part = part_slots(base, m->A.N);
    unsigned gb = 0;
    for (uint32_t i = 0; i < n; i++) {
        Group& g = groups[i];
        g.part = part + 6 * (size_t)gb;
        g.pstride = bl[i];
        g.bar = (unsigned*)(m->d_state + i * kStateStride);
        g.status = (int*)(m->d_state + i * kStateStride + 128);
        g.res = m->d_res + i * kResStride;
        g.s_begin = m->slice_ptr[i];
        g.s_end = m->slice_ptr[i + 1];
        g.g_base = gb;
        g.g_size = bl[i];
        for (uint32_t k = 0; k < bl[i]; k++) map[gb + k] = i;
        gb += bl[i];
    }
    NBG_CHECK(cudaMemcpy(m->d_groups, groups.data(), n * sizeof(Group), cudaMemcpyHostToDevice));
    NBG_CHECK(cudaMemcpy(m->d_map, map.data(), G * 4, cudaMemcpyHostToDevice));
    m->blocks = bl;
    m->G = G;
    m->dyn = dyn;
    m->gamma = gamma;
    drop_graph(m);
    return NBG_OK;
}

// The work of one batch launch, enqueued on s (captured into the graph).
cudaError_t batch_enqueue(nbg_mixed_batch* m, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(m->x, 0, 8 * (size_t)m->A.N, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->d_state, 0, (size_t)m->n_sys * kStateStride, s);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(m->G);
    cfg.blockDim = dim3(kBatThreads);
    cfg.dynamicSmemBytes = m->dyn;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const Group* groups = m->d_groups;
    const uint32_t* map = m->d_map;
    e = m->args.resident ? cudaLaunchKernelEx(&cfg, k_cg_mixed_many<true>, m->args, groups, map)
                         : cudaLaunchKernelEx(&cfg, k_cg_mixed_many<false>, m->args, groups, map);
    if (e != cudaSuccess || !m->sens) return e;
    const int rc = nbg_simp_sensitivity_f64(m->nen, m->N_elem, m->nod, m->conn, m->nu,
                                            m->thickness, m->rho, m->penal, m->E0, m->Emin, m->x,
                                            m->x, m->dJ, s);
    return rc == NBG_OK ? cudaSuccess : cudaErrorLaunchFailure;
}

// The function attribute is shared by every batch in the process: set it
// to this batch's size before capturing and before each replay.
int set_smem(const nbg_mixed_batch* m) {
    if (m->args.resident)
        NBG_CHECK(cudaFuncSetAttribute((const void*)k_cg_mixed_many<true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)m->dyn));
    return NBG_OK;
}

int build_graph(nbg_mixed_batch* m) {
    const int rc = set_smem(m);
    if (rc != NBG_OK) return rc;
    cudaStream_t cap;
    NBG_CHECK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const cudaError_t e1 = batch_enqueue(m, cap);
        cudaGraph_t g = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(cap, &g);
        e = e1 != cudaSuccess ? e1 : e2;
        if (e == cudaSuccess) {
            m->graph = g;
            e = cudaGraphInstantiate(&m->exec, g, 0);
        } else if (g) {
            cudaGraphDestroy(g);
        }
    }
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) {
        drop_graph(m);
        return nbg_cuda_error(e);
    }
    return NBG_OK;
}

}  // namespace

extern "C" int nbg_mixed_batch_create(nbg_mixed_batch_t** out, const nbg_bsr_t* A,
                                      const double* b, double* x, uint32_t n_sys,
                                      const uint32_t* slice_ptr, uint32_t max_iter, double tol,
                                      double delta, unsigned flags, void* stream) {
    if (!out || !A || A->perm) return NBG_ERR_ARG;  // instances own contiguous slices
    *out = nullptr;
    if (!A || !b || !x || !slice_ptr || n_sys == 0 || n_sys > kMaxBlocks || !A->b64 ||
        !A->b32 || !A->blo || !A->bxt || !A->dinv32 || !(delta > 0.0 && delta < 1.0))
        return NBG_ERR_ARG;
    if (slice_ptr[0] != 0 || slice_ptr[n_sys] != A->n_slices) return NBG_ERR_ARG;
    for (uint32_t i = 0; i < n_sys; i++)
        if (slice_ptr[i + 1] < slice_ptr[i]) return NBG_ERR_ARG;
    nbg_mixed_batch* m = new (std::nothrow) nbg_mixed_batch();
    if (!m) return NBG_ERR_NOMEM;
    m->A = *A;
    m->b = b;
    m->x = x;
    m->n_sys = n_sys;
    m->slice_ptr.assign(slice_ptr, slice_ptr + n_sys + 1);
    m->max_iter = max_iter;
    m->tol = tol;
    m->delta = delta;
    m->flags = flags;
    m->stream = (cudaStream_t)stream;
    const size_t need = batch_bytes(A->N, n_sys);
    cudaError_t e = cudaMalloc(&m->ws, need);
    if (e != cudaSuccess) {
        delete m;
        return nbg_cuda_error(e);
    }
    char* p = (char*)m->ws + mixed_bytes(A->N);
    m->d_state = (unsigned char*)p;
    p += align256((size_t)n_sys * kStateStride);
    m->d_res = (double*)p;
    p += align256((size_t)n_sys * kResStride * 8);
    m->d_groups = (Group*)p;
    p += align256((size_t)n_sys * sizeof(Group));
    m->d_map = (uint32_t*)p;
    int rc = batch_plan(m, 1.0);
    if (rc != NBG_OK) {
        nbg_mixed_batch_destroy(m);
        return rc;
    }
    *out = m;
    return NBG_OK;
}

extern "C" void nbg_mixed_batch_destroy(nbg_mixed_batch_t* m) {
    if (!m) return;
    drop_graph(m);
    if (m->ws) cudaFree(m->ws);
    delete m;
}

extern "C" int nbg_mixed_batch_plan(nbg_mixed_batch_t* m, double gamma) {
    if (!m || !(gamma >= 0.0 && gamma <= 4.0)) return NBG_ERR_ARG;
    return batch_plan(m, gamma);
}

extern "C" uint32_t nbg_mixed_batch_blocks(const nbg_mixed_batch_t* m, uint32_t* blocks,
                                           double* gamma) {
    if (!m) return 0;
    if (blocks) std::copy(m->blocks.begin(), m->blocks.end(), blocks);
    if (gamma) *gamma = m->gamma;
    return m->G;
}

extern "C" int nbg_mixed_batch_set_sensitivity(nbg_mixed_batch_t* m, uint32_t nen,
                                               uint32_t N_elem, const double* nod,
                                               const uint32_t* conn, double nu, double thickness,
                                               const double* rho, double penal, double E0,
                                               double Emin, double* dJ) {
    if (!m || (nen != 3 && nen != 4) || (N_elem && (!nod || !conn || !rho || !dJ)))
        return NBG_ERR_ARG;
    m->sens = N_elem > 0;
    m->nen = nen;
    m->N_elem = N_elem;
    m->nod = nod;
    m->conn = conn;
    m->nu = nu;
    m->thickness = thickness;
    m->rho = rho;
    m->penal = penal;
    m->E0 = E0;
    m->Emin = Emin;
    m->dJ = dJ;
    drop_graph(m);
    return NBG_OK;
}

extern "C" int nbg_mixed_batch_launch(nbg_mixed_batch_t* m) {
    if (!m) return NBG_ERR_ARG;
    const int rc = m->exec ? set_smem(m) : build_graph(m);
    if (rc != NBG_OK) return rc;
    NBG_CHECK(cudaGraphLaunch(m->exec, m->stream));
    return NBG_OK;
}

extern "C" int nbg_mixed_batch_results(nbg_mixed_batch_t* m, nbg_mixed_result_t* res,
                                       double* J) {
    if (!m) return NBG_ERR_ARG;
    std::vector<double> h((size_t)m->n_sys * kResStride);
    NBG_CHECK(cudaMemcpyAsync(h.data(), m->d_res, h.size() * 8, cudaMemcpyDeviceToHost,
                              m->stream));
    NBG_CHECK(cudaStreamSynchronize(m->stream));
    int worst = NBG_OK;
    for (uint32_t i = 0; i < m->n_sys; i++) {
        const double* r = &h[(size_t)i * kResStride];
        nbg_mixed_result_t t;
        t.niter = (uint32_t)r[0];
        t.n_updates = (uint32_t)r[1];
        t.status = (int)r[2];
        t.bnorm = std::sqrt(r[4]);
        t.relres = r[4] > 0 ? std::sqrt(r[3] / r[4]) : std::sqrt(r[3]);
        if (res) res[i] = t;
        if (J) J[i] = r[5];
        if (t.status < 0 && worst >= 0) worst = t.status;
        else if (t.status > 0 && worst == NBG_OK) worst = t.status;
    }
    return worst;
}

extern "C" int nbg_mixed_batch_tune(nbg_mixed_batch_t* m, uint32_t n_cand, const double* gammas,
                                    double* ms) {
    if (!m || !n_cand || !gammas) return NBG_ERR_ARG;
    cudaEvent_t t0, t1;
    NBG_CHECK(cudaEventCreate(&t0));
    NBG_CHECK(cudaEventCreate(&t1));
    int rc = NBG_OK;
    double best_ms = 0.0, best_g = gammas[0];
    for (uint32_t c = 0; c < n_cand && rc == NBG_OK; c++) {
        rc = nbg_mixed_batch_plan(m, gammas[c]);
        if (rc == NBG_OK) rc = nbg_mixed_batch_launch(m);  // builds the graph, warms up
        if (rc == NBG_OK) rc = cu(cudaEventRecord(t0, m->stream));
        if (rc == NBG_OK) rc = nbg_mixed_batch_launch(m);
        if (rc == NBG_OK) rc = cu(cudaEventRecord(t1, m->stream));
        if (rc == NBG_OK) rc = cu(cudaEventSynchronize(t1));
        float t = 0.f;
        if (rc == NBG_OK) rc = cu(cudaEventElapsedTime(&t, t0, t1));
        if (rc == NBG_OK) {
            const int st = nbg_mixed_batch_results(m, nullptr, nullptr);
            if (st < 0) rc = st;
        }
        if (ms) ms[c] = t;
        if (rc == NBG_OK && (c == 0 || t < best_ms)) {
            best_ms = t;
            best_g = gammas[c];
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (rc != NBG_OK) return rc;
    return nbg_mixed_batch_plan(m, best_g);
}
