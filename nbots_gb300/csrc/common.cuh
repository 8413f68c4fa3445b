// Shared device helpers for the nbots GB300 kernels.
//
//  * exact FP64 helpers: nbots is built with -std=c99, i.e. GCC's
//    -ffp-contract=off (CMakeLists.txt:33), so every product is rounded
//    before it is added.  The parity kernels spell each operation with the
//    _rn intrinsics, which nvcc never contracts into an FMA.
//  * a bounded grid barrier for cooperative (co-resident) launches: every
//    spin has a time limit; on expiry the kernel records NBG_ERR_TIMEOUT in
//    a device status word and all blocks leave their loops.
//  * fixed-order block reductions, so every run produces the same bits.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "nbots_gb300.h"

#define NBG_CHECK(call)                                            \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return nbg_cuda_error(e_);          \
    } while (0)

int nbg_cuda_error(cudaError_t e);
// Records `text` as the thread's last error message and returns `code`.
int nbg_error_text(int code, const char* text);

namespace nbg {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

__device__ __forceinline__ uint64_t globaltimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }

// Spin limit of every device-side wait (nanoseconds of %globaltimer).
constexpr uint64_t kSpinLimitNs = 2000000000ull;

// L2 eviction priority for streamed loads.  An iterative solver re-reads
// the same matrix every iteration; when it is about as large as L2, plain
// loads evict it in LRU order and every pass comes from HBM.  Marking a
// fixed part of it evict_last (and the rest evict_first) keeps that part in
// L2 from one iteration to the next.
__device__ __forceinline__ uint64_t l2_policy(bool keep) {
    uint64_t p;
    if (keep)
        asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    else
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ float4 ld_hint(const float4* a, uint64_t pol) {
    float4 v;
    asm volatile("ld.global.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(a), "l"(pol));
    return v;
}

__device__ __forceinline__ double2 ld_hint(const double2* a, uint64_t pol) {
    double2 v;
    asm volatile("ld.global.L2::cache_hint.v2.f64 {%0,%1}, [%2], %3;"
                 : "=d"(v.x), "=d"(v.y)
                 : "l"(a), "l"(pol));
    return v;
}

__device__ __forceinline__ uint2 ld_hint(const uint2* a, uint64_t pol) {
    uint2 v;
    asm volatile("ld.global.L2::cache_hint.v2.u32 {%0,%1}, [%2], %3;"
                 : "=r"(v.x), "=r"(v.y)
                 : "l"(a), "l"(pol));
    return v;
}

__device__ __forceinline__ uint32_t ld_hint(const uint16_t* a, uint64_t pol) {
    unsigned short v;
    asm volatile("ld.global.L2::cache_hint.u16 %0, [%1], %2;" : "=h"(v) : "l"(a), "l"(pol));
    return v;
}

__device__ __forceinline__ uint32_t ld_hint(const uint32_t* a, uint64_t pol) {
    uint32_t v;
    asm volatile("ld.global.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
    return v;
}

// Barrier over the `nblocks` co-resident blocks of a group (the whole grid,
// or one system of a batched launch), one arrival word *bar (zero at launch).
// Thread 0 of the block of rank 0 adds 2^31 - (nblocks - 1), every other
// block adds 1, each with one release atomic; the word has then grown by
// exactly 2^31 once all have arrived, so each block waits (acquire loads)
// for bit 31 to differ from the value its own atomic returned.  No reset is
// needed between barriers.  Requires co-residency (cooperative launch).
// Split in two so that a block can do work that needs no other block's
// data between its arrival and its wait.  The wait is bounded
// (kSpinLimitNs, checked every 64 polls).  barrier_wait returns nonzero when
// the caller must stop (timeout here or an error recorded by another block).
__device__ __forceinline__ unsigned barrier_arrive(unsigned* bar, unsigned nblocks,
                                                   unsigned rank) {
    __syncthreads();
    unsigned old = 0;
    if (threadIdx.x == 0) {
        const unsigned add = rank == 0 ? 0x80000000u - (nblocks - 1) : 1u;
        asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;"
                     : "=r"(old)
                     : "l"(bar), "r"(add)
                     : "memory");
    }
    return old;  // meaningful in thread 0
}

__device__ __forceinline__ int barrier_wait(unsigned* bar, unsigned old, int* status) {
    __shared__ int s_stop;
    if (threadIdx.x == 0) {
        int stop = 0;
        uint64_t t0 = 0;
        for (unsigned it = 0;; it++) {
            if ((ld_acquire(bar) ^ old) & 0x80000000u) break;
            if ((it & 63u) == 0) {
                const uint64_t t = globaltimer();
                if (it == 0) {
                    t0 = t;
                } else if (t - t0 > kSpinLimitNs) {
                    atomicCAS(status, 0, NBG_ERR_TIMEOUT);
                    stop = 1;
                    break;
                }
            }
        }
        if (!stop && ld_volatile(status) != 0) stop = 1;
        s_stop = stop;
    }
    __syncthreads();
    return s_stop;
}

__device__ __forceinline__ int grid_barrier(unsigned* bar, unsigned nblocks, unsigned rank,
                                            int* status) {
    const unsigned old = barrier_arrive(bar, nblocks, rank);
    return barrier_wait(bar, old, status);
}

// Counting form of the same barrier: every block adds 1 per barrier with a
// release reduction that returns nothing (no round trip before the first
// poll) and waits, with acquire loads, until the word reaches nblocks times
// the number of barriers it has passed, which each thread keeps in
// `target` (zero at the start; every block of the group passes the same
// barriers).  The word is zero at launch.  Bounded as barrier_wait.
__device__ __forceinline__ int grid_barrier_count(unsigned* bar, unsigned nblocks,
                                                  unsigned& target, int* status) {
    __shared__ int s_stop;
    __syncthreads();
    target += nblocks;
    if (threadIdx.x == 0) {
        asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(bar), "r"(1u) : "memory");
        int stop = 0;
        uint64_t t0 = 0;
        for (unsigned it = 0;; it++) {
            if ((int)(ld_acquire(bar) - target) >= 0) break;
            if ((it & 63u) == 0) {
                const uint64_t t = globaltimer();
                if (it == 0) {
                    t0 = t;
                } else if (t - t0 > kSpinLimitNs) {
                    atomicCAS(status, 0, NBG_ERR_TIMEOUT);
                    stop = 1;
                    break;
                }
            }
        }
        if (!stop && ld_volatile(status) != 0) stop = 1;
        s_stop = stop;
    }
    __syncthreads();
    return s_stop;
}

// Block-wide sum of NV values per thread, fixed tree order.  Result valid in
// thread 0.  `scratch` holds NV * 32 doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] = add(v[k], __shfl_down_sync(0xffffffffu, v[k], o));
    }
    __syncthreads();
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) scratch[k * 32 + warp] = v[k];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = lane < nwarps ? scratch[k * 32 + lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s = add(s, __shfl_down_sync(0xffffffffu, s, o));
            v[k] = s;
        }
    }
}

// Float flavour with Kahan-compensated accumulation carried as (sum, comp).
struct Kahan {
    float s, c;
    __device__ __forceinline__ void add(float x) {
        float y = __fsub_rn(x, c);
        float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// Float-float (unevaluated sum hi + lo of two FP32 numbers) built from the
// classic error-free transformations: Knuth's TwoSum, Dekker's FastTwoSum
// and the FMA form of TwoProduct.  Every step is spelled with _rn
// intrinsics so no contraction or reassociation can break them.
struct FF {
    float hi, lo;
};

__device__ __forceinline__ FF two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ FF fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ FF two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

// Accumulator for sum_k (a_hi + a_lo)(x_hi + x_lo): the a_lo x_lo term is
// below the working precision and dropped.
struct FFAcc {
    float s, c;
    __device__ __forceinline__ void fma2(float ahi, float alo, float xhi, float xlo) {
        FF p = two_prod(ahi, xhi);
        float e = __fmaf_rn(ahi, xlo, p.lo);
        e = __fmaf_rn(alo, xhi, e);
        FF t = two_sum(s, p.hi);
        s = t.hi;
        c = __fadd_rn(c, __fadd_rn(t.lo, e));
    }
    // (ahi + s ahi)(xhi + xlo) with the remainder given by its scale s
    // (rem23_scale): the term s ahi xhi uses the rounded product ahi xhi.
    __device__ __forceinline__ void fma2s(float ahi, float sc, float xhi, float xlo) {
        FF p = two_prod(ahi, xhi);
        float e = __fmaf_rn(ahi, xlo, p.lo);
        e = __fmaf_rn(sc, p.hi, e);
        FF t = two_sum(s, p.hi);
        s = t.hi;
        c = __fadd_rn(c, __fadd_rn(t.lo, e));
    }
    __device__ __forceinline__ FF result() const { return fast_two_sum(s, c); }
};

// Two accumulators of FFAcc::fma2s side by side (the two rows of a 2x2
// block, one column at a time), on Blackwell's packed FP32x2 instructions:
// each component takes the same roundings as FFAcc, so the sums are the
// same bits, with half the instructions.
struct FFAcc2 {
    float2 s, c;
    __device__ __forceinline__ static float2 neg(float2 v) { return make_float2(-v.x, -v.y); }
    // (a + sc a)(x + xl) for the column a of a block, its remainder scales
    // sc and the entry x + xl of the vector
    __device__ __forceinline__ void fma2s(float2 a, float2 sc, float x, float xl) {
        const float2 xx = make_float2(x, x), xxl = make_float2(xl, xl);
        const float2 p = __fmul2_rn(a, xx);
        float2 e = __ffma2_rn(a, xx, neg(p));
        e = __ffma2_rn(a, xxl, e);
        e = __ffma2_rn(sc, p, e);
        const float2 t = __fadd2_rn(s, p);
        const float2 bb = __fadd2_rn(t, neg(s));
        const float2 err =
            __fadd2_rn(__fadd2_rn(s, neg(__fadd2_rn(t, neg(bb)))), __fadd2_rn(p, neg(bb)));
        s = t;
        c = __fadd2_rn(c, __fadd2_rn(err, e));
    }
};

__device__ __forceinline__ FF ff_from_double(double d) {
    const float h = (float)d;
    return {h, (float)(d - (double)h)};
}

// a + b for float-float operands
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    FF s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

// Remainder a - hi of an FP32 rounding hi = fl(a), stored as the biased
// count c = q + 2^22 of units of 2^-46 hi (|a - hi| <= 2^-24 |hi|, so
// |q| <= 2^22, clamped to 2^22 - 1): its low 16 bits in one array (blo),
// its high 7 bits in a byte of another (bxt).  hi + lo then carries about
// 47 significant bits in 7 bytes.  With 16-bit counts (about 40 bits) the
// iteration counts matched FP64 but the mixed solution kept an error of
// 1e-8 to 1e-7 in the smooth modes that its residual barely sees (a CPU
// emulation of the solver on the same cantilever: 1.3e-8 at 512x256,
// 4.9e-10 with 20-bit counts, 3.1e-10 with these, FP64's 3.1e-10).
// Decoding needs no conversion instruction: c placed in the mantissa of a
// float with exponent -23 is 2^-23 + c 2^-46, and subtracting
// 2^-23 + 2^-24 (exact: both within one binade) leaves s = q 2^-46, with
// lo = s hi.
__device__ __forceinline__ uint32_t rem23_encode(double a, float hi) {
    if (hi == 0.f) return 1u << 22;
    double q = rint((a - (double)hi) / ((double)hi * 0x1p-46));
    const double lim = (double)((1 << 22) - 1);
    q = q > lim ? lim : (q < -lim ? -lim : q);
    return (uint32_t)((int)q + (1 << 22));
}

// s = q 2^-46 for the count whose low 16 bits are bytes j0, j0 + 1 of lo and
// whose high 7 bits are byte 4 + jx of {lo, ext} (prmt numbering): one byte
// permute, one logic operation and one subtraction.
template <uint32_t kSel>
__device__ __forceinline__ float rem23_scale(uint32_t lo, uint32_t ext) {
    uint32_t t;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(t) : "r"(lo), "r"(ext), "n"(kSel));
    // byte 3: sign 0 and the exponent's top 7 bits (-23 + 127 = 0x68)
    return __fsub_rn(__uint_as_float((t & 0x00FFFFFFu) | 0x34000000u), 0x1.8p-23f);
}

// The four scales of one 2x2 block: the low halves packed two per word of
// lo, the high parts one per byte of ext.
__device__ __forceinline__ float4 rem23_scale4(uint2 lo, uint32_t ext) {
    return make_float4(rem23_scale<0x0410>(lo.x, ext), rem23_scale<0x0532>(lo.x, ext),
                       rem23_scale<0x0610>(lo.y, ext), rem23_scale<0x0732>(lo.y, ext));
}

// a * b, both float-float
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
    FF p = two_prod(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.lo, p.lo);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p.hi, e);
}

// a * b for a float-float a and an FP32 b
__device__ __forceinline__ FF ff_mulf(FF a, float b) {
    const FF p = two_prod(a.hi, b);
    return fast_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}

// Pairs of float-float numbers (the two dofs of a node row) on the packed
// FP32x2 instructions, each component rounded as ff_add, ff_mul and
// ff_mulf round it.
struct FF2 {
    float2 hi, lo;
};

__device__ __forceinline__ float2 f2neg(float2 v) { return make_float2(-v.x, -v.y); }

__device__ __forceinline__ FF2 two_sum2(float2 a, float2 b) {
    const float2 s = __fadd2_rn(a, b);
    const float2 bb = __fadd2_rn(s, f2neg(a));
    return {s, __fadd2_rn(__fadd2_rn(a, f2neg(__fadd2_rn(s, f2neg(bb)))),
                          __fadd2_rn(b, f2neg(bb)))};
}

__device__ __forceinline__ FF2 fast_two_sum2(float2 a, float2 b) {
    const float2 s = __fadd2_rn(a, b);
    return {s, __fadd2_rn(b, f2neg(__fadd2_rn(s, f2neg(a))))};
}

__device__ __forceinline__ FF2 ff2_add(FF2 a, FF2 b) {
    const FF2 s = two_sum2(a.hi, b.hi);
    return fast_two_sum2(s.hi, __fadd2_rn(s.lo, __fadd2_rn(a.lo, b.lo)));
}

// a * b with one float-float a for both components (a given as pairs
// {a.hi, a.hi}, {a.lo, a.lo})
__device__ __forceinline__ FF2 ff2_mul(FF2 a, FF2 b) {
    const float2 p = __fmul2_rn(a.hi, b.hi);
    float2 e = __ffma2_rn(a.hi, b.hi, f2neg(p));
    e = __ffma2_rn(a.hi, b.lo, e);
    e = __ffma2_rn(a.lo, b.hi, e);
    return fast_two_sum2(p, e);
}

__device__ __forceinline__ FF2 ff2_mulf(FF2 a, float2 b) {
    const float2 p = __fmul2_rn(a.hi, b);
    return fast_two_sum2(p, __ffma2_rn(a.lo, b, __ffma2_rn(a.hi, b, f2neg(p))));
}

__device__ __forceinline__ FF2 ff2_bcast(FF a) {
    return {make_float2(a.hi, a.hi), make_float2(a.lo, a.lo)};
}

// a / b, both float-float, by Dekker's long division (1971): the FP32
// quotient q1 of the leading parts, the remainder a - q1 b in float-float,
// and a second FP32 quotient of the remainder.  About 44 significant bits,
// all on the FP32 pipe.
__device__ __forceinline__ FF ff_div(FF a, FF b) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const FF p = ff_mul(FF{q1, 0.f}, b);
    const FF r = ff_add(a, FF{-p.hi, -p.lo});
    return fast_two_sum(q1, __fdiv_rn(r.hi, b.hi));
}

// Rows row0 .. row0 + nrows - 1 (nrows <= 32) of a CSR matrix times x in
// nbots' order (each row starts at 0 and adds its rounded products left to
// right, sparse.c:405-414), so the sums are bit-exact.  The warp stages the
// products of all its rows through `prod` (kStage doubles of this warp's
// shared memory) with coalesced loads of values and columns and independent
// gathers of x; then each lane adds its own row's products in column order
// and gets its row's sum (0 for lanes >= nrows).  All 32 lanes must call it.
template <int kStage>
__device__ __forceinline__ double warp_rows_exact(const uint32_t* __restrict__ rp,
                                                  const uint32_t* __restrict__ ci,
                                                  const double* __restrict__ v,
                                                  const double* x, uint32_t row0,
                                                  uint32_t nrows, double* prod, int lane) {
    const uint32_t k0 = rp[row0], k1 = rp[row0 + nrows];
    uint32_t mb = 0, me = 0;
    if ((uint32_t)lane < nrows) {
        mb = rp[row0 + lane];
        me = rp[row0 + lane + 1];
    }
    double s = 0.0;
    uint32_t next = mb;  // next product of this lane's row still to add
    for (uint32_t base = k0; base < k1; base += kStage) {
        const uint32_t cnt = min((uint32_t)kStage, k1 - base);
#pragma unroll 4
        for (uint32_t t = lane; t < cnt; t += 32) prod[t] = mul(v[base + t], x[ci[base + t]]);
        __syncwarp();
        const uint32_t hi = min(me, base + cnt);
        for (; next < hi; next++) s = add(s, prod[next - base]);
        __syncwarp();
    }
    return s;
}

}  // namespace nbg
