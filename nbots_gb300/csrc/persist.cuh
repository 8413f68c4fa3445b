// Helpers shared by the persistent (one cooperative launch per solve)
// solvers on the 2x2-block SELL layout: block-to-slice partition,
// fixed-order block and grid reductions, FP64 block-row SpMV, launch sizing.
#pragma once

#include <cstdint>

#include "common.cuh"

namespace nbg {

// Launch shape of the persistent solvers (overridable at build time for tuning).
#ifndef NBG_PERSIST_THREADS
#define NBG_PERSIST_THREADS 512
#endif
#ifndef NBG_PERSIST_MIN_BLOCKS
#define NBG_PERSIST_MIN_BLOCKS 2  // 64 registers per thread: 32 warps per SM
#endif
constexpr int kPersistThreads = NBG_PERSIST_THREADS;
constexpr int kPersistMinBlocks = NBG_PERSIST_MIN_BLOCKS;
constexpr unsigned kMaxBlocks = 4096;

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Contiguous, balanced slice range [s0, s1) of this block.
__device__ __forceinline__ void slice_range(uint32_t S, uint32_t& s0, uint32_t& s1) {
    s0 = (uint32_t)(((uint64_t)S * blockIdx.x) / gridDim.x);
    s1 = (uint32_t)(((uint64_t)S * (blockIdx.x + 1)) / gridDim.x);
}

// Sum over blocks of NV partials per block, in block order; every block
// computes the same bits.
template <int NV>
__device__ __forceinline__ void grid_reduce(const double* part, double* out, double* sh) {
    const unsigned G = gridDim.x;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (unsigned b = lane; b < G; b += 32) s += part[b * NV + k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if (lane == 0) sh[k] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++) out[k] = sh[k];
    __syncthreads();
}

template <int NV>
__device__ __forceinline__ void block_sum_plain(double (&v)[NV], double* scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) scratch[k * 32 + warp] = v[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = lane < nwarps ? scratch[k * 32 + lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            v[k] = s;
        }
    }
}

// Block sum, then thread 0 stores the NV results in this block's slot.
template <int NV>
__device__ __forceinline__ void publish(double (&v)[NV], double* red, double* part) {
    block_sum_plain<NV>(v, red);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) part[blockIdx.x * NV + k] = v[k];
}

// Group flavours, for launches that run independent problems side by side:
// a group is G consecutive blocks; `rank` is the block's place in it.
__device__ __forceinline__ void group_slice_range(uint32_t sb, uint32_t se, uint32_t rank,
                                                  uint32_t G, uint32_t& s0, uint32_t& s1) {
    const uint64_t S = se - sb;
    s0 = sb + (uint32_t)((S * rank) / G);
    s1 = sb + (uint32_t)((S * (rank + 1)) / G);
}

template <int NV>
__device__ __forceinline__ void group_publish(double (&v)[NV], double* red, double* part,
                                              uint32_t rank) {
    block_sum_plain<NV>(v, red);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) part[rank * NV + k] = v[k];
}

template <int NV>
__device__ __forceinline__ void group_reduce(const double* part, uint32_t G, double* out,
                                             double* sh) {
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (unsigned b = lane; b < G; b += 32) s += part[b * NV + k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if (lane == 0) sh[k] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++) out[k] = sh[k];
    __syncthreads();
}

// GB300 issues FP64 at a small fraction of its FP32 rate, so FP64 work that
// every thread repeats (a shuffle tree over 512 threads, the division for a
// step length) costs microseconds per reduction.  The helpers below keep the
// per-thread part on the FP32 pipes and leave FP64 to one warp.

// Block sum of NV float-float values per thread, error-free FP32 shuffle
// sums throughout (within each warp, then across the warps by warp 0), fixed
// order.  The result is valid in thread 0.  `scratch` holds NV * 32 FF.
template <int NV>
__device__ __forceinline__ void ff_warp_sum(FF (&v)[NV]) {
#pragma unroll
    for (int k = 0; k < NV; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float h = __shfl_down_sync(0xffffffffu, v[k].hi, o);
            const float l = __shfl_down_sync(0xffffffffu, v[k].lo, o);
            v[k] = ff_add(v[k], FF{h, l});
        }
}

template <int NV>
__device__ __forceinline__ void block_sum_ff(FF (&v)[NV], float2* scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    ff_warp_sum<NV>(v);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) scratch[k * 32 + warp] = make_float2(v[k].hi, v[k].lo);
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            const float2 t = lane < nwarps ? scratch[k * 32 + lane] : make_float2(0.f, 0.f);
            v[k] = FF{t.x, t.y};
        }
        ff_warp_sum<NV>(v);
    }
}

// Block sum, then thread 0 stores the NV float-float results in this
// block's slot of `part` (float2 per value).
template <int NV>
__device__ __forceinline__ void group_publish_ff(FF (&v)[NV], float2* scratch, float2* part,
                                                 uint32_t rank) {
    block_sum_ff<NV>(v, scratch);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) part[rank * NV + k] = make_float2(v[k].hi, v[k].lo);
}

// Sum over the group's blocks of NV float-float partials, in block order, by
// warp 0 with error-free FP32 arithmetic; the float-float result is valid in
// thread 0 only (no block synchronisation).
// Lane l adds the partials of blocks l, l + 32, ... in that order; the
// loads of kReduceBatch of them go out before the first add (one L2 round
// trip per batch instead of one per partial: 152 blocks, 5 per lane, is one
// batch).  Launches whose groups have at most 32 blocks pass 1.
constexpr int kReduceBatch = 5;

template <int NV, int kReduceBatch = kReduceBatch>
__device__ __forceinline__ void group_reduce0_ff(const float2* part, uint32_t G,
                                                 FF (&out)[NV]) {
    if (threadIdx.x < 32) {
        const uint32_t lane = threadIdx.x;
        FF v[NV];
#pragma unroll
        for (int k = 0; k < NV; k++) v[k] = FF{0.f, 0.f};
        for (uint32_t base = 0; base < G; base += 32 * kReduceBatch) {
            float2 t[kReduceBatch][NV];
#pragma unroll
            for (int j = 0; j < kReduceBatch; j++) {
                const uint32_t b = base + 32 * j + lane;
#pragma unroll
                for (int k = 0; k < NV; k++)
                    t[j][k] = b < G ? part[b * NV + k] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int j = 0; j < kReduceBatch; j++)
                if (base + 32 * j + lane < G)
#pragma unroll
                    for (int k = 0; k < NV; k++) v[k] = ff_add(v[k], FF{t[j][k].x, t[j][k].y});
        }
        ff_warp_sum<NV>(v);
#pragma unroll
        for (int k = 0; k < NV; k++) out[k] = v[k];
    }
}

// Block sum of NV FP64 values per thread with the FP64 adds done by warp 0
// alone: the partials go through shared memory (`buf` holds NV * blockDim.x
// doubles), lane l adds those of threads l, l + 32, ... in order, then a
// shuffle tree.  About a quarter of the FP64 adds of a full-block shuffle
// tree.  Result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum_f64(const double (&v)[NV], double* buf,
                                              double (&out)[NV]) {
    const int bd = blockDim.x;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++) buf[k * bd + threadIdx.x] = v[k];
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (int t = lane; t < bd; t += 32) s += buf[k * bd + t];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            out[k] = s;
        }
    }
}

// Sum over the group's blocks of NV partials, in block order, by warp 0;
// the result is valid in thread 0 only (no block synchronisation).
template <int NV>
__device__ __forceinline__ void group_reduce0(const double* part, uint32_t G, double (&out)[NV]) {
    if (threadIdx.x < 32) {
        const uint32_t lane = threadIdx.x;
        double s[NV];
#pragma unroll
        for (int k = 0; k < NV; k++) s[k] = 0.0;
        for (uint32_t base = 0; base < G; base += 32 * kReduceBatch) {
            double t[kReduceBatch][NV];
#pragma unroll
            for (int j = 0; j < kReduceBatch; j++) {
                const uint32_t b = base + 32 * j + lane;
#pragma unroll
                for (int k = 0; k < NV; k++) t[j][k] = b < G ? part[b * NV + k] : 0.0;
            }
#pragma unroll
            for (int j = 0; j < kReduceBatch; j++)
                if (base + 32 * j + lane < G)
#pragma unroll
                    for (int k = 0; k < NV; k++) s[k] += t[j][k];
        }
#pragma unroll
        for (int k = 0; k < NV; k++) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_down_sync(0xffffffffu, s[k], o);
            out[k] = s[k];
        }
    }
}

// (A x) for node row (s, lane) with FP64 values and FMAs.
__device__ __forceinline__ double2 spmv_row_f64(const nbg_bsr_t& A, uint32_t s, uint32_t lane,
                                                const double2* __restrict__ xv) {
    const double2* __restrict__ bv = reinterpret_cast<const double2*>(A.b64);
    // the 36 B/block matrix stream passes through L2 once per iteration;
    // evict_first keeps the vectors there (1M dof: 64.3 -> 62.8 us/iteration)
    const uint64_t pol = l2_policy(false);
    double y0 = 0.0, y1 = 0.0;
    const uint32_t k0 = A.slice_off[s], k1 = A.slice_off[s + 1];
#pragma unroll 3
    for (uint32_t k = k0; k < k1; k++) {
        const size_t e = (size_t)k * 32 + lane;
        const double2 xc = xv[ld_hint(A.bcol + e, pol)];
        const double2 top = ld_hint(bv + 2 * e, pol), bot = ld_hint(bv + 2 * e + 1, pol);
        y0 = fma(top.x, xc.x, y0);
        y0 = fma(top.y, xc.y, y0);
        y1 = fma(bot.x, xc.x, y1);
        y1 = fma(bot.y, xc.y, y1);
    }
    return make_double2(y0, y1);
}

// Grid size of a cooperative launch of `threads`-thread blocks: every
// co-resident block, but not more blocks than warps of slices.
inline int coop_grid(const void* fn, uint32_t n_slices, unsigned* G,
                     int threads = kPersistThreads) {
    int dev = 0, nsm = 0, occ = 0;
    NBG_CHECK(cudaGetDevice(&dev));
    NBG_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    NBG_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, 0));
    unsigned g = (unsigned)nsm * (unsigned)(occ > 0 ? occ : 1);
    const unsigned want = (n_slices + threads / 32 - 1) / (threads / 32);
    if (want < g) g = want;
    if (g < 1) g = 1;
    if (g > kMaxBlocks) g = kMaxBlocks;
    *G = g;
    return NBG_OK;
}

// Grid of a persistent kernel whose blocks keep `bytes_per_slice` of own-row
// data per slice in dynamic shared memory: the largest blocks-per-SM count
// (min_blocks, then fewer) at which every block's slices fit.  *dyn = 0
// means they do not fit even at one block per SM and the kernel must keep
// those rows in global memory.
inline int coop_grid_resident(const void* fn, uint32_t n_slices, size_t bytes_per_slice,
                              unsigned* G, size_t* dyn, int threads = kPersistThreads,
                              int min_blocks = kPersistMinBlocks) {
    int dev = 0, nsm = 0, optin = 0;
    NBG_CHECK(cudaGetDevice(&dev));
    NBG_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    NBG_CHECK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    NBG_CHECK(cudaFuncGetAttributes(&fa, fn));
    const unsigned want = (n_slices + threads / 32 - 1) / (threads / 32);
    for (int per_sm = min_blocks; bytes_per_slice && per_sm >= 1; --per_sm) {
        unsigned g = (unsigned)nsm * (unsigned)per_sm;
        if (want < g) g = want;
        if (g < 1) g = 1;
        const size_t spb = (n_slices + g - 1) / g;
        const size_t bytes = spb * bytes_per_slice;
        if (bytes + fa.sharedSizeBytes > (size_t)optin) continue;
        NBG_CHECK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bytes));
        int occ = 0;
        NBG_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, bytes));
        if ((unsigned)occ * (unsigned)nsm >= g) {
            *G = g;
            *dyn = bytes;
            return NBG_OK;
        }
    }
    *dyn = 0;
    NBG_CHECK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 0));
    return coop_grid(fn, n_slices, G, threads);
}

}  // namespace nbg
