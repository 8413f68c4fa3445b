// Gathers and scatters between the original node order and the node order
// of a block layout (nbg_bsr_t::perm).  T is one node's pair of values:
// double2 for FP64 vectors, float2 for FP32 ones.
#pragma once

#include <cstdint>
#include <type_traits>

#include "common.cuh"

namespace nbg {

template <typename T>
static __global__ void k_perm_gather(uint32_t Nn, const uint32_t* __restrict__ perm,
                              const T* __restrict__ src, T* __restrict__ dst) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < Nn) dst[i] = src[perm[i]];
}

template <typename T>
static __global__ void k_perm_scatter(uint32_t Nn, const uint32_t* __restrict__ perm,
                               const T* __restrict__ src, T* __restrict__ dst) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < Nn) dst[perm[i]] = src[i];
}

// dst[i] = src[perm[i]] over Nn node pairs (src and dst: 2 Nn scalars).
template <typename S>
static inline cudaError_t perm_gather(uint32_t Nn, const uint32_t* perm, const S* src, S* dst,
                               cudaStream_t s) {
    using T = typename std::conditional<sizeof(S) == 8, double2, float2>::type;
    if (Nn == 0) return cudaSuccess;
    k_perm_gather<T><<<(Nn + 255) / 256, 256, 0, s>>>(Nn, perm, (const T*)src, (T*)dst);
    return cudaGetLastError();
}

// dst[perm[i]] = src[i].
template <typename S>
static inline cudaError_t perm_scatter(uint32_t Nn, const uint32_t* perm, const S* src, S* dst,
                                cudaStream_t s) {
    using T = typename std::conditional<sizeof(S) == 8, double2, float2>::type;
    if (Nn == 0) return cudaSuccess;
    k_perm_scatter<T><<<(Nn + 255) / 256, 256, 0, s>>>(Nn, perm, (const T*)src, (T*)dst);
    return cudaGetLastError();
}

// Bytes a solver adds to its workspace for the permuted copies of b and x.
static inline size_t perm_tail_bytes(uint32_t N) { return 2 * (((size_t)N * 8 + 255) & ~(size_t)255); }

}  // namespace nbg
