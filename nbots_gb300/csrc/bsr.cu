// 2x2-block SELL-32 layout of nbots' stiffness matrix and its SpMVs.
//
// nb_sparse_create(graph, NULL, 2) gives each node two rows with the same
// sorted column list made of (2w, 2w+1) pairs (sparse.c:36-52), so the CSR
// is exactly a 2x2 block matrix.  The fast kernels store it by node row:
// slices of 32 node rows, each slice as wide as its longest row, entry
// (slice s, k, lane r) at ((slice_off[s] + k) * 32 + r).  A warp then reads
// 32 consecutive blocks per step (coalesced), one node row per lane; padding
// entries point at the row's own node with zero values.  One uint32 column
// serves four values, so FP32 values + index cost 5 B per nonzero instead of
// the 12 B of FP64 CSR.  The standalone SpMVs unroll the slice walk by four
// and load the matrix with an L2 evict_first policy: at 1M dof (L2 flushed)
// the FP32 one took 25.2 us against 31.4 us for the plain loop.
#include <cstdint>

#include "perm.cuh"

using namespace nbg;

namespace {

// Slice row i holds node v = perm[i] (v = i without an order); columns are
// stored in the same order (iperm).
__global__ void k_bsr_fill(uint32_t Nn, const uint32_t* __restrict__ rp,
                           const uint32_t* __restrict__ ci, const double* __restrict__ val,
                           const uint32_t* __restrict__ slice_off,
                           const uint32_t* __restrict__ perm, const uint32_t* __restrict__ iperm,
                           uint32_t* __restrict__ bcol, double* __restrict__ b64,
                           float* __restrict__ b32, uint16_t* __restrict__ blo,
                           uint8_t* __restrict__ bxt, double* __restrict__ dinv64,
                           float* __restrict__ dinv32) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Nn) return;
    const uint32_t s = i >> 5, lane = i & 31;
    const uint32_t v = perm ? perm[i] : i;
    const uint32_t width = slice_off[s + 1] - slice_off[s];
    const uint32_t r0 = rp[2 * v], r1 = rp[2 * v + 1];
    const uint32_t nb = (r1 - r0) / 2;
    double d0 = 0.0, d1 = 0.0;
    for (uint32_t k = 0; k < width; k++) {
        const size_t e = ((size_t)slice_off[s] + k) * 32 + lane;
        double a00 = 0.0, a01 = 0.0, a10 = 0.0, a11 = 0.0;
        uint32_t c = i;
        if (k < nb) {
            const uint32_t w = ci[r0 + 2 * k] >> 1;
            c = iperm ? iperm[w] : w;
            a00 = val[r0 + 2 * k];
            a01 = val[r0 + 2 * k + 1];
            a10 = val[r1 + 2 * k];
            a11 = val[r1 + 2 * k + 1];
            if (w == v) {
                d0 = a00;
                d1 = a11;
            }
        }
        bcol[e] = c;
        if (b64) {
            b64[4 * e] = a00;
            b64[4 * e + 1] = a01;
            b64[4 * e + 2] = a10;
            b64[4 * e + 3] = a11;
        }
        const float h00 = (float)a00, h01 = (float)a01, h10 = (float)a10, h11 = (float)a11;
        // FP32 values column by column (a00 a10 a01 a11): a column is a pair
        // of adjacent registers for the packed FP32x2 arithmetic
        if (b32) reinterpret_cast<float4*>(b32)[e] = make_float4(h00, h10, h01, h11);
        if (blo && bxt) {
            // remainders (exact in FP64) as biased 23-bit counts of 2^-46 hi,
            // in the same order
            const uint32_t q0 = rem23_encode(a00, h00), q1 = rem23_encode(a10, h10);
            const uint32_t q2 = rem23_encode(a01, h01), q3 = rem23_encode(a11, h11);
            uint2 packed;
            packed.x = (q0 & 0xFFFFu) | (q1 << 16);
            packed.y = (q2 & 0xFFFFu) | (q3 << 16);
            reinterpret_cast<uint2*>(blo)[e] = packed;
            reinterpret_cast<uint32_t*>(bxt)[e] =
                (q0 >> 16) | ((q1 >> 16) << 8) | ((q2 >> 16) << 16) | ((q3 >> 16) << 24);
        }
    }
    if (dinv64) {
        dinv64[2 * i] = 1.0 / d0;
        dinv64[2 * i + 1] = 1.0 / d1;
    }
    if (dinv32) {
        dinv32[2 * i] = (float)(1.0 / d0);
        dinv32[2 * i + 1] = (float)(1.0 / d1);
    }
}

__global__ void __launch_bounds__(256) k_spmv_bsr_f64(uint32_t Nn, const uint32_t* __restrict__ so,
                                                      const uint32_t* __restrict__ bcol,
                                                      const double* __restrict__ b64,
                                                      const double* __restrict__ x,
                                                      double* __restrict__ y) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Nn) return;
    const uint32_t s = i >> 5, lane = i & 31;
    const uint32_t k0 = so[s], k1 = so[s + 1];
    const double2* __restrict__ xv = reinterpret_cast<const double2*>(x);
    const double2* __restrict__ bv = reinterpret_cast<const double2*>(b64);
    const uint64_t pol = l2_policy(false);  // the matrix streams through L2 once
    double y0 = 0.0, y1 = 0.0;
#pragma unroll 4
    for (uint32_t k = k0; k < k1; k++) {
        const size_t e = (size_t)k * 32 + lane;
        const double2 xc = xv[ld_hint(bcol + e, pol)];
        const double2 top = ld_hint(bv + 2 * e, pol), bot = ld_hint(bv + 2 * e + 1, pol);
        y0 = fma(top.x, xc.x, y0);
        y0 = fma(top.y, xc.y, y0);
        y1 = fma(bot.x, xc.x, y1);
        y1 = fma(bot.y, xc.y, y1);
    }
    reinterpret_cast<double2*>(y)[i] = make_double2(y0, y1);
}

__global__ void __launch_bounds__(256) k_spmv_bsr_f32(uint32_t Nn, const uint32_t* __restrict__ so,
                                                      const uint32_t* __restrict__ bcol,
                                                      const float* __restrict__ b32,
                                                      const float* __restrict__ x,
                                                      float* __restrict__ y) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Nn) return;
    const uint32_t s = i >> 5, lane = i & 31;
    const uint32_t k0 = so[s], k1 = so[s + 1];
    const float2* __restrict__ xv = reinterpret_cast<const float2*>(x);
    const float4* __restrict__ bv = reinterpret_cast<const float4*>(b32);
    const uint64_t pol = l2_policy(false);  // the matrix streams through L2 once
    float y0 = 0.f, y1 = 0.f;
#pragma unroll 4
    for (uint32_t k = k0; k < k1; k++) {
        const size_t e = (size_t)k * 32 + lane;
        const float4 a = ld_hint(bv + e, pol);
        const float2 xc = xv[ld_hint(bcol + e, pol)];
        y0 = fmaf(a.x, xc.x, y0);  // a = (a00 a10 a01 a11)
        y0 = fmaf(a.z, xc.y, y0);
        y1 = fmaf(a.y, xc.x, y1);
        y1 = fmaf(a.w, xc.y, y1);
    }
    reinterpret_cast<float2*>(y)[i] = make_float2(y0, y1);
}

}  // namespace

extern "C" int nbg_bsr_plan(uint32_t N, const uint32_t* row_ptr, const uint32_t* col_idx,
                            uint32_t* slice_off) {
    if (N & 1) return NBG_ERR_PATTERN;
    const uint32_t Nn = N / 2, S = (Nn + 31) / 32;
    slice_off[0] = 0;
    for (uint32_t s = 0; s < S; s++) {
        uint32_t w = 0;
        for (uint32_t i = s * 32; i < Nn && i < s * 32 + 32; i++) {
            const uint32_t a = row_ptr[2 * i], b = row_ptr[2 * i + 1], c = row_ptr[2 * i + 2];
            if (b - a != c - b || ((b - a) & 1)) return NBG_ERR_PATTERN;
            for (uint32_t k = 0; k < b - a; k += 2) {
                const uint32_t c0 = col_idx[a + k];
                if ((c0 & 1) || col_idx[a + k + 1] != c0 + 1 || col_idx[b + k] != c0 ||
                    col_idx[b + k + 1] != c0 + 1)
                    return NBG_ERR_PATTERN;
            }
            if ((b - a) / 2 > w) w = (b - a) / 2;
        }
        slice_off[s + 1] = slice_off[s] + w;
    }
    return NBG_OK;
}

extern "C" int nbg_bsr_fill(const nbg_bsr_t* A, const uint32_t* row_ptr, const uint32_t* col_idx,
                            const double* val, void* stream) {
    if (A->Nn == 0) return NBG_OK;
    if ((A->perm == nullptr) != (A->iperm == nullptr)) return NBG_ERR_ARG;
    k_bsr_fill<<<(A->Nn + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        A->Nn, row_ptr, col_idx, val, A->slice_off, A->perm, A->iperm, (uint32_t*)A->bcol,
        (double*)A->b64, (float*)A->b32, (uint16_t*)A->blo, (uint8_t*)A->bxt,
        (double*)A->dinv64, (float*)A->dinv32);
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}

// y = A x with x and y in the original node order: with a node order the
// vectors pass through permuted device copies.
template <typename T, typename K>
static int spmv_perm(const nbg_bsr_t* A, const T* x, T* y, cudaStream_t s, K launch) {
    if (!A->perm) {
        launch(x, y);
        NBG_CHECK(cudaGetLastError());
        return NBG_OK;
    }
    T* tmp = nullptr;
    NBG_CHECK(cudaMalloc(&tmp, 2 * sizeof(T) * (size_t)A->N));
    cudaError_t e = perm_gather(A->Nn, A->perm, x, tmp, s);
    if (e == cudaSuccess) {
        launch(tmp, tmp + A->N);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = perm_scatter(A->Nn, A->perm, tmp + A->N, y, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(tmp);
    if (e != cudaSuccess) return nbg_cuda_error(e);
    return NBG_OK;
}

extern "C" int nbg_spmv_bsr_f64(const nbg_bsr_t* A, const double* x, double* y, void* stream) {
    if (A->Nn == 0) return NBG_OK;
    if (!A->b64) return NBG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    return spmv_perm(A, x, y, s, [&](const double* xx, double* yy) {
        k_spmv_bsr_f64<<<(A->Nn + 255) / 256, 256, 0, s>>>(A->Nn, A->slice_off, A->bcol, A->b64,
                                                            xx, yy);
    });
}

extern "C" int nbg_spmv_bsr_f32(const nbg_bsr_t* A, const float* x, float* y, void* stream) {
    if (A->Nn == 0) return NBG_OK;
    if (!A->b32) return NBG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    return spmv_perm(A, x, y, s, [&](const float* xx, float* yy) {
        k_spmv_bsr_f32<<<(A->Nn + 255) / 256, 256, 0, s>>>(A->Nn, A->slice_off, A->bcol, A->b32,
                                                            xx, yy);
    });
}
