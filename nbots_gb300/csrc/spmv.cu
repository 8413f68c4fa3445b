// SpMV kernels over nbots' CSR (row_ptr / col_idx / FP64 values).
//
// k_spmv_csr_exact: y_i = sum_k A_ik x_col in nbots' order (start at 0, add
// each rounded product left to right, sparse.c:405-414), so y is bit-exact.
// One warp owns 32 consecutive rows: it stages their (value, column) span
// through shared memory with coalesced loads, forms the rounded products in
// parallel, then each lane adds its own row's products in column order.
#include <cstdint>

#include "common.cuh"

using namespace nbg;

namespace {

constexpr int kWarps = 8;            // warps per block
constexpr int kStage = 640;          // products staged per warp per pass (40 KB smem)

__global__ void __launch_bounds__(kWarps * 32) k_spmv_csr_exact(uint32_t N,
                                                               const uint32_t* __restrict__ rp,
                                                               const uint32_t* __restrict__ ci,
                                                               const double* __restrict__ v,
                                                               const double* __restrict__ x,
                                                               double* __restrict__ y) {
    __shared__ double prod[kWarps][kStage];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t row0 = (blockIdx.x * kWarps + warp) * 32u;
    if (row0 >= N) return;
    const uint32_t nrows = min(32u, N - row0);
    const uint32_t my_row = row0 + lane;
    const double s = warp_rows_exact<kStage>(rp, ci, v, x, row0, nrows, prod[warp], lane);
    if (lane < nrows) y[my_row] = s;
}

}  // namespace

extern "C" int nbg_spmv_csr_f64(uint32_t N, const uint32_t* row_ptr, const uint32_t* col_idx,
                                const double* val, const double* x, double* y, void* stream) {
    if (N == 0) return NBG_OK;
    const unsigned rows_per_block = kWarps * 32;
    const unsigned grid = (N + rows_per_block - 1) / rows_per_block;
    k_spmv_csr_exact<<<grid, kWarps * 32, 0, (cudaStream_t)stream>>>(N, row_ptr, col_idx, val, x,
                                                                      y);
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}
