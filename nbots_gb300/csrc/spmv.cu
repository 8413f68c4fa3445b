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
    const uint32_t k0 = rp[row0], k1 = rp[row0 + nrows];
    const uint32_t my_row = row0 + lane;
    uint32_t mb = 0, me = 0;
    if (lane < nrows) {
        mb = rp[my_row];
        me = rp[my_row + 1];
    }
    double s = 0.0;
    uint32_t next = mb;  // next product of my row still to add
    for (uint32_t base = k0; base < k1; base += kStage) {
        const uint32_t cnt = min((uint32_t)kStage, k1 - base);
        for (uint32_t t = lane; t < cnt; t += 32) prod[warp][t] = mul(v[base + t], x[ci[base + t]]);
        __syncwarp();
        const uint32_t hi = min(me, base + cnt);
        for (; next < hi; next++) s = add(s, prod[warp][next - base]);
        __syncwarp();
    }
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
