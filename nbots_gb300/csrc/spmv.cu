// SpMV over nbots' CSR (row_ptr / col_idx / FP64 values).
//
// k_spmv_csr_exact: y_i = sum_k A_ik x_col in nbots' order (start at 0, add
// each rounded product left to right, sparse.c:405-414), so y is bit-exact.
// One thread per row; the row is walked four entries at a time with the
// four columns, values and gathers loaded before the four ordered adds, so
// each thread keeps four gathers in flight.  The kernel is bound by GB300's
// FP64 pipe (one DMUL and one DADD per stored value, no FMA, as nbots); on
// the 1M-dof cantilever it took 89 us against 97 us for staging 32 rows'
// products through shared memory per warp, and 11 against 13 us at 16,770
// dof.
#include <cstdint>

#include "common.cuh"

using namespace nbg;

namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_spmv_csr_exact(uint32_t N,
                                                            const uint32_t* __restrict__ rp,
                                                            const uint32_t* __restrict__ ci,
                                                            const double* __restrict__ v,
                                                            const double* __restrict__ x,
                                                            double* __restrict__ y) {
    const uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= N) return;
    const uint32_t e = rp[i + 1];
    uint32_t k = rp[i];
    double s = 0.0;
    for (; k + 4 <= e; k += 4) {
        const uint32_t c0 = ci[k], c1 = ci[k + 1], c2 = ci[k + 2], c3 = ci[k + 3];
        const double v0 = v[k], v1 = v[k + 1], v2 = v[k + 2], v3 = v[k + 3];
        const double x0 = x[c0], x1 = x[c1], x2 = x[c2], x3 = x[c3];
        s = add(s, mul(v0, x0));
        s = add(s, mul(v1, x1));
        s = add(s, mul(v2, x2));
        s = add(s, mul(v3, x3));
    }
    for (; k < e; k++) s = add(s, mul(v[k], x[ci[k]]));
    y[i] = s;
}

}  // namespace

extern "C" int nbg_spmv_csr_f64(uint32_t N, const uint32_t* row_ptr, const uint32_t* col_idx,
                                const double* val, const double* x, double* y, void* stream) {
    if (N == 0) return NBG_OK;
    k_spmv_csr_exact<<<(N + kThreads - 1) / kThreads, kThreads, 0, (cudaStream_t)stream>>>(
        N, row_ptr, col_idx, val, x, y);
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}
