// Streamed SpMVs on the 2x2-block SELL layout: each warp owns a contiguous
// run of slices and streams them through a double-buffered shared-memory
// ring with cp.async.bulk (stream.cuh); the x gathers of a slice are issued
// together.  One launch covers the matrix with one block of kWarps warps per
// SM.
//
//  k_spmv_split_stream  y = A x with A = b32 + blo (FP32 hi + bfloat16 lo)
//                       and x = xh + xl (FP32 hi + bfloat16 lo); products
//                       and sums by error-free transformations; y as
//                       yh + yl.  The operator of the mixed-precision CG.
//  k_spmv_f64_stream    y = A x with FP64 values and FMAs.
#include <cstdint>

#include "persist.cuh"
#include "stream.cuh"

using namespace nbg;

namespace {

constexpr int kWarps = 8;
constexpr int kStages = 2;
constexpr int kMaxWSplit = 12;   // entries per lane a stage holds (Q4: 9, T3: 7 on average)
constexpr int kMaxW64 = 10;
constexpr int kBSplit = 28;      // b32 16 + blo 8 + bcol 4
constexpr int kB64 = 36;         // b64 32 + bcol 4

// contiguous slice run of warp gw out of TW warps
__device__ __forceinline__ void warp_run(uint32_t S, uint32_t gw, uint32_t TW, uint32_t& a,
                                         uint32_t& b) {
    a = (uint32_t)(((uint64_t)S * gw) / TW);
    b = (uint32_t)(((uint64_t)S * (gw + 1)) / TW);
}

__global__ void __launch_bounds__(kWarps * 32, 1)
    k_spmv_split_stream(nbg_bsr_t A, const float* __restrict__ xh, const __nv_bfloat16* __restrict__ xl,
                        float* __restrict__ yh, __nv_bfloat16* __restrict__ yl, int* status) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bars[kWarps][kStages];
    using WS = WarpStream<kStages, kMaxWSplit, kBSplit>;
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned char* wbuf = smem + (size_t)w * WS::kBytes;
    uint32_t s_beg, s_end;
    warp_run(A.n_slices, blockIdx.x * kWarps + w, gridDim.x * kWarps, s_beg, s_end);
    const uint32_t n = s_end - s_beg;
    if (lane == 0) {
        for (int st = 0; st < kStages; st++) mbar_init(&bars[w][st], 1);
        fence_mbar_init();
    }
    __syncwarp();
    const float4* __restrict__ gb32 = reinterpret_cast<const float4*>(A.b32);
    const uint2* __restrict__ gblo = reinterpret_cast<const uint2*>(A.blo);
    const float2* __restrict__ x2h = reinterpret_cast<const float2*>(xh);
    const __nv_bfloat162* __restrict__ x2l = reinterpret_cast<const __nv_bfloat162*>(xl);

    auto issue = [&](uint32_t j) {  // lane 0 only
        const uint32_t s = s_beg + j, st = j % kStages;
        const uint32_t k0 = A.slice_off[s], width = A.slice_off[s + 1] - k0;
        if (width > (uint32_t)kMaxWSplit) {
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&bars[w][st]))
                         : "memory");
            return;
        }
        unsigned char* sb = wbuf + st * WS::kStageBytes;
        const size_t e0 = (size_t)k0 * 32;
        mbar_expect_tx(&bars[w][st], width * 32u * kBSplit);
        bulk_g2s(sb, gb32 + e0, width * 512u, &bars[w][st]);
        bulk_g2s(sb + kMaxWSplit * 512, gblo + e0, width * 256u, &bars[w][st]);
        bulk_g2s(sb + kMaxWSplit * 768, A.bcol + e0, width * 128u, &bars[w][st]);
    };
    if (lane == 0)
        for (uint32_t j = 0; j < n && j < (uint32_t)kStages; j++) issue(j);

    for (uint32_t j = 0; j < n; j++) {
        const uint32_t s = s_beg + j, st = j % kStages;
        const uint32_t k0 = A.slice_off[s], width = A.slice_off[s + 1] - k0;
        if (!mbar_wait(&bars[w][st], (j / kStages) & 1, status)) return;
        const unsigned char* sb = wbuf + st * WS::kStageBytes;
        const bool staged = width <= (uint32_t)kMaxWSplit;
        const float4* mb = staged ? reinterpret_cast<const float4*>(sb) : gb32 + (size_t)k0 * 32;
        const uint2* ml = staged ? reinterpret_cast<const uint2*>(sb + kMaxWSplit * 512)
                                 : gblo + (size_t)k0 * 32;
        const uint32_t* mc = staged ? reinterpret_cast<const uint32_t*>(sb + kMaxWSplit * 768)
                                    : A.bcol + (size_t)k0 * 32;
        FFAcc c0{0.f, 0.f}, c1{0.f, 0.f};
#pragma unroll 4
        for (uint32_t k = 0; k < width; k++) {
            const uint32_t c = mc[k * 32 + lane];
            const float2 pc = x2h[c];
            const float2 pcl = __bfloat1622float2(x2l[c]);
            const float4 m = mb[k * 32 + lane];
            const float4 sc = rem16_scale4(ml[k * 32 + lane]);
            c0.fma2s(m.x, sc.x, pc.x, pcl.x);
            c0.fma2s(m.y, sc.y, pc.y, pcl.y);
            c1.fma2s(m.z, sc.z, pc.x, pcl.x);
            c1.fma2s(m.w, sc.w, pc.y, pcl.y);
        }
        const uint32_t i = s * 32 + lane;
        if (i < A.Nn) {
            const FF y0 = c0.result(), y1 = c1.result();
            reinterpret_cast<float2*>(yh)[i] = make_float2(y0.hi, y1.hi);
            reinterpret_cast<__nv_bfloat162*>(yl)[i] = __floats2bfloat162_rn(y0.lo, y1.lo);
        }
        __syncwarp();
        if (lane == 0 && j + kStages < n) issue(j + kStages);
    }
}

__global__ void __launch_bounds__(kWarps * 32, 1)
    k_spmv_f64_stream(nbg_bsr_t A, const double* __restrict__ x, double* __restrict__ y,
                      int* status) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bars[kWarps][kStages];
    using WS = WarpStream<kStages, kMaxW64, kB64>;
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned char* wbuf = smem + (size_t)w * WS::kBytes;
    uint32_t s_beg, s_end;
    warp_run(A.n_slices, blockIdx.x * kWarps + w, gridDim.x * kWarps, s_beg, s_end);
    const uint32_t n = s_end - s_beg;
    if (lane == 0) {
        for (int st = 0; st < kStages; st++) mbar_init(&bars[w][st], 1);
        fence_mbar_init();
    }
    __syncwarp();
    const double2* __restrict__ gb = reinterpret_cast<const double2*>(A.b64);
    const double2* __restrict__ x2 = reinterpret_cast<const double2*>(x);

    auto issue = [&](uint32_t j) {
        const uint32_t s = s_beg + j, st = j % kStages;
        const uint32_t k0 = A.slice_off[s], width = A.slice_off[s + 1] - k0;
        if (width > (uint32_t)kMaxW64) {
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&bars[w][st]))
                         : "memory");
            return;
        }
        unsigned char* sb = wbuf + st * WS::kStageBytes;
        const size_t e0 = (size_t)k0 * 32;
        mbar_expect_tx(&bars[w][st], width * 32u * kB64);
        bulk_g2s(sb, A.b64 + 4 * e0, width * 1024u, &bars[w][st]);
        bulk_g2s(sb + kMaxW64 * 1024, A.bcol + e0, width * 128u, &bars[w][st]);
    };
    if (lane == 0)
        for (uint32_t j = 0; j < n && j < (uint32_t)kStages; j++) issue(j);

    for (uint32_t j = 0; j < n; j++) {
        const uint32_t s = s_beg + j, st = j % kStages;
        const uint32_t k0 = A.slice_off[s], width = A.slice_off[s + 1] - k0;
        if (!mbar_wait(&bars[w][st], (j / kStages) & 1, status)) return;
        const unsigned char* sb = wbuf + st * WS::kStageBytes;
        const bool staged = width <= (uint32_t)kMaxW64;
        const double2* mb = staged ? reinterpret_cast<const double2*>(sb) : gb + (size_t)k0 * 64;
        const uint32_t* mc = staged ? reinterpret_cast<const uint32_t*>(sb + kMaxW64 * 1024)
                                    : A.bcol + (size_t)k0 * 32;
        double y0 = 0.0, y1 = 0.0;
#pragma unroll 4
        for (uint32_t k = 0; k < width; k++) {
            const uint32_t e = k * 32 + lane;
            const double2 xc = x2[mc[e]];
            const double2 top = mb[2 * e], bot = mb[2 * e + 1];
            y0 = fma(top.x, xc.x, y0);
            y0 = fma(top.y, xc.y, y0);
            y1 = fma(bot.x, xc.x, y1);
            y1 = fma(bot.y, xc.y, y1);
        }
        const uint32_t i = s * 32 + lane;
        if (i < A.Nn) reinterpret_cast<double2*>(y)[i] = make_double2(y0, y1);
        __syncwarp();
        if (lane == 0 && j + kStages < n) issue(j + kStages);
    }
}

template <typename K>
int launch_stream(K kern, size_t smem_bytes, void** args, cudaStream_t s) {
    int dev = 0, nsm = 0;
    NBG_CHECK(cudaGetDevice(&dev));
    NBG_CHECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    NBG_CHECK(cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem_bytes));
    NBG_CHECK(cudaLaunchKernel((const void*)kern, dim3(nsm), dim3(kWarps * 32), args, smem_bytes, s));
    return NBG_OK;
}

}  // namespace

extern "C" int nbg_spmv_bsr_split(const nbg_bsr_t* A, const float* xh, const uint16_t* xl,
                                  float* yh, uint16_t* yl, int* status, void* stream) {
    if (!A || !A->b32 || !A->blo || !status) return NBG_ERR_ARG;
    if (A->Nn == 0) return NBG_OK;
    nbg_bsr_t a = *A;
    const __nv_bfloat16* xlb = reinterpret_cast<const __nv_bfloat16*>(xl);
    __nv_bfloat16* ylb = reinterpret_cast<__nv_bfloat16*>(yl);
    void* args[] = {&a, &xh, &xlb, &yh, &ylb, &status};
    return launch_stream(k_spmv_split_stream, kWarps * WarpStream<kStages, kMaxWSplit, kBSplit>::kBytes,
                         args, (cudaStream_t)stream);
}

extern "C" int nbg_spmv_bsr_f64_stream(const nbg_bsr_t* A, const double* x, double* y,
                                       int* status, void* stream) {
    if (!A || !A->b64 || !status) return NBG_ERR_ARG;
    if (A->Nn == 0) return NBG_OK;
    nbg_bsr_t a = *A;
    void* args[] = {&a, &x, &y, &status};
    return launch_stream(k_spmv_f64_stream, kWarps * WarpStream<kStages, kMaxW64, kB64>::kBytes,
                         args, (cudaStream_t)stream);
}
