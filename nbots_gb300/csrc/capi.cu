// Library-wide pieces of the C ABI: version, error text, device memory.
#include <cstdio>
#include <cstring>

#include "common.cuh"

namespace {
thread_local char g_last_error[256] = "";
}

int nbg_cuda_error(cudaError_t e) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", cudaGetErrorName(e),
                  cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation) return NBG_ERR_NOMEM;
    return NBG_ERR_CUDA;
}

int nbg_error_text(int code, const char* text) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s", text);
    return code;
}

extern "C" const char* nbg_version(void) { return "nbots_gb300 0.1 (sm_103a)"; }

extern "C" const char* nbg_last_error(void) { return g_last_error; }

extern "C" int nbg_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

extern "C" int nbg_dev_alloc(void** ptr, size_t bytes) {
    if (!ptr) return NBG_ERR_ARG;
    *ptr = nullptr;
    NBG_CHECK(cudaMalloc(ptr, bytes ? bytes : 1));
    return NBG_OK;
}

extern "C" int nbg_dev_free(void* ptr) {
    if (ptr) NBG_CHECK(cudaFree(ptr));
    return NBG_OK;
}

extern "C" int nbg_h2d(void* dst, const void* src, size_t bytes, void* stream) {
    if (bytes == 0) return NBG_OK;
    NBG_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    return NBG_OK;
}

extern "C" int nbg_d2h(void* dst, const void* src, size_t bytes, void* stream) {
    if (bytes == 0) return NBG_OK;
    NBG_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    return NBG_OK;
}

extern "C" int nbg_d2d(void* dst, const void* src, size_t bytes, void* stream) {
    if (bytes == 0) return NBG_OK;
    NBG_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return NBG_OK;
}

extern "C" int nbg_memset(void* dst, int value, size_t bytes, void* stream) {
    if (bytes == 0) return NBG_OK;
    NBG_CHECK(cudaMemsetAsync(dst, value, bytes, (cudaStream_t)stream));
    return NBG_OK;
}

extern "C" int nbg_stream_sync(void* stream) {
    NBG_CHECK(cudaStreamSynchronize((cudaStream_t)stream));
    return NBG_OK;
}

extern "C" int nbg_host_memory_access(void) {
    int dev = 0, pageable = 0, host_tables = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                               dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return pageable == 1 && host_tables == 1;
}

extern "C" int nbg_host_alloc(void** ptr, size_t bytes) {
    if (!ptr) return NBG_ERR_ARG;
    *ptr = nullptr;
    NBG_CHECK(cudaMallocHost(ptr, bytes ? bytes : 1));
    return NBG_OK;
}

extern "C" int nbg_host_free(void* ptr) {
    if (ptr) NBG_CHECK(cudaFreeHost(ptr));
    return NBG_OK;
}

namespace {
// One thread waits until *flag == expect or `limit_ns` has passed; on expiry
// it records NBG_ERR_TIMEOUT in *status and returns.  The same bounded wait
// guards every grid barrier of the persistent solvers.
__global__ void k_wait_flag(const int* flag, int expect, uint64_t limit_ns, int* status) {
    const uint64_t t0 = nbg::globaltimer();
    while (nbg::ld_volatile(flag) != expect) {
        if (nbg::globaltimer() - t0 > limit_ns) {
            atomicCAS(status, 0, NBG_ERR_TIMEOUT);
            return;
        }
        __nanosleep(1000);
    }
}
}  // namespace

extern "C" int nbg_wait_flag(const int* flag, int expect, uint64_t limit_ns, int* status,
                             void* stream) {
    if (!flag || !status) return NBG_ERR_ARG;
    k_wait_flag<<<1, 1, 0, (cudaStream_t)stream>>>(flag, expect, limit_ns, status);
    NBG_CHECK(cudaGetLastError());
    return NBG_OK;
}
