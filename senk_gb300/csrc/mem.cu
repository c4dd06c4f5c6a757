// Device memory helpers of the C ABI, so that host code above it (the drop-in
// headers in include/) can stage arrays without including CUDA headers, and the
// element-wise products of senk::blas1 (HadProd / HadDiv).
#include "device.hpp"

using namespace senkgpu;

extern "C" {

int senk_mem_alloc(void **p, size_t bytes)
{
    return guarded("senk_mem_alloc", [&] {
        SENK_REQUIRE(p != nullptr, "p is null");
        *p = nullptr;
        if (bytes) SENK_CUDA(cudaMalloc(p, bytes));
        return (int)kOk;
    });
}

int senk_mem_free(void *p)
{
    return guarded("senk_mem_free", [&] {
        if (p) SENK_CUDA(cudaFree(p));
        return (int)kOk;
    });
}

int senk_mem_h2d(void *dst, const void *src, size_t bytes)
{
    return guarded("senk_mem_h2d", [&] {
        if (bytes) SENK_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
        return (int)kOk;
    });
}

int senk_mem_d2h(void *dst, const void *src, size_t bytes)
{
    return guarded("senk_mem_d2h", [&] {
        if (bytes) SENK_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
        return (int)kOk;
    });
}

int senk_mem_sync(void)
{
    return guarded("senk_mem_sync", [&] {
        SENK_CUDA(cudaDeviceSynchronize());
        return (int)kOk;
    });
}

// 1 when p is device (or managed) memory the GPU can dereference, 0 for
// pageable or pinned host memory, negative on error.
int senk_mem_is_device(const void *p)
{
    if (!p) return 0;
    cudaPointerAttributes a{};
    const cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_last_error(std::string("senk_mem_is_device: ") + cudaGetErrorString(e));
        return -(int)kErrCuda;
    }
    return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) ? 1 : 0;
}

int senk_dev_hadprod_d(const double *x, double *y, int N, void *stream)
{
    return guarded("senk_dev_hadprod_d", [&] {
        SENK_REQUIRE(N >= 0, "N must be non-negative");
        if (N == 0) return (int)kOk;
        k_elementwise<double, 5><<<stream_grid(N, kThreads, 8), kThreads, 0, (cudaStream_t)stream>>>(
            0.0, nullptr, 1.0, 0.0, x, y, nullptr, N, nullptr);
        SENK_LAUNCH_CHECK();
        return (int)kOk;
    });
}

int senk_dev_haddiv_d(const double *x, double *y, int N, void *stream)
{
    return guarded("senk_dev_haddiv_d", [&] {
        SENK_REQUIRE(N >= 0, "N must be non-negative");
        if (N == 0) return (int)kOk;
        k_elementwise<double, 6><<<stream_grid(N, kThreads, 8), kThreads, 0, (cudaStream_t)stream>>>(
            0.0, nullptr, 1.0, 0.0, x, y, nullptr, N, nullptr);
        SENK_LAUNCH_CHECK();
        return (int)kOk;
    });
}

}  // extern "C"
