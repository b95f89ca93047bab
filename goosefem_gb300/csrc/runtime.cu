// CUDA error plumbing of the gfgpu library.
#include <string>

#include "common.cuh"

namespace gfgpu {

int check_cuda(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return GFGPU_OK;
    return fail(GFGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int check_launch(const char* what)
{
    return check_cuda(cudaGetLastError(), what);
}

} // namespace gfgpu

using gfgpu::check_cuda;

extern "C" {

int gfgpu_malloc(void** ptr, int64_t bytes)
{
    GF_REQUIRE(ptr && bytes >= 0, "bad argument");
    *ptr = nullptr;
    if (bytes == 0) return GFGPU_OK;
    return check_cuda(cudaMalloc(ptr, static_cast<size_t>(bytes)), "cudaMalloc");
}

int gfgpu_free(void* ptr)
{
    return ptr ? check_cuda(cudaFree(ptr), "cudaFree") : GFGPU_OK;
}

int gfgpu_memcpy_h2d(void* dst, const void* src, int64_t bytes)
{
    GF_REQUIRE(bytes >= 0 && (bytes == 0 || (dst && src)), "bad argument");
    if (bytes == 0) return GFGPU_OK;
    return check_cuda(cudaMemcpy(dst, src, static_cast<size_t>(bytes), cudaMemcpyHostToDevice),
                      "cudaMemcpy H2D");
}

int gfgpu_memcpy_d2h(void* dst, const void* src, int64_t bytes)
{
    GF_REQUIRE(bytes >= 0 && (bytes == 0 || (dst && src)), "bad argument");
    if (bytes == 0) return GFGPU_OK;
    return check_cuda(cudaMemcpy(dst, src, static_cast<size_t>(bytes), cudaMemcpyDeviceToHost),
                      "cudaMemcpy D2H");
}

int gfgpu_memcpy_d2d(void* dst, const void* src, int64_t bytes)
{
    GF_REQUIRE(bytes >= 0 && (bytes == 0 || (dst && src)), "bad argument");
    if (bytes == 0) return GFGPU_OK;
    return check_cuda(cudaMemcpy(dst, src, static_cast<size_t>(bytes), cudaMemcpyDeviceToDevice),
                      "cudaMemcpy D2D");
}

int gfgpu_memset(void* ptr, int value, int64_t bytes)
{
    GF_REQUIRE(bytes >= 0 && (bytes == 0 || ptr), "bad argument");
    if (bytes == 0) return GFGPU_OK;
    return check_cuda(cudaMemset(ptr, value, static_cast<size_t>(bytes)), "cudaMemset");
}

int gfgpu_synchronize(void)
{
    return check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
}

} // extern "C"
