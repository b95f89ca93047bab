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
