// Shared helpers of the gfgpu CUDA library: error reporting, launch shapes and the
// strict / fast arithmetic switch.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/gfgpu.h"

namespace gfgpu {

// Per-thread message of the last failing call (returned by gfgpu_last_error()).
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int check_cuda(cudaError_t e, const char* what);
int check_launch(const char* what);
bool strict_mode();
int variant_elem();
int variant_node();
int nn_tensor_path(); // 32 -> 32 network layers: 0 = mma.sync, 1 = tcgen05, 2 = tcgen05 + TMA pipeline

inline cudaStream_t S(gfgpu_stream_t s)
{
    return reinterpret_cast<cudaStream_t>(s);
}

constexpr int kBlock = 256;

inline unsigned grid_for(int64_t n, int block = kBlock)
{
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    return static_cast<unsigned>(g);
}

// Grid-stride loop bound used by elementwise kernels.
#define GF_FOR(i, n)                                                                            \
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < (n);      \
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)

// Strict arithmetic: every product and sum rounded on its own (no FMA contraction), which
// reproduces a reference compiled with -ffp-contract=off bit for bit. Fast arithmetic lets
// the compiler contract a*b+c into one DFMA.
template <bool Strict>
__device__ __forceinline__ double mul(double a, double b)
{
    if constexpr (Strict) return __dmul_rn(a, b);
    else return a * b;
}

template <bool Strict>
__device__ __forceinline__ double add(double a, double b)
{
    if constexpr (Strict) return __dadd_rn(a, b);
    else return a + b;
}

template <bool Strict>
__device__ __forceinline__ double sub(double a, double b)
{
    if constexpr (Strict) return __dsub_rn(a, b);
    else return a - b;
}

// a*b + c (fast: one DFMA).
template <bool Strict>
__device__ __forceinline__ double madd(double a, double b, double c)
{
    if constexpr (Strict) return __dadd_rn(__dmul_rn(a, b), c);
    else return fma(a, b, c);
}

// Element forces of dof t summed in the dof CSR's order (ascending flat elemvec index), from 0.
// On a Regular Quad4 mesh with plain dofs (reg_nx > 0, set by gfgpu_verlet_detect_regular) the
// contributing elements are found by index arithmetic in the same order: same bits, no tables.
__device__ __forceinline__ double gather_dof(int64_t t, const int32_t* __restrict__ dofs,
                                             const int32_t* __restrict__ ptr,
                                             const int32_t* __restrict__ idx,
                                             const double* __restrict__ fe, int64_t reg_nx, int64_t reg_ny)
{
    double f = 0.0;
    if (reg_nx > 0) {
        const int64_t node = t >> 1, i = t & 1, W = reg_nx + 1;
        const int64_t iy = node / W, ix = node - iy * W;
        if (iy > 0 && ix > 0) f += __ldg(fe + (((iy - 1) * reg_nx + ix - 1) * 4 + 2) * 2 + i);
        if (iy > 0 && ix < reg_nx) f += __ldg(fe + (((iy - 1) * reg_nx + ix) * 4 + 3) * 2 + i);
        if (iy < reg_ny && ix > 0) f += __ldg(fe + ((iy * reg_nx + ix - 1) * 4 + 1) * 2 + i);
        if (iy < reg_ny && ix < reg_nx) f += __ldg(fe + ((iy * reg_nx + ix) * 4 + 0) * 2 + i);
        return f;
    }
    const int32_t d = __ldg(dofs + t);
    const int32_t b = __ldg(ptr + d), e = __ldg(ptr + d + 1);
    for (int32_t j = b; j < e; ++j) f += __ldg(fe + __ldg(idx + j));
    return f;
}

inline bool too_big(int64_t n)
{
    return n < 0 || n > INT32_MAX;
}

} // namespace gfgpu

#define GF_REQUIRE(cond, msg)                                                                   \
    do {                                                                                        \
        if (!(cond)) return ::gfgpu::fail(GFGPU_ERR_ARG, std::string(__func__) + ": " + (msg)); \
    } while (0)

#define GF_TRY(expr)                                                                            \
    do {                                                                                        \
        int _rc = (expr);                                                                       \
        if (_rc != GFGPU_OK) return _rc;                                                        \
    } while (0)
