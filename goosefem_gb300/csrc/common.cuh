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
int pair_kernel();    // float-float explicit increment: 2 (default) / 0 = persistent TMA pipeline (31 x 15 / 31 x 7 tiles), 1 = one tile per CTA
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

// The static solvers' view of a Regular mesh (all zero: gather through the dof CSR). soa: the
// element forces are stored component-major, fe[(m * 3 + i) * nelem + e] (the cube Hex8 kernel's
// layout for these solvers, coalesced for the gather); otherwise fe[(e * nne + m) * ndim + i].
struct RegGrid {
    int64_t nx, ny, nz;
    int32_t soa;
};

inline RegGrid reg_grid(const gfgpu_verlet_desc* d)
{
    RegGrid g{d->reg_nx, d->reg_ny, d->reg_nz, 0};
    g.soa = (d->reg_nz > 0 && d->nne == 8 && d->uniform && d->coef) ? 1 : 0;
    return g;
}

// Element forces of dof t summed in the dof CSR's order (ascending flat elemvec index), from 0.
// On a Regular Quad4 mesh (reg.nx > 0, reg.nz == 0; gfgpu_verlet_detect_regular) or a Regular
// Hex8 mesh (reg.nz > 0; gfgpu_verlet_detect_regular_hex8), both with plain dofs, the contributing
// elements are found by index arithmetic in the same order: same bits, no tables.
__device__ __forceinline__ double gather_dof(int64_t t, const int32_t* __restrict__ dofs,
                                             const int32_t* __restrict__ ptr,
                                             const int32_t* __restrict__ idx,
                                             const double* __restrict__ fe, const RegGrid& reg)
{
    double f = 0.0;
    // the detections only accept meshes whose elemvec has < 2^31 entries: 32-bit index arithmetic
    if (reg.nz > 0) {
        // node (ix, iy, iz); element (ex, ey, ez) holds it as local node m = 4 dz + q(dx, dy) with
        // (dx, dy, dz) = node - element, q(0,0) = 0, q(1,0) = 1, q(1,1) = 2, q(0,1) = 3
        const uint32_t nx = static_cast<uint32_t>(reg.nx), ny = static_cast<uint32_t>(reg.ny);
        const uint32_t nz = static_cast<uint32_t>(reg.nz);
        const uint32_t tt = static_cast<uint32_t>(t), node = tt / 3u, i = tt - node * 3u;
        // element e's entry (m, i) at e * es + (m * 3 + i) * cs
        const uint32_t es = reg.soa ? 1u : 24u, cs = reg.soa ? nx * ny * nz : 1u;
        const uint32_t W = nx + 1u, A = W * (ny + 1u);
        const uint32_t iz = node / A, rem = node - iz * A, iy = rem / W, ix = rem - iy * W;
#pragma unroll
        for (int dz = 1; dz >= 0; --dz) {
            if ((dz && iz == 0u) || (!dz && iz >= nz)) continue;
#pragma unroll
            for (int dy = 1; dy >= 0; --dy) {
                if ((dy && iy == 0u) || (!dy && iy >= ny)) continue;
#pragma unroll
                for (int dx = 1; dx >= 0; --dx) {
                    if ((dx && ix == 0u) || (!dx && ix >= nx)) continue;
                    const int m = 4 * dz + (dy ? (dx ? 2 : 3) : (dx ? 1 : 0));
                    const uint32_t e = ((iz - dz) * ny + (iy - dy)) * nx + (ix - dx);
                    f += __ldg(fe + e * es + (m * 3u + i) * cs);
                }
            }
        }
        return f;
    }
    if (reg.nx > 0) {
        const uint32_t nx = static_cast<uint32_t>(reg.nx), ny = static_cast<uint32_t>(reg.ny);
        const uint32_t tt = static_cast<uint32_t>(t), node = tt >> 1, i = tt & 1u, W = nx + 1u;
        const uint32_t iy = node / W, ix = node - iy * W;
        if (iy > 0u && ix > 0u) f += __ldg(fe + (((iy - 1u) * nx + ix - 1u) * 4u + 2u) * 2u + i);
        if (iy > 0u && ix < nx) f += __ldg(fe + (((iy - 1u) * nx + ix) * 4u + 3u) * 2u + i);
        if (iy < ny && ix > 0u) f += __ldg(fe + ((iy * nx + ix - 1u) * 4u + 1u) * 2u + i);
        if (iy < ny && ix < nx) f += __ldg(fe + ((iy * nx + ix) * 4u + 0u) * 2u + i);
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
