// Matrix-free Jacobi-preconditioned conjugate gradients for the static linear elastic problem
// with prescribed displacements (the partitioned solve of MatrixPartitionedSolver,
// MatrixPartitioned.h:526-642: A_uu x_u = b_u - A_up x_p), in FP64.
//
// The stiffness action A p is the internal force of the displacement p: the element kernel of
// the explicit step (uniform closed form or general per-Gauss-point path) followed by a dof-CSR
// gather. All vectors are nodevecs [nnode, ndim]; prescribed dofs (part >= nnu) are held at zero
// in p, r, z. Dot products use a fixed grid and a fixed reduction tree, so every run gives the
// same bits. The iteration scalars (alpha, beta) stay on the device; the host reads the residual
// only every `check_every` iterations.
#include <cmath>
#include <vector>

#include "common.cuh"
#include "ffpair.cuh"

namespace gfgpu {

constexpr int kRedBlocks = 1024; // fixed: determinism of the reductions
constexpr int kRedThreads = 256;

// scalar slots
enum { SC_RZ = 0, SC_RZ_NEW, SC_PQ, SC_RR, SC_BB, SC_ALPHA, SC_BETA, SC_COUNT };

__device__ __forceinline__ double block_sum(double v, double* sh)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = lane < (blockDim.x >> 5) ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r; // valid in thread 0
}

// Final fixed-order reduction of `nparts` partial rows (kRedBlocks each) into scalars.
__global__ void k_reduce(const double* __restrict__ partials, int nparts, double* __restrict__ sc,
                         int slot0)
{
    __shared__ double sh[32];
    for (int p = 0; p < nparts; ++p) {
        double v = 0.0;
        for (int i = threadIdx.x; i < kRedBlocks; i += blockDim.x) v += partials[p * kRedBlocks + i];
        double s = block_sum(v, sh);
        if (threadIdx.x == 0) sc[slot0 + p] = s;
        __syncthreads();
    }
}

// q = A p on free dofs (gather of the element forces), 0 on prescribed dofs; partial p.q.
__global__ void __launch_bounds__(kRedThreads)
k_pcg_gather(const int32_t* __restrict__ dofs, const int32_t* __restrict__ ptr,
             const int32_t* __restrict__ idx, const int32_t* __restrict__ part, int64_t nnu,
             const double* __restrict__ fe, const double* __restrict__ p, int64_t n,
             double* __restrict__ q, double* __restrict__ partial, RegGrid reg)
{
    __shared__ double sh[32];
    double acc = 0.0;
    GF_FOR(t, n)
    {
        double f = 0.0;
        if (__ldg(part + t) < nnu) {
            f = gather_dof(t, dofs, ptr, idx, fe, reg);
            acc = fma(p[t], f, acc);
        }
        q[t] = f;
    }
    double s = block_sum(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// p.q from the gather's partial row, then alpha = r.z / p.q (one launch)
__global__ void k_reduce_alpha(const double* __restrict__ partials, double* __restrict__ sc)
{
    __shared__ double sh[32];
    double v = 0.0;
    for (int i = threadIdx.x; i < kRedBlocks; i += blockDim.x) v += partials[i];
    double s = block_sum(v, sh);
    if (threadIdx.x == 0) {
        sc[SC_PQ] = s;
        sc[SC_ALPHA] = sc[SC_RZ] / s;
    }
}

// x += alpha p, r -= alpha q, z = M^-1 r (free dofs); partials r.z and r.r.
__global__ void __launch_bounds__(kRedThreads)
k_pcg_update(const int32_t* __restrict__ part, int64_t nnu, const double* __restrict__ minv,
             const double* __restrict__ p, const double* __restrict__ q, int64_t n,
             const double* __restrict__ sc, double* __restrict__ x, double* __restrict__ r,
             double* __restrict__ z, double* __restrict__ partial)
{
    __shared__ double sh[32];
    double alpha = sc[SC_ALPHA];
    double rz = 0.0, rr = 0.0;
    GF_FOR(t, n)
    {
        if (__ldg(part + t) < nnu) {
            x[t] = fma(alpha, p[t], x[t]);
            double rv = fma(-alpha, q[t], r[t]);
            double zv = minv[t] * rv;
            r[t] = rv;
            z[t] = zv;
            rz = fma(rv, zv, rz);
            rr = fma(rv, rv, rr);
        }
    }
    double s1 = block_sum(rz, sh);
    double s2 = block_sum(rr, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = s1;
        partial[kRedBlocks + blockIdx.x] = s2;
    }
}

// r.z (new) and r.r from the update's partial rows, then beta = r.z_new / r.z (one launch)
__global__ void k_reduce_beta(const double* __restrict__ partials, double* __restrict__ sc)
{
    __shared__ double sh[32];
    double v0 = 0.0, v1 = 0.0;
    for (int i = threadIdx.x; i < kRedBlocks; i += blockDim.x) {
        v0 += partials[i];
        v1 += partials[kRedBlocks + i];
    }
    double rz = block_sum(v0, sh);
    double rr = block_sum(v1, sh);
    if (threadIdx.x == 0) {
        sc[SC_RZ_NEW] = rz;
        sc[SC_RR] = rr;
        sc[SC_BETA] = rz / sc[SC_RZ];
        sc[SC_RZ] = rz;
    }
}

// p = z + beta p
__global__ void k_pcg_direction(const double* __restrict__ z, const double* __restrict__ sc,
                                int64_t n, double* __restrict__ p)
{
    double beta = sc[SC_BETA];
    GF_FOR(t, n) p[t] = fma(beta, p[t], z[t]);
}

// r = -(A x) on free dofs, 0 elsewhere; z = M^-1 r; partials r.z, r.r.
__global__ void __launch_bounds__(kRedThreads)
k_pcg_residual(const int32_t* __restrict__ dofs, const int32_t* __restrict__ ptr,
               const int32_t* __restrict__ idx, const int32_t* __restrict__ part, int64_t nnu,
               const double* __restrict__ fe, const double* __restrict__ b,
               const double* __restrict__ minv, int64_t n, double* __restrict__ r,
               double* __restrict__ z, double* __restrict__ p, double* __restrict__ partial,
               RegGrid reg)
{
    __shared__ double sh[32];
    double rz = 0.0, rr = 0.0;
    GF_FOR(t, n)
    {
        double rv = 0.0, zv = 0.0;
        if (__ldg(part + t) < nnu) {
            const double f = gather_dof(t, dofs, ptr, idx, fe, reg);
            rv = (b ? b[t] : 0.0) - f;
            zv = minv[t] * rv;
            rz = fma(rv, zv, rz);
            rr = fma(rv, rv, rr);
        }
        r[t] = rv;
        z[t] = zv;
        if (p) p[t] = zv;
    }
    double s1 = block_sum(rz, sh);
    double s2 = block_sum(rr, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = s1;
        partial[kRedBlocks + blockIdx.x] = s2;
    }
}

// free dofs of v set to zero (copy of x with the unknowns removed)
__global__ void k_keep_prescribed(const int32_t* __restrict__ part, int64_t nnu,
                                  const double* __restrict__ x, int64_t n, double* __restrict__ o)
{
    GF_FOR(t, n) o[t] = part[t] < nnu ? 0.0 : x[t];
}


// ---------------------------------------------------------------- float-float operator
//
// On a Regular cube Hex8 mesh the iterations can apply A p in pair arithmetic (ffpair.cuh: a value
// is h + l, two FP32 numbers): the FP64 closed form issues ~171 FP64 instructions per element at
// GB300's FP64 rate (~1.7 per SM and clock), the pair form ~1500 FP32 instructions at 128 per SM
// and clock. The direction p stays FP64 (the CG recurrences and dot products need it); the
// direction update also writes it as pairs (pp), the element kernel reads pp and writes pair
// element forces into the fe buffer (8 bytes per value, like a double), and the gather sums a
// dof's forces as pairs and returns the sum to FP64.

// folded coefficient factors as pairs (see gfgpu_internal_hex8_cube_factors) and the grid
struct CubePair {
    float2 a0, a1, c2;
    uint32_t nx, ny, nz;
};

__device__ __forceinline__ ffv pfl(float2 q)
{
    return ff_make(q.x, q.y);
}

__device__ __forceinline__ float2 split_pair(double x)
{
    const ffv p = ff_from_double(x);
    return make_float2(p.h, p.l);
}

// Walsh-Hadamard transform of 8 pairs without the mean (the operator does not use it)
__device__ __forceinline__ void fwht8_nomean_pair(ffv (&v)[8])
{
#pragma unroll
    for (int h = 1; h < 4; h <<= 1)
#pragma unroll
        for (int i = 0; i < 8; ++i)
            if ((i & h) == 0) {
                const ffv a = v[i], b = v[i + h];
                v[i] = ff_add(a, b);
                v[i + h] = ff_sub(a, b);
            }
#pragma unroll
    for (int i = 1; i < 4; ++i) {
        const ffv a = v[i], b = v[i + 4];
        v[i] = ff_add(a, b);
        v[i + 4] = ff_sub(a, b);
    }
    v[4] = ff_sub(v[0], v[4]);
}

// Element forces of the cube closed form (k_elem_force_hex8_cube, the same modes and merges) on
// pairs; element e = (ez ny + ey) nx + ex of Regular(nx, ny, nz), its nodes by index arithmetic;
// fe component-major (fe[(m * 3 + j) * nelem + e], the layout the Regular gather reads).
__global__ void __launch_bounds__(128)
k_elem_force_hex8_cube_pair(const float2* __restrict__ up, const float4* __restrict__ lg, CubePair c,
                            int64_t nelem, float2* __restrict__ fe)
{
    constexpr int pos[8] = {0, 1, 3, 2, 4, 5, 7, 6};
    const uint32_t W = c.nx + 1u, A = W * (c.ny + 1u);
    GF_FOR(e, nelem)
    {
        const uint32_t ee = static_cast<uint32_t>(e), t = ee / c.nx, ex = ee - t * c.nx;
        const uint32_t ez = t / c.ny, ey = t - ez * c.ny;
        const uint32_t n0 = ez * A + ey * W + ex;
        // binary order b = bx + 2 by + 4 bz
        ffv H[3][8];
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            const float2* un = up + static_cast<int64_t>(n0 + (b & 1) + ((b >> 1) & 1) * W + (b >> 2) * A) * 3;
            H[0][b] = pfl(__ldg(un));
            H[1][b] = pfl(__ldg(un + 1));
            H[2][b] = pfl(__ldg(un + 2));
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            fwht8_nomean_pair(H[j]);
#pragma unroll
            for (int b = 1; b < 8; ++b) H[j][b] = ff_norm(H[j][b]);
        }
        const float4 q = __ldg(lg + e);
        const ffv lam = ff_make(q.x, q.y), G = ff_make(q.z, q.w);
        const ffv L0 = ff_mul(pfl(c.a0), lam), G0 = ff_mul(pfl(c.a0), G), G0x2 = ff_twice(G0);
        const ffv L1 = ff_mul(pfl(c.a1), lam), G1 = ff_mul(pfl(c.a1), G), G1x2 = ff_twice(G1);
        const ffv G1x3 = ff_add(G1x2, G1);
        const ffv kH = ff_mul(pfl(c.c2), ff_add(lam, ff_twice(ff_twice(G))));
        // modes (A1 = -H1, A2 = -H2, A3 = -H4, A4 = H3, A5 = H6, A6 = H5, A7 = -H7)
        ffv A1[3], A2[3], A3[3], A4[3], A5[3], A6[3], A7[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            A1[j] = ff_neg(H[j][1]);
            A2[j] = ff_neg(H[j][2]);
            A4[j] = H[j][3];
            A3[j] = ff_neg(H[j][4]);
            A6[j] = H[j][5];
            A5[j] = H[j][6];
            A7[j] = ff_neg(H[j][7]);
        }
        ffv F[8][3];
        {
            const ffv Lt = ff_mul(L0, ff_add(ff_add(A1[0], A2[1]), A3[2]));
            F[1][0] = ff_add(ff_mul(G0x2, A1[0]), Lt);
            F[2][1] = ff_add(ff_mul(G0x2, A2[1]), Lt);
            F[3][2] = ff_add(ff_mul(G0x2, A3[2]), Lt);
            const ffv s01 = ff_mul(G0, ff_add(A1[1], A2[0]));
            const ffv s02 = ff_mul(G0, ff_add(A1[2], A3[0]));
            const ffv s12 = ff_mul(G0, ff_add(A2[2], A3[1]));
            F[1][1] = s01;
            F[2][0] = s01;
            F[1][2] = s02;
            F[3][0] = s02;
            F[2][2] = s12;
            F[3][1] = s12;
        }
        {
            const ffv Lxi = ff_mul(L1, ff_add(A4[1], A6[2]));
            const ffv Let = ff_mul(L1, ff_add(A4[0], A5[2]));
            const ffv Lze = ff_mul(L1, ff_add(A6[0], A5[1]));
            F[4][0] = ff_add(ff_mul(G1x3, A4[0]), Let);
            F[4][1] = ff_add(ff_mul(G1x3, A4[1]), Lxi);
            F[4][2] = ff_add(ff_mul(G1x2, A4[2]), ff_mul(G1, ff_add(A5[0], A6[1])));
            F[5][0] = ff_add(ff_mul(G1x2, A5[0]), ff_mul(G1, ff_add(A6[1], A4[2])));
            F[5][1] = ff_add(ff_mul(G1x3, A5[1]), Lze);
            F[5][2] = ff_add(ff_mul(G1x3, A5[2]), Let);
            F[6][0] = ff_add(ff_mul(G1x3, A6[0]), Lze);
            F[6][1] = ff_add(ff_mul(G1x2, A6[1]), ff_mul(G1, ff_add(A5[0], A4[2])));
            F[6][2] = ff_add(ff_mul(G1x3, A6[2]), Lxi);
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) F[7][j] = ff_mul(kH, A7[j]);
        // inverse transform of (0, -F1, -F2, F4, -F3, F6, F5, -F7) in binary order
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const ffv b1 = ff_neg(F[1][j]);
            ffv v[8] = {b1, F[1][j], ff_sub(F[4][j], F[2][j]), ff_neg(ff_add(F[2][j], F[4][j])),
                        ff_sub(F[6][j], F[3][j]), ff_neg(ff_add(F[3][j], F[6][j])),
                        ff_sub(F[5][j], F[7][j]), ff_add(F[5][j], F[7][j])};
#pragma unroll
            for (int h = 2; h < 8; h <<= 1)
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    if ((i & h) == 0) {
                        const ffv a = v[i], b = v[i + h];
                        v[i] = ff_add(a, b);
                        v[i + h] = ff_sub(a, b);
                    }
#pragma unroll
            for (int m = 0; m < 8; ++m) {
                const ffv o = v[pos[m]];
                fe[(m * 3 + j) * nelem + e] = make_float2(o.h, o.l);
            }
        }
    }
}

// q = A p on free dofs from the pair element forces (the Regular Hex8 gather order of gather_dof,
// summed as pairs, returned to FP64), 0 on prescribed dofs; partial p.q in FP64.
__global__ void __launch_bounds__(kRedThreads)
k_pcg_gather_pair(const int32_t* __restrict__ part, int64_t nnu, const float2* __restrict__ fe,
                  const double* __restrict__ p, int64_t n, double* __restrict__ q,
                  double* __restrict__ partial, RegGrid reg)
{
    __shared__ double sh[32];
    double acc = 0.0;
    const uint32_t nx = static_cast<uint32_t>(reg.nx), ny = static_cast<uint32_t>(reg.ny);
    const uint32_t nz = static_cast<uint32_t>(reg.nz), cs = nx * ny * nz;
    const uint32_t W = nx + 1u, A = W * (ny + 1u);
    GF_FOR(t, n)
    {
        double fv = 0.0;
        if (__ldg(part + t) < nnu) {
            const uint32_t tt = static_cast<uint32_t>(t), node = tt / 3u, i = tt - node * 3u;
            const uint32_t iz = node / A, rem = node - iz * A, iy = rem / W, ix = rem - iy * W;
            ffv f = ff_make(0.0f, 0.0f);
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
                        f = ff_add(f, pfl(__ldg(fe + e + (m * 3u + i) * cs)));
                    }
                }
            }
            fv = ff_to_double(f);
            acc = fma(p[t], fv, acc);
        }
        q[t] = fv;
    }
    double s = block_sum(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// p = z + beta p, and p as pairs
__global__ void k_pcg_direction_pair(const double* __restrict__ z, const double* __restrict__ sc,
                                     int64_t n, double* __restrict__ p, float2* __restrict__ pp)
{
    double beta = sc[SC_BETA];
    GF_FOR(t, n)
    {
        const double v = fma(beta, p[t], z[t]);
        p[t] = v;
        pp[t] = split_pair(v);
    }
}

__global__ void k_pcg_split(const double* __restrict__ p, int64_t n, float2* __restrict__ pp)
{
    GF_FOR(t, n) pp[t] = split_pair(p[t]);
}

// {lam, G} per element as pairs, lam = K - 2G/3 (the FP64 expression of k_hex8_cube_coef)
__global__ void k_pcg_pair_coef(const double* __restrict__ Km, const double* __restrict__ Gm,
                                int64_t nelem, float4* __restrict__ out)
{
    GF_FOR(e, nelem)
    {
        const double G = Gm[e], lam = Km[e] - 2.0 * G / 3.0;
        const float2 a = split_pair(lam), b = split_pair(G);
        out[e] = make_float4(a.x, a.y, b.x, b.y);
    }
}

// which pair operator applies: 1 = Regular cube Hex8 mesh with the index-arithmetic gather
// (component-major fe; pair element kernel, pair gather), 2 = uniform square Quad4 mesh (pair
// element kernel with FP64 input and output, the FP64 gathers); 0 = none
inline int pcg_pair_kind(const gfgpu_verlet_desc* d)
{
    if (d->nelem > 0 && reg_grid(d).soa && d->reg_nx * d->reg_ny * d->reg_nz == d->nelem) return 1;
    if (d->nelem > 0 && d->uniform && d->nne == 4 && d->ndim == 2 && d->coef) return 2;
    return 0;
}

// Jacobi: diagonal of the element stiffness per (element, node, direction) for isotropic
// linear elasticity, K_e[(m,j),(m,j)] = sum_q vol (lam dNx(m,j)^2 + G dNx(m,j)^2 + G |dNx(m,:)|^2).
template <int NNE, int ND>
__global__ void k_elem_diag(const double* __restrict__ dNx, const double* __restrict__ vol,
                            const double* __restrict__ Km, const double* __restrict__ Gm,
                            int64_t nelem, int nip, double* __restrict__ out)
{
    GF_FOR(t, nelem * NNE)
    {
        int64_t e = t / NNE;
        int m = static_cast<int>(t - e * NNE);
        double G = Gm[e], lam = Km[e] - 2.0 * G / 3.0;
        double acc[ND];
#pragma unroll
        for (int j = 0; j < ND; ++j) acc[j] = 0.0;
        for (int q = 0; q < nip; ++q) {
            const double* g = dNx + ((e * nip + q) * NNE + m) * ND;
            double v = vol[e * nip + q];
            double n2 = 0.0;
#pragma unroll
            for (int k = 0; k < ND; ++k) n2 += g[k] * g[k];
#pragma unroll
            for (int j = 0; j < ND; ++j) acc[j] += v * ((lam + G) * g[j] * g[j] + G * n2);
        }
#pragma unroll
        for (int j = 0; j < ND; ++j) out[t * ND + j] = acc[j];
    }
}

__global__ void k_inv_free(const int32_t* __restrict__ part, int64_t nnu,
                           const double* __restrict__ diag, int64_t n, double* __restrict__ minv)
{
    GF_FOR(t, n) minv[t] = part[t] < nnu ? 1.0 / diag[t] : 0.0;
}

struct PcgWs {
    double *fe, *p, *r, *z, *q, *minv, *bvec, *partial, *sc;
    float2* pp; // the direction as pairs (pair operator)
};

static int64_t align256(int64_t b)
{
    return (b + 255) / 256 * 256;
}

static PcgWs carve(const gfgpu_verlet_desc* d, void* ws)
{
    char* c = static_cast<char*>(ws);
    int64_t n = d->nnode * d->ndim;
    PcgWs w;
    w.fe = reinterpret_cast<double*>(c);
    c += align256(d->nelem * d->nne * d->ndim * 8);
    double** vecs[] = {&w.p, &w.r, &w.z, &w.q, &w.minv, &w.bvec};
    for (auto v : vecs) {
        *v = reinterpret_cast<double*>(c);
        c += align256(n * 8);
    }
    w.partial = reinterpret_cast<double*>(c);
    c += align256(2 * kRedBlocks * 8);
    w.sc = reinterpret_cast<double*>(c);
    c += align256(SC_COUNT * 8 + 64);
    w.pp = reinterpret_cast<float2*>(c);
    return w;
}

static int64_t pcg_bytes(const gfgpu_verlet_desc* d)
{
    int64_t n = d->nnode * d->ndim;
    return align256(d->nelem * d->nne * d->ndim * 8) + 6 * align256(n * 8) +
           align256(2 * kRedBlocks * 8) + align256(SC_COUNT * 8 + 64) + align256(n * 8);
}

} // namespace gfgpu

using namespace gfgpu;

// element kernel launch shared with the explicit step (dynamics.cu)
int gfgpu_internal_element_forces(const gfgpu_verlet_desc* d, const double* u, double* fe,
                                  cudaStream_t s);
void gfgpu_internal_hex8_cube_factors(const gfgpu_verlet_desc* d, double* a0, double* a1, double* c2);
// the uniform square Quad4 pair operator (verlet_pair.cu)
int gfgpu_internal_pair_element_forces_f64(const gfgpu_verlet_desc* d, const double* u, double* fe,
                                           cudaStream_t s);
int gfgpu_internal_pair_coef_square(const gfgpu_verlet_desc* d, float* coef, cudaStream_t s);

// Element forces of an iteration's search direction: the Quad4 pair operator when d->pcg_pair is set
// on a square Quad4 mesh, else the FP64 element kernel (also used by the flexible CG, learned.cu).
int gfgpu_internal_iteration_element_forces(const gfgpu_verlet_desc* d, const double* u, double* fe,
                                            cudaStream_t s)
{
    if (d->pcg_pair && pcg_pair_kind(d) == 2) return gfgpu_internal_pair_element_forces_f64(d, u, fe, s);
    return gfgpu_internal_element_forces(d, u, fe, s);
}

extern "C" {

int64_t gfgpu_pcg_workspace_bytes(const gfgpu_verlet_desc* d)
{
    return d ? pcg_bytes(d) : 0;
}

int64_t gfgpu_pcg_pair_coef_floats(const gfgpu_verlet_desc* d)
{
    if (!d) return 0;
    const int k = pcg_pair_kind(d);
    return k == 1 ? 4 * d->nelem : (k == 2 ? 6 * d->nelem : 0);
}

int gfgpu_pcg_precompute_pair(gfgpu_verlet_desc* d, float* coef, gfgpu_stream_t stream)
{
    GF_REQUIRE(d && coef && d->K && d->G, "bad argument");
    GF_REQUIRE(reinterpret_cast<uintptr_t>(coef) % 16 == 0, "coef must be 16-byte aligned");
    const int kind = pcg_pair_kind(d);
    if (kind == 0)
        return fail(GFGPU_ERR_UNSUPPORTED, "gfgpu_pcg_precompute_pair: Regular cube Hex8 meshes with the "
                                           "index-arithmetic gather or uniform square Quad4 meshes only");
    if (kind == 1) {
        k_pcg_pair_coef<<<grid_for(d->nelem), kBlock, 0, S(stream)>>>(d->K, d->G, d->nelem,
                                                                      reinterpret_cast<float4*>(coef));
        GF_TRY(check_launch("pcg_precompute_pair"));
    }
    else {
        GF_TRY(gfgpu_internal_pair_coef_square(d, coef, S(stream)));
    }
    d->pcg_pair = coef;
    return GFGPU_OK;
}

int gfgpu_elastic_diagonal(const gfgpu_verlet_desc* d, double* diag, void* workspace,
                           gfgpu_stream_t stream)
{
    GF_REQUIRE(d && diag && workspace && d->dNx && d->vol, "bad argument (needs dNx and vol)");
    GF_REQUIRE((d->nne == 4 && d->ndim == 2) || (d->nne == 8 && d->ndim == 3), "Quad4 / Hex8 only");
    double* fe = static_cast<double*>(workspace);
    cudaStream_t s = S(stream);
    if (d->nne == 4)
        k_elem_diag<4, 2><<<grid_for(d->nelem * 4), kBlock, 0, s>>>(d->dNx, d->vol, d->K, d->G,
                                                                   d->nelem, d->nip, fe);
    else
        k_elem_diag<8, 3><<<grid_for(d->nelem * 8), kBlock, 0, s>>>(d->dNx, d->vol, d->K, d->G,
                                                                   d->nelem, d->nip, fe);
    GF_TRY(check_launch("elastic_diagonal"));
    return gfgpu_assemble_node(d->csr_ptr, d->csr_idx, d->dofs, d->nnode, d->ndim, fe, diag, stream);
}

static CubePair cube_pair(const gfgpu_verlet_desc* d)
{
    double a0, a1, c2;
    gfgpu_internal_hex8_cube_factors(d, &a0, &a1, &c2);
    auto sp = [](double x) {
        const float h = static_cast<float>(x);
        return make_float2(h, static_cast<float>(x - static_cast<double>(h)));
    };
    CubePair c;
    c.a0 = sp(a0);
    c.a1 = sp(a1);
    c.c2 = sp(c2);
    c.nx = static_cast<uint32_t>(d->reg_nx);
    c.ny = static_cast<uint32_t>(d->reg_ny);
    c.nz = static_cast<uint32_t>(d->reg_nz);
    return c;
}

// One Jacobi-PCG iteration: 6 launches (element forces, gather, alpha, update, beta, direction);
// with d->pcg_pair the element forces and the gather run on pairs and the direction update also
// writes the pair copy of p that the next iteration's element kernel reads.
static int pcg_iteration(const gfgpu_verlet_desc* d, const PcgWs& w, double* x, int64_t n,
                         cudaStream_t s)
{
    const unsigned gb = kRedBlocks;
    const bool pair = d->pcg_pair != nullptr && d->nne == 8;
    if (pair) {
        k_elem_force_hex8_cube_pair<<<grid_for(d->nelem, 128), 128, 0, s>>>(
            w.pp, reinterpret_cast<const float4*>(d->pcg_pair), cube_pair(d), d->nelem,
            reinterpret_cast<float2*>(w.fe));
        k_pcg_gather_pair<<<gb, kRedThreads, 0, s>>>(d->part, d->nnu, reinterpret_cast<const float2*>(w.fe),
                                                      w.p, n, w.q, w.partial, reg_grid(d));
    }
    else {
        GF_TRY(gfgpu_internal_iteration_element_forces(d, w.p, w.fe, s));
        k_pcg_gather<<<gb, kRedThreads, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe,
                                                 w.p, n, w.q, w.partial, reg_grid(d));
    }
    k_reduce_alpha<<<1, 1024, 0, s>>>(w.partial, w.sc);
    k_pcg_update<<<gb, kRedThreads, 0, s>>>(d->part, d->nnu, w.minv, w.p, w.q, n, w.sc, x, w.r, w.z,
                                             w.partial);
    k_reduce_beta<<<1, 1024, 0, s>>>(w.partial, w.sc);
    if (pair)
        k_pcg_direction_pair<<<grid_for(n), kBlock, 0, s>>>(w.z, w.sc, n, w.p, w.pp);
    else
        k_pcg_direction<<<grid_for(n), kBlock, 0, s>>>(w.z, w.sc, n, w.p);
    return GFGPU_OK;
}

// the pair operator's validity (the caller may have changed the descriptor since the precompute)
static int pcg_pair_check(const gfgpu_verlet_desc* d)
{
    if (d->pcg_pair && pcg_pair_kind(d) == 0)
        return fail(GFGPU_ERR_UNSUPPORTED, "pcg_pair is set but the mesh is neither a Regular cube Hex8 mesh "
                                           "with the index-arithmetic gather nor a uniform square Quad4 mesh");
    return GFGPU_OK;
}

int gfgpu_pcg_solve(const gfgpu_verlet_desc* d, const double* diag, double* x, double tol,
                    int64_t maxiter, int32_t check_every, void* workspace, gfgpu_stream_t stream,
                    int64_t* iters, double* relres)
{
    GF_REQUIRE(d && diag && x && workspace && iters && relres && tol > 0.0 && maxiter >= 0,
               "bad argument");
    GF_REQUIRE(d->part && d->conn && d->csr_ptr && d->csr_idx && d->dofs && d->K && d->G,
               "null table");
    GF_TRY(pcg_pair_check(d));
    if (check_every < 1) check_every = 1;
    cudaStream_t s = S(stream);
    PcgWs w = carve(d, workspace);
    int64_t n = d->nnode * d->ndim;
    const unsigned gb = kRedBlocks;
    double* hsc = nullptr;
    GF_TRY(check_cuda(cudaMallocHost(&hsc, SC_COUNT * sizeof(double)), "cudaMallocHost"));
    int rc = GFGPU_OK;
    auto fail_out = [&](int code) {
        cudaFreeHost(hsc);
        return code;
    };
    k_inv_free<<<grid_for(n), kBlock, 0, s>>>(d->part, d->nnu, diag, n, w.minv);
    // b = -(A x_p) on the free dofs
    k_keep_prescribed<<<grid_for(n), kBlock, 0, s>>>(d->part, d->nnu, x, n, w.p);
    if ((rc = gfgpu_internal_element_forces(d, w.p, w.fe, s)) != GFGPU_OK) return fail_out(rc);
    k_pcg_residual<<<gb, kRedThreads, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe,
                                               nullptr, w.minv, n, w.bvec, w.z, nullptr, w.partial, reg_grid(d));
    k_reduce<<<1, 1024, 0, s>>>(w.partial + kRedBlocks, 1, w.sc, SC_BB);
    // r = b - A x, z = M^-1 r, p = z
    if ((rc = gfgpu_internal_element_forces(d, x, w.fe, s)) != GFGPU_OK) return fail_out(rc);
    k_pcg_residual<<<gb, kRedThreads, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe,
                                               nullptr, w.minv, n, w.r, w.z, w.p, w.partial, reg_grid(d));
    k_reduce<<<1, 1024, 0, s>>>(w.partial, 2, w.sc, SC_RZ); // SC_RZ, SC_RZ_NEW(=rr, overwritten)
    if (d->pcg_pair && d->nne == 8) k_pcg_split<<<grid_for(n), kBlock, 0, s>>>(w.p, n, w.pp);
    if ((rc = check_launch("pcg set-up")) != GFGPU_OK) return fail_out(rc);
    cudaMemcpyAsync(hsc, w.sc, SC_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s);
    if ((rc = check_cuda(cudaStreamSynchronize(s), "pcg set-up")) != GFGPU_OK) return fail_out(rc);
    double bb = hsc[SC_BB];
    double rr = hsc[SC_RZ_NEW];
    double bnorm = std::sqrt(bb);
    if (bnorm == 0.0) bnorm = 1.0;
    int64_t it = 0;
    double rel = std::sqrt(rr) / bnorm;
    // check_every iterations replay as one CUDA graph (captured on a private stream, launched on
    // the caller's); a remainder shorter than that runs eagerly
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cs = nullptr;
    auto release = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (cs) cudaStreamDestroy(cs);
        exec = nullptr;
        cs = nullptr;
    };
    while (rel > tol && it < maxiter) {
        int64_t nb = std::min<int64_t>(check_every, maxiter - it);
        if (nb == check_every && !exec) {
            rc = check_cuda(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "cudaStreamCreate");
            cudaGraph_t graph = nullptr;
            if (rc == GFGPU_OK)
                rc = check_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "capture");
            if (rc == GFGPU_OK) {
                int crc = GFGPU_OK;
                for (int64_t k = 0; k < nb && crc == GFGPU_OK; ++k) crc = pcg_iteration(d, w, x, n, cs);
                cudaError_t e = cudaStreamEndCapture(cs, &graph);
                rc = crc != GFGPU_OK ? crc : check_cuda(e, "cudaStreamEndCapture");
                if (rc == GFGPU_OK)
                    rc = check_cuda(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
                if (graph) cudaGraphDestroy(graph);
            }
            if (rc != GFGPU_OK) {
                release();
                return fail_out(rc);
            }
        }
        if (nb == check_every) {
            rc = check_cuda(cudaGraphLaunch(exec, s), "cudaGraphLaunch");
        }
        else {
            for (int64_t k = 0; k < nb && rc == GFGPU_OK; ++k) rc = pcg_iteration(d, w, x, n, s);
        }
        if (rc != GFGPU_OK) {
            release();
            return fail_out(rc);
        }
        it += nb;
        if ((rc = check_launch("pcg iteration")) != GFGPU_OK) {
            release();
            return fail_out(rc);
        }
        cudaMemcpyAsync(hsc, w.sc, SC_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s);
        if ((rc = check_cuda(cudaStreamSynchronize(s), "pcg iteration")) != GFGPU_OK) {
            release();
            return fail_out(rc);
        }
        rr = hsc[SC_RR];
        if (!std::isfinite(rr)) {
            release();
            *iters = it;
            *relres = rr;
            return fail_out(fail(GFGPU_ERR_NAN, "gfgpu_pcg_solve: non-finite residual"));
        }
        rel = std::sqrt(rr) / bnorm;
    }
    release();
    // true residual of the partitioned system: b_u - A_uu x_u = -(A x)_u, x holding x_p as well
    if ((rc = gfgpu_internal_element_forces(d, x, w.fe, s)) != GFGPU_OK) return fail_out(rc);
    k_pcg_residual<<<gb, kRedThreads, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe,
                                               nullptr, w.minv, n, w.r, w.z, nullptr, w.partial, reg_grid(d));
    k_reduce<<<1, 1024, 0, s>>>(w.partial + kRedBlocks, 1, w.sc, SC_RR);
    cudaMemcpyAsync(hsc, w.sc, SC_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s);
    if ((rc = check_cuda(cudaStreamSynchronize(s), "pcg final residual")) != GFGPU_OK)
        return fail_out(rc);
    *iters = it;
    *relres = std::sqrt(hsc[SC_RR]) / bnorm;
    cudaFreeHost(hsc);
    if (*relres > tol) return fail(GFGPU_ERR_DIVERGED, "gfgpu_pcg_solve: tolerance not reached");
    return GFGPU_OK;
}

// ---------------------------------------------------------------- step-by-step session

int gfgpu_pcg_begin(const gfgpu_verlet_desc* d, const double* diag, const double* rhs,
                    const double* x, void* workspace, gfgpu_stream_t stream)
{
    GF_REQUIRE(d && diag && x && workspace, "bad argument");
    GF_TRY(pcg_pair_check(d));
    cudaStream_t s = S(stream);
    PcgWs w = carve(d, workspace);
    int64_t n = d->nnode * d->ndim;
    const unsigned gb = kRedBlocks;
    k_inv_free<<<grid_for(n), kBlock, 0, s>>>(d->part, d->nnu, diag, n, w.minv);
    // b = rhs_u - (A x_p)_u
    k_keep_prescribed<<<grid_for(n), kBlock, 0, s>>>(d->part, d->nnu, x, n, w.p);
    GF_TRY(gfgpu_internal_element_forces(d, w.p, w.fe, s));
    k_pcg_residual<<<gb, kRedThreads, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe,
                                               rhs, w.minv, n, w.bvec, w.z, nullptr, w.partial, reg_grid(d));
    k_reduce<<<1, 1024, 0, s>>>(w.partial + kRedBlocks, 1, w.sc, SC_BB);
    // r = rhs_u - (A x)_u, z = M^-1 r, p = z
    GF_TRY(gfgpu_internal_element_forces(d, x, w.fe, s));
    k_pcg_residual<<<gb, kRedThreads, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part, d->nnu, w.fe,
                                               rhs, w.minv, n, w.r, w.z, w.p, w.partial, reg_grid(d));
    k_reduce<<<1, 1024, 0, s>>>(w.partial, 2, w.sc, SC_RZ); // SC_RZ = r.z, SC_RZ_NEW = r.r
    k_reduce<<<1, 1024, 0, s>>>(w.partial + kRedBlocks, 1, w.sc, SC_RR);
    if (d->pcg_pair && d->nne == 8) k_pcg_split<<<grid_for(n), kBlock, 0, s>>>(w.p, n, w.pp);
    return check_launch("pcg_begin");
}

int gfgpu_pcg_iterate(const gfgpu_verlet_desc* d, int64_t niter, double* x, void* workspace,
                      gfgpu_stream_t stream)
{
    GF_REQUIRE(d && x && workspace && niter >= 0, "bad argument");
    GF_TRY(pcg_pair_check(d));
    cudaStream_t s = S(stream);
    PcgWs w = carve(d, workspace);
    int64_t n = d->nnode * d->ndim;
    for (int64_t k = 0; k < niter; ++k) GF_TRY(pcg_iteration(d, w, x, n, s));
    return check_launch("pcg_iterate");
}

int gfgpu_pcg_vector(const gfgpu_verlet_desc* d, void* workspace, int32_t which, double** ptr)
{
    GF_REQUIRE(d && workspace && ptr && which >= 0 && which <= 3, "bad argument");
    PcgWs w = carve(d, workspace);
    double* const v[4] = {w.r, w.z, w.p, w.q};
    *ptr = v[which];
    return GFGPU_OK;
}

int gfgpu_pcg_norms(const gfgpu_verlet_desc* d, const void* workspace, double* rr, double* bb,
                    gfgpu_stream_t stream)
{
    GF_REQUIRE(d && workspace && rr && bb, "bad argument");
    PcgWs w = carve(d, const_cast<void*>(workspace));
    double h[SC_COUNT];
    GF_TRY(check_cuda(cudaMemcpyAsync(h, w.sc, sizeof(h), cudaMemcpyDeviceToHost, S(stream)),
                      "cudaMemcpyAsync"));
    GF_TRY(check_cuda(cudaStreamSynchronize(S(stream)), "cudaStreamSynchronize"));
    *rr = h[SC_RR];
    *bb = h[SC_BB];
    return GFGPU_OK;
}

} // extern "C"
