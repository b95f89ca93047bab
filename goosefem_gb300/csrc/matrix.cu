// Assembled sparse matrices on the device: GooseFEM's Matrix and MatrixPartitioned (Matrix.h,
// MatrixPartitioned.h) as CSR. The pattern and, per nonzero, the list of element-matrix entries
// that land on it (in the order Eigen's setFromTriplets sums them: the triplet push order) are
// built once on the host (gfgpu_host_matrix_pattern). Assembly is then a deterministic gather:
// bit-exact in strict mode. Products follow Eigen's column-major sparse x dense product (per row
// a sum from zero in ascending column order); the partitioned product sums the unknown and the
// prescribed columns apart and adds them, as B_u = A_uu X_u + A_up X_p does. The solve of the
// unknown block (MatrixPartitionedSolver, Eigen SimplicialLDLT in the reference) is a Jacobi-PCG
// with fixed-order reductions, replayed as a CUDA graph.
#include "common.cuh"

#include <algorithm>
#include <cmath>

namespace gfgpu {

namespace {

constexpr int kMRed = 1024; // fixed grid of the solver reductions

// MatrixPartitioned.h:156-200 / Matrix.h:704-733 through setFromTriplets: first entry, then +=
template <bool S>
__global__ void k_matrix_assemble(const int32_t* __restrict__ cptr, const int32_t* __restrict__ cidx,
                                  int64_t nnz, const double* __restrict__ elemmat,
                                  double* __restrict__ val)
{
    GF_FOR(k, nnz)
    {
        int32_t q0 = cptr[k], q1 = cptr[k + 1];
        double acc = elemmat[cidx[q0]];
        for (int32_t q = q0 + 1; q < q1; ++q) acc = add<S>(acc, elemmat[cidx[q]]);
        val[k] = acc;
    }
}

// b = A x on dofval (Matrix.h:810-815)
template <bool S>
__global__ void k_matrix_dot(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                             const double* __restrict__ val, int64_t n, const double* __restrict__ x,
                             double* __restrict__ b)
{
    GF_FOR(r, n)
    {
        double acc = 0.0;
        for (int32_t k = rowptr[r]; k < rowptr[r + 1]; ++k) acc = madd<S>(val[k], x[col[k]], acc);
        b[r] = acc;
    }
}

// Partitioned rows [r0, r1): b[iperm[r]] = (A_.u x_u) + (A_.p x_p), x and b dofval in the
// original numbering, iperm[p] = original dof of partitioned index p
// (MatrixPartitioned.h:378-398 dot, :421-433 reaction)
template <bool S>
__global__ void k_matrixp_rows(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                               const double* __restrict__ val, int64_t r0, int64_t r1, int64_t nnu,
                               const int32_t* __restrict__ iperm, const double* __restrict__ x,
                               double* __restrict__ b)
{
    GF_FOR(t, r1 - r0)
    {
        int64_t r = r0 + t;
        double su = 0.0, sp = 0.0;
        for (int32_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
            int32_t c = col[k];
            if (c < nnu) su = madd<S>(val[k], x[iperm[c]], su);
            else sp = madd<S>(val[k], x[iperm[c]], sp);
        }
        b[iperm[r]] = add<S>(su, sp);
    }
}

__device__ __forceinline__ double block_sum(double v, double* sh)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = lane < static_cast<int>(blockDim.x >> 5) ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;
}

// ---------------------------------------------------------------- Jacobi-PCG on A_uu

enum { M_RZ = 0, M_RR, M_PQ, M_BB, M_ALPHA, M_BETA, M_COUNT };

// rhs = b_u - A_up x_p, r = rhs - A_uu x_u, z = D^-1 r, p = z (x_u from x); partials rhs.rhs,
// r.z, r.r
__global__ void __launch_bounds__(256)
k_mp_init(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
          const double* __restrict__ val, int64_t nnu, const int32_t* __restrict__ iperm,
          const double* __restrict__ b, const double* __restrict__ x, double* __restrict__ xu,
          double* __restrict__ dinv, double* __restrict__ r, double* __restrict__ z,
          double* __restrict__ p, double* __restrict__ partial)
{
    __shared__ double sh[32];
    double bb = 0.0, rz = 0.0, rr = 0.0;
    GF_FOR(i, nnu)
    {
        double su = 0.0, sp = 0.0, d = 0.0;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            int32_t c = col[k];
            double xv = x[iperm[c]];
            if (c < nnu) su = fma(val[k], xv, su);
            else sp = fma(val[k], xv, sp);
            if (c == i) d = val[k];
        }
        double rhs = b[iperm[i]] - sp;
        double rv = rhs - su;
        double di = 1.0 / d;
        double zv = di * rv;
        xu[i] = x[iperm[i]];
        dinv[i] = di;
        r[i] = rv;
        z[i] = zv;
        p[i] = zv;
        bb = fma(rhs, rhs, bb);
        rz = fma(rv, zv, rz);
        rr = fma(rv, rv, rr);
    }
    double s0 = block_sum(bb, sh), s1 = block_sum(rz, sh), s2 = block_sum(rr, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = s0;
        partial[kMRed + blockIdx.x] = s1;
        partial[2 * kMRed + blockIdx.x] = s2;
    }
}

// q = A_uu p (the row's columns < nnu; columns are sorted); partial p.q
__global__ void __launch_bounds__(256)
k_mp_spmv(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
          const double* __restrict__ val, int64_t nnu, const double* __restrict__ p,
          double* __restrict__ q, double* __restrict__ partial)
{
    __shared__ double sh[32];
    double pq = 0.0;
    GF_FOR(i, nnu)
    {
        double acc = 0.0;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            int32_t c = col[k];
            if (c >= nnu) break;
            acc = fma(val[k], p[c], acc);
        }
        q[i] = acc;
        pq = fma(p[i], acc, pq);
    }
    double s = block_sum(pq, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// sc[dst0 + row] = fixed-order sum of partial row `row`, rows [0, nrows); with_alpha: then
// alpha = r.z / p.q
__global__ void k_mp_reduce(const double* __restrict__ partial, int nrows, double* __restrict__ sc,
                            int dst0, int with_alpha)
{
    __shared__ double sh[32];
    for (int row = 0; row < nrows; ++row) {
        double v = 0.0;
        for (int i = threadIdx.x; i < kMRed; i += blockDim.x) v += partial[row * kMRed + i];
        double s = block_sum(v, sh);
        if (threadIdx.x == 0) sc[dst0 + row] = s;
        __syncthreads();
    }
    if (threadIdx.x == 0 && with_alpha) sc[M_ALPHA] = sc[M_RZ] / sc[M_PQ];
}

// x_u += alpha p, r -= alpha q, z = D^-1 r; partials r.z, r.r
__global__ void __launch_bounds__(256)
k_mp_update(int64_t nnu, const double* __restrict__ dinv, const double* __restrict__ p,
            const double* __restrict__ q, const double* __restrict__ sc, double* __restrict__ xu,
            double* __restrict__ r, double* __restrict__ z, double* __restrict__ partial)
{
    __shared__ double sh[32];
    double alpha = sc[M_ALPHA];
    double rz = 0.0, rr = 0.0;
    GF_FOR(i, nnu)
    {
        xu[i] = fma(alpha, p[i], xu[i]);
        double rv = fma(-alpha, q[i], r[i]);
        double zv = dinv[i] * rv;
        r[i] = rv;
        z[i] = zv;
        rz = fma(rv, zv, rz);
        rr = fma(rv, rv, rr);
    }
    double s0 = block_sum(rz, sh), s1 = block_sum(rr, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = s0;
        partial[kMRed + blockIdx.x] = s1;
    }
}

// r.z_new, r.r from the update's partials; beta = r.z_new / r.z
__global__ void k_mp_beta(const double* __restrict__ partial, double* __restrict__ sc)
{
    __shared__ double sh[32];
    double v0 = 0.0, v1 = 0.0;
    for (int i = threadIdx.x; i < kMRed; i += blockDim.x) {
        v0 += partial[i];
        v1 += partial[kMRed + i];
    }
    double rz = block_sum(v0, sh);
    double rr = block_sum(v1, sh);
    if (threadIdx.x == 0) {
        sc[M_BETA] = rz / sc[M_RZ];
        sc[M_RZ] = rz;
        sc[M_RR] = rr;
    }
}

__global__ void k_mp_direction(int64_t nnu, const double* __restrict__ z,
                               const double* __restrict__ sc, double* __restrict__ p)
{
    double beta = sc[M_BETA];
    GF_FOR(i, nnu) p[i] = fma(beta, p[i], z[i]);
}

__global__ void k_mp_scatter(int64_t nnu, const int32_t* __restrict__ iperm,
                             const double* __restrict__ xu, double* __restrict__ x)
{
    GF_FOR(i, nnu) x[iperm[i]] = xu[i];
}

// true residual of the unknown block: r = (b_u - A_up x_p) - A_uu x_u; partial r.r
__global__ void __launch_bounds__(256)
k_mp_residual(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
              const double* __restrict__ val, int64_t nnu, const int32_t* __restrict__ iperm,
              const double* __restrict__ b, const double* __restrict__ x,
              double* __restrict__ partial)
{
    __shared__ double sh[32];
    double rr = 0.0;
    GF_FOR(i, nnu)
    {
        double su = 0.0, sp = 0.0;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            int32_t c = col[k];
            if (c < nnu) su = fma(val[k], x[iperm[c]], su);
            else sp = fma(val[k], x[iperm[c]], sp);
        }
        double rv = (b[iperm[i]] - sp) - su;
        rr = fma(rv, rv, rr);
    }
    double s = block_sum(rr, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// ---------------------------------------------------------------- MINRES on a full CSR

// Scalar slots of the MINRES recurrences (Paige & Saunders 1975, preconditioned form).
enum {
    R_BETA = 0, R_OLDB, R_ALFA, R_DBAR, R_EPS, R_OLDEPS, R_CS, R_SN, R_PHI, R_PHIBAR, R_DELTA,
    R_DENOM, R_BETA1, R_BB, R_RR, R_COUNT
};

// v = y / beta; Av = A v - (beta / oldb) r1 (k > 0); partial v.Av -> alfa
__global__ void __launch_bounds__(256)
k_mr_lanczos(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
             const double* __restrict__ val, int64_t n, int64_t clim, const double* __restrict__ sc,
             int first,
             const double* __restrict__ yv, double* __restrict__ v, const double* __restrict__ r1,
             double* __restrict__ yo, double* __restrict__ partial)
{
    __shared__ double sh[32];
    const double s = 1.0 / sc[R_BETA];
    const double c = first ? 0.0 : sc[R_BETA] / sc[R_OLDB];
    double a = 0.0;
    GF_FOR(i, n)
    {
        double acc = 0.0;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
            if (col[k] < clim) acc = fma(val[k], s * yv[col[k]], acc);
        double vi = s * yv[i];
        double yi = first ? acc : fma(-c, r1[i], acc);
        v[i] = vi;
        yo[i] = yi;
        a = fma(vi, yi, a);
    }
    double t = block_sum(a, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// y -= (alfa / beta) r2; r1 = r2; r2 = y; z = Minv r2; partial r2.z
__global__ void __launch_bounds__(256)
k_mr_rotate(int64_t n, const double* __restrict__ sc, const double* __restrict__ minv,
            const double* __restrict__ yo, double* __restrict__ r1, double* __restrict__ r2,
            double* __restrict__ z, double* __restrict__ partial)
{
    __shared__ double sh[32];
    const double c = sc[R_ALFA] / sc[R_BETA];
    double a = 0.0;
    GF_FOR(i, n)
    {
        double yi = fma(-c, r2[i], yo[i]);
        r1[i] = r2[i];
        r2[i] = yi;
        double zi = minv[i] * yi;
        z[i] = zi;
        a = fma(yi, zi, a);
    }
    double t = block_sum(a, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// fixed-order sum of a partial row into sc[slot]; then the scalar step of MINRES (mode 1: after
// alfa; mode 2: after beta_new)
__global__ void k_mr_scalar(const double* __restrict__ partial, double* __restrict__ sc, int mode)
{
    __shared__ double sh[32];
    double a = 0.0;
    for (int i = threadIdx.x; i < kMRed; i += blockDim.x) a += partial[i];
    double t = block_sum(a, sh);
    if (threadIdx.x != 0) return;
    if (mode == 1) {
        sc[R_ALFA] = t;
        return;
    }
    double alfa = sc[R_ALFA];
    double oldb = sc[R_BETA];
    double beta = sqrt(fmax(t, 0.0));
    double oldeps = sc[R_EPS];
    double cs = sc[R_CS], sn = sc[R_SN], dbar = sc[R_DBAR];
    double delta = cs * dbar + sn * alfa;
    double gbar = sn * dbar - cs * alfa;
    double epsln = sn * beta;
    dbar = -cs * beta;
    double gamma = fmax(sqrt(gbar * gbar + beta * beta), 1e-300);
    cs = gbar / gamma;
    sn = beta / gamma;
    double phi = cs * sc[R_PHIBAR];
    sc[R_PHIBAR] = sn * sc[R_PHIBAR];
    sc[R_OLDB] = oldb;
    sc[R_BETA] = beta;
    sc[R_OLDEPS] = oldeps;
    sc[R_EPS] = epsln;
    sc[R_DBAR] = dbar;
    sc[R_CS] = cs;
    sc[R_SN] = sn;
    sc[R_PHI] = phi;
    sc[R_DELTA] = delta;
    sc[R_DENOM] = 1.0 / gamma;
}

// w1 = w2; w2 = w; w = (v - oldeps w1 - delta w2) / gamma; x += phi w; next y = z
__global__ void k_mr_step(int64_t n, const double* __restrict__ sc, const double* __restrict__ v,
                          double* __restrict__ w1, double* __restrict__ w2, double* __restrict__ w,
                          double* __restrict__ x)
{
    const double oe = sc[R_OLDEPS], de = sc[R_DELTA], dn = sc[R_DENOM], ph = sc[R_PHI];
    GF_FOR(i, n)
    {
        double a = w2[i], b = w[i];
        double wn = (v[i] - oe * a - de * b) * dn;
        w1[i] = a;
        w2[i] = b;
        w[i] = wn;
        x[i] = fma(ph, wn, x[i]);
    }
}

// r = b - A x (partial r.r in row 0, b.b in row 1), z = Minv r; minv = 1 / |diag| (1 if 0)
__global__ void __launch_bounds__(256)
k_mr_init(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
          const double* __restrict__ val, int64_t n, int64_t clim, const double* __restrict__ b,
          const double* __restrict__ x, double* __restrict__ minv, double* __restrict__ r,
          double* __restrict__ z, double* __restrict__ partial)
{
    __shared__ double sh[32];
    double rz = 0.0, bb = 0.0;
    GF_FOR(i, n)
    {
        double acc = 0.0, d = 0.0;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            if (col[k] >= clim) continue;
            acc = fma(val[k], x[col[k]], acc);
            if (col[k] == i) d = val[k];
        }
        double mi = d != 0.0 ? 1.0 / fabs(d) : 1.0;
        double ri = b[i] - acc;
        minv[i] = mi;
        r[i] = ri;
        z[i] = mi * ri;
        rz = fma(ri, mi * ri, rz);
        bb = fma(b[i], b[i], bb);
    }
    double t0 = block_sum(rz, sh), t1 = block_sum(bb, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = t0;
        partial[kMRed + blockIdx.x] = t1;
    }
}

__global__ void k_mr_start(const double* __restrict__ partial, double* __restrict__ sc)
{
    __shared__ double sh[32];
    double a = 0.0, c = 0.0;
    for (int i = threadIdx.x; i < kMRed; i += blockDim.x) {
        a += partial[i];
        c += partial[kMRed + i];
    }
    double rz = block_sum(a, sh), bb = block_sum(c, sh);
    if (threadIdx.x == 0) {
        double beta1 = sqrt(fmax(rz, 0.0));
        for (int k = 0; k < R_COUNT; ++k) sc[k] = 0.0;
        sc[R_BETA] = beta1;
        sc[R_BETA1] = beta1;
        sc[R_PHIBAR] = beta1;
        sc[R_CS] = -1.0;
        sc[R_BB] = bb;
    }
}

// true residual: partial ||b - A x||^2
__global__ void __launch_bounds__(256)
k_mr_resid(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
           const double* __restrict__ val, int64_t n, int64_t clim, const double* __restrict__ b,
           const double* __restrict__ x, double* __restrict__ partial)
{
    __shared__ double sh[32];
    double rr = 0.0;
    GF_FOR(i, n)
    {
        double acc = 0.0;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
            if (col[k] < clim) acc = fma(val[k], x[col[k]], acc);
        double ri = b[i] - acc;
        rr = fma(ri, ri, rr);
    }
    double t = block_sum(rr, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

__global__ void k_mr_rr(const double* __restrict__ partial, double* __restrict__ sc)
{
    __shared__ double sh[32];
    double a = 0.0;
    for (int i = threadIdx.x; i < kMRed; i += blockDim.x) a += partial[i];
    double t = block_sum(a, sh);
    if (threadIdx.x == 0) sc[R_RR] = t;
}

// rhs_u = b_u - A_up x_p and x_u from x (original numbering through iperm)
__global__ void k_mp_rhs(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                         const double* __restrict__ val, int64_t nnu, const int32_t* __restrict__ iperm,
                         const double* __restrict__ b, const double* __restrict__ x,
                         double* __restrict__ rhs, double* __restrict__ xu)
{
    GF_FOR(i, nnu)
    {
        double sp = 0.0;
        for (int32_t k = rowptr[i]; k < rowptr[i + 1]; ++k)
            if (col[k] >= nnu) sp = fma(val[k], x[iperm[col[k]]], sp);
        rhs[i] = b[iperm[i]] - sp;
        xu[i] = x[iperm[i]];
    }
}

struct MpWs {
    double *xu, *dinv, *r, *z, *p, *q, *partial, *sc;
};

inline int64_t a256(int64_t b)
{
    return (b + 255) / 256 * 256;
}

inline MpWs carve_mp(int64_t nnu, void* ws)
{
    char* c = static_cast<char*>(ws);
    MpWs w;
    double** v[] = {&w.xu, &w.dinv, &w.r, &w.z, &w.p, &w.q};
    for (auto b : v) {
        *b = reinterpret_cast<double*>(c);
        c += a256(nnu * 8);
    }
    w.partial = reinterpret_cast<double*>(c);
    c += a256(3 * kMRed * 8);
    w.sc = reinterpret_cast<double*>(c);
    return w;
}

} // namespace

} // namespace gfgpu

using namespace gfgpu;

extern "C" {

int gfgpu_matrix_assemble(const int32_t* cptr, const int32_t* cidx, int64_t nnz,
                          const double* elemmat, double* val, gfgpu_stream_t stream)
{
    GF_REQUIRE(cptr && cidx && elemmat && val && nnz >= 0 && !too_big(nnz), "bad argument");
    if (nnz == 0) return GFGPU_OK;
    if (strict_mode())
        k_matrix_assemble<true><<<grid_for(nnz), kBlock, 0, S(stream)>>>(cptr, cidx, nnz, elemmat, val);
    else
        k_matrix_assemble<false><<<grid_for(nnz), kBlock, 0, S(stream)>>>(cptr, cidx, nnz, elemmat, val);
    return check_launch("matrix_assemble");
}

int gfgpu_matrix_dot_dofval(const int32_t* rowptr, const int32_t* col, const double* val, int64_t n,
                            const double* x, double* b, gfgpu_stream_t stream)
{
    GF_REQUIRE(rowptr && col && val && x && b && n >= 0 && !too_big(n), "bad argument");
    if (n == 0) return GFGPU_OK;
    if (strict_mode())
        k_matrix_dot<true><<<grid_for(n), kBlock, 0, S(stream)>>>(rowptr, col, val, n, x, b);
    else
        k_matrix_dot<false><<<grid_for(n), kBlock, 0, S(stream)>>>(rowptr, col, val, n, x, b);
    return check_launch("matrix_dot");
}

static int matrixp_rows(const int32_t* rowptr, const int32_t* col, const double* val, int64_t ndof,
                        int64_t nnu, const int32_t* iperm, const double* x, double* b, int64_t r0,
                        gfgpu_stream_t stream)
{
    GF_REQUIRE(rowptr && col && val && iperm && x && b && nnu >= 0 && nnu <= ndof && !too_big(ndof),
               "bad argument");
    GF_REQUIRE(x != b, "x and b must not alias");
    if (ndof - r0 <= 0) return GFGPU_OK;
    unsigned g = grid_for(ndof - r0);
    if (strict_mode())
        k_matrixp_rows<true><<<g, kBlock, 0, S(stream)>>>(rowptr, col, val, r0, ndof, nnu, iperm, x, b);
    else
        k_matrixp_rows<false><<<g, kBlock, 0, S(stream)>>>(rowptr, col, val, r0, ndof, nnu, iperm, x, b);
    return check_launch("matrixp product");
}

int gfgpu_matrixp_dot_dofval(const int32_t* rowptr, const int32_t* col, const double* val,
                             int64_t ndof, int64_t nnu, const int32_t* iperm, const double* x,
                             double* b, gfgpu_stream_t stream)
{
    return matrixp_rows(rowptr, col, val, ndof, nnu, iperm, x, b, 0, stream);
}

int gfgpu_matrixp_reaction_dofval(const int32_t* rowptr, const int32_t* col, const double* val,
                                  int64_t ndof, int64_t nnu, const int32_t* iperm, const double* x,
                                  double* b, gfgpu_stream_t stream)
{
    return matrixp_rows(rowptr, col, val, ndof, nnu, iperm, x, b, nnu, stream);
}

int64_t gfgpu_matrixp_solve_workspace_bytes(int64_t nnu)
{
    return nnu < 0 ? 0 : 6 * a256(nnu * 8) + a256(3 * kMRed * 8) + a256(M_COUNT * 8);
}

int gfgpu_matrixp_solve(const int32_t* rowptr, const int32_t* col, const double* val, int64_t ndof,
                        int64_t nnu, const int32_t* iperm, const double* b, double* x, double tol,
                        int64_t maxiter, int32_t check_every, void* workspace,
                        gfgpu_stream_t stream, int64_t* iters, double* relres)
{
    GF_REQUIRE(rowptr && col && val && iperm && b && x && workspace && iters && relres,
               "bad argument");
    GF_REQUIRE(nnu > 0 && nnu <= ndof && !too_big(ndof) && tol > 0.0 && maxiter >= 0, "bad argument");
    if (check_every < 1) check_every = 1;
    cudaStream_t s = S(stream);
    MpWs w = carve_mp(nnu, workspace);
    const unsigned gb = kMRed;
    double h[M_COUNT];
    auto read = [&]() -> int {
        GF_TRY(check_cuda(cudaMemcpyAsync(h, w.sc, sizeof(h), cudaMemcpyDeviceToHost, s), "copy"));
        return check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    };
    auto iteration = [&](cudaStream_t st) {
        k_mp_spmv<<<gb, 256, 0, st>>>(rowptr, col, val, nnu, w.p, w.q, w.partial);
        k_mp_reduce<<<1, 1024, 0, st>>>(w.partial, 1, w.sc, M_PQ, 1);
        k_mp_update<<<gb, 256, 0, st>>>(nnu, w.dinv, w.p, w.q, w.sc, w.xu, w.r, w.z, w.partial);
        k_mp_beta<<<1, 1024, 0, st>>>(w.partial, w.sc);
        k_mp_direction<<<grid_for(nnu), kBlock, 0, st>>>(nnu, w.z, w.sc, w.p);
    };
    k_mp_init<<<gb, 256, 0, s>>>(rowptr, col, val, nnu, iperm, b, x, w.xu, w.dinv, w.r, w.z, w.p,
                                 w.partial);
    // rows 0, 1, 2 = rhs.rhs, r.z, r.r -> M_BB, M_RZ, M_RR
    k_mp_reduce<<<1, 1024, 0, s>>>(w.partial, 1, w.sc, M_BB, 0);
    k_mp_reduce<<<1, 1024, 0, s>>>(w.partial + kMRed, 1, w.sc, M_RZ, 0);
    k_mp_reduce<<<1, 1024, 0, s>>>(w.partial + 2 * kMRed, 1, w.sc, M_RR, 0);
    GF_TRY(check_launch("matrixp_solve set-up"));
    GF_TRY(read());
    double bnorm = std::sqrt(h[M_BB]);
    if (bnorm == 0.0) bnorm = 1.0;
    double rel = std::sqrt(h[M_RR]) / bnorm;
    int64_t it = 0;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cs = nullptr;
    int rc = GFGPU_OK;
    while (rel > tol && it < maxiter) {
        int64_t nb = std::min<int64_t>(check_every, maxiter - it);
        if (nb == check_every && !exec) {
            rc = check_cuda(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "cudaStreamCreate");
            cudaGraph_t graph = nullptr;
            if (rc == GFGPU_OK)
                rc = check_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "capture");
            if (rc == GFGPU_OK) {
                for (int64_t k = 0; k < nb; ++k) iteration(cs);
                rc = check_cuda(cudaStreamEndCapture(cs, &graph), "cudaStreamEndCapture");
                if (rc == GFGPU_OK)
                    rc = check_cuda(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
                if (graph) cudaGraphDestroy(graph);
            }
            if (rc != GFGPU_OK) break;
        }
        if (nb == check_every) {
            rc = check_cuda(cudaGraphLaunch(exec, s), "cudaGraphLaunch");
        }
        else {
            for (int64_t k = 0; k < nb; ++k) iteration(s);
            rc = check_launch("matrixp_solve iteration");
        }
        if (rc != GFGPU_OK) break;
        it += nb;
        rc = read();
        if (rc != GFGPU_OK) break;
        if (!std::isfinite(h[M_RR])) {
            rc = fail(GFGPU_ERR_NAN, "gfgpu_matrixp_solve: non-finite residual");
            break;
        }
        rel = std::sqrt(h[M_RR]) / bnorm;
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (cs) cudaStreamDestroy(cs);
    *iters = it;
    GF_TRY(rc);
    k_mp_scatter<<<grid_for(nnu), kBlock, 0, s>>>(nnu, iperm, w.xu, x);
    k_mp_residual<<<gb, 256, 0, s>>>(rowptr, col, val, nnu, iperm, b, x, w.partial);
    k_mp_reduce<<<1, 1024, 0, s>>>(w.partial, 1, w.sc, M_RR, 0);
    GF_TRY(check_launch("matrixp_solve residual"));
    GF_TRY(read());
    *relres = std::sqrt(h[M_RR]) / bnorm;
    if (*relres > tol) return fail(GFGPU_ERR_DIVERGED, "gfgpu_matrixp_solve: tolerance not reached");
    return GFGPU_OK;
}

int64_t gfgpu_matrix_solve_workspace_bytes(int64_t n)
{
    return n < 0 ? 0 : 10 * a256(std::max<int64_t>(n, 1) * 8) + a256(2 * kMRed * 8) + a256(R_COUNT * 8);
}

static int minres_core(const int32_t* rowptr, const int32_t* col, const double* val, int64_t n,
                       int64_t clim, const double* b, double* x, double tol, int64_t maxiter,
                       int32_t check_every, void* workspace, cudaStream_t s, int64_t* iters,
                       double* relres)
{
    if (check_every < 1) check_every = 1;
    char* c = static_cast<char*>(workspace);
    double* vec[10];
    for (auto& p : vec) {
        p = reinterpret_cast<double*>(c);
        c += a256(n * 8);
    }
    double *minv = vec[0], *r1 = vec[1], *r2 = vec[2], *y = vec[3], *v = vec[4], *yo = vec[5],
           *w = vec[6], *w1 = vec[7], *w2 = vec[8];
    double* partial = reinterpret_cast<double*>(c);
    c += a256(2 * kMRed * 8);
    double* sc = reinterpret_cast<double*>(c);
    const unsigned gb = kMRed;
    double h[R_COUNT];
    auto read = [&]() -> int {
        GF_TRY(check_cuda(cudaMemcpyAsync(h, sc, sizeof(h), cudaMemcpyDeviceToHost, s), "copy"));
        return check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    };
    // r1 = r2 = b - A x, y = Minv r1, beta1 = sqrt(r1.y), w = w1 = w2 = 0
    k_mr_init<<<gb, 256, 0, s>>>(rowptr, col, val, n, clim, b, x, minv, r1, y, partial);
    k_mr_start<<<1, 1024, 0, s>>>(partial, sc);
    GF_TRY(check_cuda(cudaMemcpyAsync(r2, r1, n * 8, cudaMemcpyDeviceToDevice, s), "copy"));
    GF_TRY(check_cuda(cudaMemsetAsync(w, 0, n * 8, s), "memset"));
    GF_TRY(check_cuda(cudaMemsetAsync(w1, 0, n * 8, s), "memset"));
    GF_TRY(check_cuda(cudaMemsetAsync(w2, 0, n * 8, s), "memset"));
    GF_TRY(check_launch("matrix_solve set-up"));
    GF_TRY(read());
    double bnorm = std::sqrt(h[R_BB]);
    if (bnorm == 0.0) bnorm = 1.0;
    const double beta1 = h[R_BETA1];
    int64_t it = 0;
    // MINRES (Paige & Saunders) with the SPD preconditioner diag(|A_ii|); phibar estimates the
    // preconditioned residual norm, the exit test uses the true residual
    double rel = beta1 > 0.0 ? 1.0 : 0.0;
    int rc = GFGPU_OK;
    while (rel > tol && it < maxiter) {
        int64_t nb = std::min<int64_t>(check_every, maxiter - it);
        for (int64_t k = 0; k < nb; ++k) {
            k_mr_lanczos<<<gb, 256, 0, s>>>(rowptr, col, val, n, clim, sc, it + k == 0, y, v, r1, yo, partial);
            k_mr_scalar<<<1, 1024, 0, s>>>(partial, sc, 1);
            k_mr_rotate<<<gb, 256, 0, s>>>(n, sc, minv, yo, r1, r2, y, partial);
            k_mr_scalar<<<1, 1024, 0, s>>>(partial, sc, 2);
            k_mr_step<<<grid_for(n), kBlock, 0, s>>>(n, sc, v, w1, w2, w, x);
        }
        it += nb;
        rc = check_launch("matrix_solve iteration");
        if (rc != GFGPU_OK) break;
        rc = read();
        if (rc != GFGPU_OK) break;
        if (!std::isfinite(h[R_PHIBAR])) {
            rc = fail(GFGPU_ERR_NAN, "MINRES: non-finite residual");
            break;
        }
        if (h[R_PHIBAR] <= tol * beta1 || h[R_BETA] == 0.0) {
            k_mr_resid<<<gb, 256, 0, s>>>(rowptr, col, val, n, clim, b, x, partial);
            k_mr_rr<<<1, 1024, 0, s>>>(partial, sc);
            rc = read();
            if (rc != GFGPU_OK) break;
            rel = std::sqrt(h[R_RR]) / bnorm;
            if (h[R_BETA] == 0.0) break; // exact Krylov breakdown: the solution is reached
        }
    }
    *iters = it;
    GF_TRY(rc);
    k_mr_resid<<<gb, 256, 0, s>>>(rowptr, col, val, n, clim, b, x, partial);
    k_mr_rr<<<1, 1024, 0, s>>>(partial, sc);
    GF_TRY(check_launch("matrix_solve residual"));
    GF_TRY(read());
    *relres = std::sqrt(h[R_RR]) / bnorm;
    if (*relres > tol) return fail(GFGPU_ERR_DIVERGED, "MINRES: tolerance not reached");
    return GFGPU_OK;
}


int gfgpu_matrix_solve(const int32_t* rowptr, const int32_t* col, const double* val, int64_t n,
                       const double* b, double* x, double tol, int64_t maxiter, int32_t check_every,
                       void* workspace, gfgpu_stream_t stream, int64_t* iters, double* relres)
{
    GF_REQUIRE(rowptr && col && val && b && x && workspace && iters && relres, "bad argument");
    GF_REQUIRE(n > 0 && !too_big(n) && tol > 0.0 && maxiter >= 0, "bad argument");
    return minres_core(rowptr, col, val, n, n, b, x, tol, maxiter, check_every, workspace, S(stream),
                       iters, relres);
}

int64_t gfgpu_matrixp_solve_minres_workspace_bytes(int64_t nnu)
{
    return nnu < 0 ? 0 : gfgpu_matrix_solve_workspace_bytes(nnu) + 2 * a256(std::max<int64_t>(nnu, 1) * 8);
}

int gfgpu_matrixp_solve_minres(const int32_t* rowptr, const int32_t* col, const double* val,
                               int64_t ndof, int64_t nnu, const int32_t* iperm, const double* b,
                               double* x, double tol, int64_t maxiter, int32_t check_every,
                               void* workspace, gfgpu_stream_t stream, int64_t* iters,
                               double* relres)
{
    GF_REQUIRE(rowptr && col && val && iperm && b && x && workspace && iters && relres,
               "bad argument");
    GF_REQUIRE(nnu > 0 && nnu <= ndof && !too_big(ndof) && tol > 0.0 && maxiter >= 0, "bad argument");
    cudaStream_t s = S(stream);
    char* c = static_cast<char*>(workspace);
    double* rhs = reinterpret_cast<double*>(c);
    c += a256(nnu * 8);
    double* xu = reinterpret_cast<double*>(c);
    c += a256(nnu * 8);
    k_mp_rhs<<<grid_for(nnu), kBlock, 0, s>>>(rowptr, col, val, nnu, iperm, b, x, rhs, xu);
    GF_TRY(check_launch("matrixp_solve_minres rhs"));
    int rc = minres_core(rowptr, col, val, nnu, nnu, rhs, xu, tol, maxiter, check_every, c, s, iters,
                         relres);
    if (rc == GFGPU_OK || rc == GFGPU_ERR_DIVERGED) {
        k_mp_scatter<<<grid_for(nnu), kBlock, 0, s>>>(nnu, iperm, xu, x);
        GF_TRY(check_launch("matrixp_solve_minres scatter"));
    }
    return rc;
}

} // extern "C"
