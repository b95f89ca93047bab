// Periodic tyings (GooseFEM Tyings::Periodic, VectorPartitionedTyings, MatrixPartitionedTyings;
// TyingsPeriodic.h, VectorPartitionedTyings.h, MatrixPartitionedTyings.h) on the device.
//
// The dofs are renumbered on the host as [u (independent unknown), p (independent prescribed),
// d (dependent)] (gfgpu_host_tyings_periodic) and the tying matrix u_d = C_di u_i is kept as CSR
// (gfgpu_host_tyings_cdi) together with its transpose C_id (gfgpu_host_csr_transpose). The
// system matrix is the assembled CSR of matrix.cu in that numbering, so its nine blocks are index
// ranges. The condensed operator of MatrixPartitionedTyingsSolver,
//   A_uu + A_ud C_du + C_ud A_du + C_ud A_dd C_du,
// is applied matrix-free from those blocks (w = C_du x_u; t = A [x_u; 0; w]; y = t_u + C_ud t_d)
// inside a Jacobi-PCG whose diagonal is the exact diagonal of the condensed matrix.
#include "common.cuh"

#include <algorithm>
#include <cmath>

namespace gfgpu {

namespace {

constexpr int kTRed = 1024; // fixed grid of the solver reductions

// out[d - lo] = x[t] for the nodevec entries t whose (renumbered) dof d is in [lo, hi)
__global__ void k_ty_to_dofval(const int32_t* __restrict__ tdofs, int64_t n,
                               const double* __restrict__ x, int64_t lo, int64_t hi,
                               double* __restrict__ out)
{
    GF_FOR(t, n)
    {
        int64_t d = tdofs[t];
        if (d >= lo && d < hi) out[d - lo] = x[t];
    }
}

// y[r] (mode 0: =, 1: y +, 2: y -) sum over the row's columns c in [clo, chi) of val x[c - cshift],
// from 0 in ascending column order (Eigen's column-major sparse x dense product)
template <bool S>
__global__ void k_ty_spmv(const int32_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                          const double* __restrict__ val, int64_t row0, int64_t nrow, int64_t clo,
                          int64_t chi, int64_t cshift, const double* __restrict__ x, int mode,
                          double* __restrict__ y)
{
    GF_FOR(t, nrow)
    {
        int64_t r = row0 + t;
        double acc = 0.0;
        for (int32_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
            int64_t c = col[k];
            if (c >= clo && c < chi) acc = madd<S>(val[k], x[c - cshift], acc);
        }
        y[t] = mode == 0 ? acc : (mode == 1 ? add<S>(y[t], acc) : sub<S>(y[t], acc));
    }
}

// value of (r, c) in a CSR with sorted columns (0 if absent)
__device__ __forceinline__ double csr_at(const int32_t* __restrict__ rowptr,
                                         const int32_t* __restrict__ col,
                                         const double* __restrict__ val, int64_t r, int64_t c)
{
    int32_t lo = rowptr[r], hi = rowptr[r + 1];
    while (lo < hi) {
        int32_t mid = (lo + hi) >> 1;
        if (col[mid] < c) lo = mid + 1;
        else hi = mid;
    }
    return (lo < rowptr[r + 1] && col[lo] == c) ? val[lo] : 0.0;
}

// 1 / diagonal of the condensed matrix: A_ii + sum_d C_di (A_i,d + A_d,i) + sum_dd' C_di A_dd' C_d'i
__global__ void k_ty_dinv(const int32_t* __restrict__ arow, const int32_t* __restrict__ acol,
                          const double* __restrict__ aval, const int32_t* __restrict__ crow,
                          const int32_t* __restrict__ ccol, const double* __restrict__ cval,
                          int64_t nnu, int64_t nni, double* __restrict__ dinv)
{
    GF_FOR(i, nnu)
    {
        double d = csr_at(arow, acol, aval, i, i);
        for (int32_t k = crow[i]; k < crow[i + 1]; ++k) {
            int64_t dd = ccol[k];
            double c = cval[k];
            d += c * (csr_at(arow, acol, aval, i, nni + dd) + csr_at(arow, acol, aval, nni + dd, i));
            for (int32_t k2 = crow[i]; k2 < crow[i + 1]; ++k2)
                d += c * csr_at(arow, acol, aval, nni + dd, nni + ccol[k2]) * cval[k2];
        }
        dinv[i] = 1.0 / d;
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

enum { T_RZ = 0, T_RR, T_PQ, T_BB, T_ALPHA, T_BETA, T_COUNT };

// partial dots a.b (row 0) and, if c, c.d (row 1)
__global__ void __launch_bounds__(256)
k_ty_dots(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
          const double* __restrict__ c, const double* __restrict__ d, double* __restrict__ partial)
{
    __shared__ double sh[32];
    double s0 = 0.0, s1 = 0.0;
    GF_FOR(i, n)
    {
        s0 = fma(a[i], b[i], s0);
        if (c) s1 = fma(c[i], d[i], s1);
    }
    double v0 = block_sum(s0, sh);
    double v1 = block_sum(s1, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = v0;
        partial[kTRed + blockIdx.x] = v1;
    }
}

// sc[dst + row] = fixed-order sums of partial rows [0, nrows); then alpha / beta as asked
__global__ void k_ty_reduce(const double* __restrict__ partial, int nrows, double* __restrict__ sc,
                            int dst, int then)
{
    __shared__ double sh[32];
    double v[2] = {0.0, 0.0};
    for (int row = 0; row < nrows; ++row) {
        double a = 0.0;
        for (int i = threadIdx.x; i < kTRed; i += blockDim.x) a += partial[row * kTRed + i];
        v[row] = block_sum(a, sh);
    }
    if (threadIdx.x == 0) {
        if (then == 1) { // p.q -> alpha
            sc[T_PQ] = v[0];
            sc[T_ALPHA] = sc[T_RZ] / v[0];
        }
        else if (then == 2) { // r.z (new), r.r -> beta
            sc[T_BETA] = v[0] / sc[T_RZ];
            sc[T_RZ] = v[0];
            sc[T_RR] = v[1];
        }
        else {
            for (int row = 0; row < nrows; ++row) sc[dst + row] = v[row];
        }
    }
}

// r = rhs - y; z = dinv r; p = z
__global__ void k_ty_start(int64_t n, const double* __restrict__ rhs, const double* __restrict__ y,
                           const double* __restrict__ dinv, double* __restrict__ r,
                           double* __restrict__ z, double* __restrict__ p)
{
    GF_FOR(i, n)
    {
        double rv = rhs[i] - y[i];
        double zv = dinv[i] * rv;
        r[i] = rv;
        z[i] = zv;
        p[i] = zv;
    }
}

__global__ void k_ty_update(int64_t n, const double* __restrict__ sc, const double* __restrict__ p,
                            const double* __restrict__ q, const double* __restrict__ dinv,
                            double* __restrict__ x, double* __restrict__ r, double* __restrict__ z)
{
    double a = sc[T_ALPHA];
    GF_FOR(i, n)
    {
        x[i] = fma(a, p[i], x[i]);
        double rv = fma(-a, q[i], r[i]);
        r[i] = rv;
        z[i] = dinv[i] * rv;
    }
}

__global__ void k_ty_direction(int64_t n, const double* __restrict__ sc, const double* __restrict__ z,
                               double* __restrict__ p)
{
    double b = sc[T_BETA];
    GF_FOR(i, n) p[i] = fma(b, p[i], z[i]);
}

__global__ void k_ty_sub(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                         double* __restrict__ out)
{
    GF_FOR(i, n) out[i] = a[i] - b[i];
}

// nodevec x: entries with dof < nnu from xu, entries with dof >= nni from xd
__global__ void k_ty_scatter(const int32_t* __restrict__ tdofs, int64_t n, int64_t nnu, int64_t nni,
                             const double* __restrict__ xu, const double* __restrict__ xd,
                             double* __restrict__ x)
{
    GF_FOR(t, n)
    {
        int64_t d = tdofs[t];
        if (d < nnu) x[t] = xu[d];
        else if (d >= nni) x[t] = xd[d - nni];
    }
}

inline int64_t a256(int64_t b)
{
    return (b + 255) / 256 * 256;
}

struct TyWs {
    double *Bu, *Bd, *Xp, *xu, *w, *tu, *td, *rhs, *r, *z, *p, *q, *dinv, *partial, *sc;
};

inline TyWs carve_ty(int64_t nnu, int64_t nnp, int64_t nnd, void* ws)
{
    char* c = static_cast<char*>(ws);
    TyWs t;
    auto take = [&](double*& p, int64_t n) {
        p = reinterpret_cast<double*>(c);
        c += a256(std::max<int64_t>(n, 1) * 8);
    };
    take(t.Bu, nnu);
    take(t.Bd, nnd);
    take(t.Xp, nnp);
    take(t.xu, nnu);
    take(t.w, nnd);
    take(t.tu, nnu);
    take(t.td, nnd);
    take(t.rhs, nnu);
    take(t.r, nnu);
    take(t.z, nnu);
    take(t.p, nnu);
    take(t.q, nnu);
    take(t.dinv, nnu);
    take(t.partial, 2 * kTRed);
    take(t.sc, T_COUNT);
    return t;
}

inline int64_t ty_bytes(int64_t nnu, int64_t nnp, int64_t nnd)
{
    auto b = [](int64_t n) { return a256(std::max<int64_t>(n, 1) * 8); };
    return 10 * b(nnu) + 3 * b(nnd) + b(nnp) + b(2 * kTRed) + b(T_COUNT);
}

} // namespace

} // namespace gfgpu

using namespace gfgpu;

namespace {

struct Csr {
    const int32_t* rowptr;
    const int32_t* col;
    const double* val;
};

// y (rows [row0, row0 + nrow) of M, columns [clo, chi) applied to x[c - cshift])
inline void spmv(const Csr& M, int64_t row0, int64_t nrow, int64_t clo, int64_t chi, int64_t cshift,
                 const double* x, int mode, double* y, cudaStream_t s)
{
    if (nrow <= 0) return;
    if (strict_mode())
        k_ty_spmv<true><<<grid_for(nrow), kBlock, 0, s>>>(M.rowptr, M.col, M.val, row0, nrow, clo, chi,
                                                         cshift, x, mode, y);
    else
        k_ty_spmv<false><<<grid_for(nrow), kBlock, 0, s>>>(M.rowptr, M.col, M.val, row0, nrow, clo, chi,
                                                          cshift, x, mode, y);
}

} // namespace

extern "C" {

int gfgpu_tyings_as_dofs_i(const int32_t* tdofs, int64_t nnode, int32_t ndim, int64_t nni,
                           int64_t nnd, const int32_t* cid_rowptr, const int32_t* cid_col,
                           const double* cid_val, const double* nodevec, int32_t apply_tyings,
                           double* dofval_i, double* work_d, gfgpu_stream_t stream)
{
    GF_REQUIRE(tdofs && nodevec && dofval_i && nnode >= 0 && ndim > 0 && nni >= 0 && nnd >= 0,
               "bad argument");
    GF_REQUIRE(!apply_tyings || (cid_rowptr && cid_col && cid_val && (nnd == 0 || work_d)),
               "apply_tyings needs C_id and a work array of nnd doubles");
    cudaStream_t s = S(stream);
    const int64_t n = nnode * ndim;
    // VectorPartitionedTyings.h:208-239
    if (nni > 0) GF_TRY(check_cuda(cudaMemsetAsync(dofval_i, 0, nni * 8, s), "cudaMemsetAsync"));
    if (n > 0) k_ty_to_dofval<<<grid_for(n), kBlock, 0, s>>>(tdofs, n, nodevec, 0, nni, dofval_i);
    if (apply_tyings && nnd > 0 && nni > 0) {
        k_ty_to_dofval<<<grid_for(n), kBlock, 0, s>>>(tdofs, n, nodevec, nni, nni + nnd, work_d);
        Csr cid{cid_rowptr, cid_col, cid_val};
        spmv(cid, 0, nni, 0, nnd, 0, work_d, 1, dofval_i, s);
    }
    return check_launch("tyings_as_dofs_i");
}

int64_t gfgpu_tyings_solve_workspace_bytes(int64_t nnu, int64_t nnp, int64_t nnd)
{
    return nnu < 0 || nnp < 0 || nnd < 0 ? 0 : ty_bytes(nnu, nnp, nnd);
}

int gfgpu_tyings_solve(const int32_t* a_rowptr, const int32_t* a_col, const double* a_val,
                       const int32_t* cdi_rowptr, const int32_t* cdi_col, const double* cdi_val,
                       const int32_t* cid_rowptr, const int32_t* cid_col, const double* cid_val,
                       const int32_t* tdofs, int64_t nnode, int32_t ndim, int64_t nnu, int64_t nnp,
                       int64_t nnd, const double* b, double* x, double tol, int64_t maxiter,
                       int32_t check_every, void* workspace, gfgpu_stream_t stream, int64_t* iters,
                       double* relres)
{
    GF_REQUIRE(a_rowptr && a_col && a_val && cdi_rowptr && cdi_col && cdi_val && cid_rowptr &&
                   cid_col && cid_val && tdofs && b && x && workspace && iters && relres,
               "bad argument");
    GF_REQUIRE(nnu > 0 && nnp >= 0 && nnd >= 0 && ndim > 0 && tol > 0.0 && maxiter >= 0,
               "bad argument");
    if (check_every < 1) check_every = 1;
    cudaStream_t s = S(stream);
    const int64_t nni = nnu + nnp, ndof = nni + nnd, n = nnode * ndim;
    TyWs w = carve_ty(nnu, nnp, nnd, workspace);
    const Csr A{a_rowptr, a_col, a_val}, Cdi{cdi_rowptr, cdi_col, cdi_val}, Cid{cid_rowptr, cid_col, cid_val};
    const unsigned gb = kTRed;
    double h[T_COUNT];
    auto read = [&]() -> int {
        GF_TRY(check_cuda(cudaMemcpyAsync(h, w.sc, sizeof(h), cudaMemcpyDeviceToHost, s), "copy"));
        return check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    };
    // y = (A_uu + A_ud C_du + C_ud A_du + C_ud A_dd C_du) v: w = C_du v; t = A [v; 0; w];
    // y = t_u + C_ud t_d (y in w.tu)
    auto condensed = [&](const double* v, double* y, cudaStream_t st) {
        spmv(Cdi, 0, nnd, 0, nnu, 0, v, 0, w.w, st);
        spmv(A, 0, nnu, 0, nnu, 0, v, 0, y, st);
        spmv(A, 0, nnu, nni, ndof, nni, w.w, 1, y, st);
        spmv(A, nni, nnd, 0, nnu, 0, v, 0, w.td, st);
        spmv(A, nni, nnd, nni, ndof, nni, w.w, 1, w.td, st);
        spmv(Cid, 0, nnu, 0, nnd, 0, w.td, 1, y, st);
    };
    // MatrixPartitionedTyings.h solve_nodevec_impl: B_u += C_ud B_d; rhs = B_u - AC_up X_p
    k_ty_to_dofval<<<grid_for(n), kBlock, 0, s>>>(tdofs, n, b, 0, nnu, w.Bu);
    if (nnd > 0) k_ty_to_dofval<<<grid_for(n), kBlock, 0, s>>>(tdofs, n, b, nni, ndof, w.Bd);
    if (nnp > 0) k_ty_to_dofval<<<grid_for(n), kBlock, 0, s>>>(tdofs, n, x, nnu, nni, w.Xp);
    k_ty_to_dofval<<<grid_for(n), kBlock, 0, s>>>(tdofs, n, x, 0, nnu, w.xu);
    spmv(Cid, 0, nnu, 0, nnd, 0, w.Bd, 1, w.Bu, s);
    // AC_up X_p = t'_u + C_ud t'_d with t' = A [0; X_p; C_dp X_p]
    spmv(Cdi, 0, nnd, nnu, nni, nnu, w.Xp, 0, w.w, s);
    spmv(A, 0, nnu, nnu, nni, nnu, w.Xp, 0, w.tu, s);
    spmv(A, 0, nnu, nni, ndof, nni, w.w, 1, w.tu, s);
    spmv(A, nni, nnd, nnu, nni, nnu, w.Xp, 0, w.td, s);
    spmv(A, nni, nnd, nni, ndof, nni, w.w, 1, w.td, s);
    spmv(Cid, 0, nnu, 0, nnd, 0, w.td, 1, w.tu, s);
    k_ty_sub<<<grid_for(nnu), kBlock, 0, s>>>(nnu, w.Bu, w.tu, w.rhs);
    k_ty_dinv<<<grid_for(nnu), kBlock, 0, s>>>(a_rowptr, a_col, a_val, cid_rowptr, cid_col, cid_val,
                                               nnu, nni, w.dinv);
    // r = rhs - AC_uu x_u, z = D^-1 r, p = z
    condensed(w.xu, w.q, s);
    k_ty_start<<<grid_for(nnu), kBlock, 0, s>>>(nnu, w.rhs, w.q, w.dinv, w.r, w.z, w.p);
    k_ty_dots<<<gb, 256, 0, s>>>(nnu, w.r, w.z, w.r, w.r, w.partial);
    k_ty_reduce<<<1, 1024, 0, s>>>(w.partial, 2, w.sc, T_RZ, 0); // T_RZ, T_RR
    k_ty_dots<<<gb, 256, 0, s>>>(nnu, w.rhs, w.rhs, nullptr, nullptr, w.partial);
    k_ty_reduce<<<1, 1024, 0, s>>>(w.partial, 1, w.sc, T_BB, 0);
    GF_TRY(check_launch("tyings_solve set-up"));
    GF_TRY(read());
    double bnorm = std::sqrt(h[T_BB]);
    if (bnorm == 0.0) bnorm = 1.0;
    double rel = std::sqrt(h[T_RR]) / bnorm;
    auto iteration = [&](cudaStream_t st) {
        condensed(w.p, w.q, st);
        k_ty_dots<<<gb, 256, 0, st>>>(nnu, w.p, w.q, nullptr, nullptr, w.partial);
        k_ty_reduce<<<1, 1024, 0, st>>>(w.partial, 1, w.sc, 0, 1);
        k_ty_update<<<grid_for(nnu), kBlock, 0, st>>>(nnu, w.sc, w.p, w.q, w.dinv, w.xu, w.r, w.z);
        k_ty_dots<<<gb, 256, 0, st>>>(nnu, w.r, w.z, w.r, w.r, w.partial);
        k_ty_reduce<<<1, 1024, 0, st>>>(w.partial, 2, w.sc, 0, 2);
        k_ty_direction<<<grid_for(nnu), kBlock, 0, st>>>(nnu, w.sc, w.z, w.p);
    };
    int64_t it = 0;
    int rc = GFGPU_OK;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cs = nullptr;
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
            rc = check_launch("tyings_solve iteration");
        }
        if (rc != GFGPU_OK) break;
        it += nb;
        rc = read();
        if (rc != GFGPU_OK) break;
        if (!std::isfinite(h[T_RR])) {
            rc = fail(GFGPU_ERR_NAN, "gfgpu_tyings_solve: non-finite residual");
            break;
        }
        rel = std::sqrt(h[T_RR]) / bnorm;
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (cs) cudaStreamDestroy(cs);
    *iters = it;
    GF_TRY(rc);
    // X_d = C_du X_u + C_dp X_p; write x_u, x_d into the nodevec
    spmv(Cdi, 0, nnd, 0, nnu, 0, w.xu, 0, w.td, s);
    spmv(Cdi, 0, nnd, nnu, nni, nnu, w.Xp, 1, w.td, s);
    k_ty_scatter<<<grid_for(n), kBlock, 0, s>>>(tdofs, n, nnu, nni, w.xu, w.td, x);
    // true residual rhs - AC_uu x_u
    condensed(w.xu, w.q, s);
    k_ty_sub<<<grid_for(nnu), kBlock, 0, s>>>(nnu, w.rhs, w.q, w.r);
    k_ty_dots<<<gb, 256, 0, s>>>(nnu, w.r, w.r, nullptr, nullptr, w.partial);
    k_ty_reduce<<<1, 1024, 0, s>>>(w.partial, 1, w.sc, T_RR, 0);
    GF_TRY(check_launch("tyings_solve residual"));
    GF_TRY(read());
    *relres = std::sqrt(h[T_RR]) / bnorm;
    if (*relres > tol) return fail(GFGPU_ERR_DIVERGED, "gfgpu_tyings_solve: tolerance not reached");
    return GFGPU_OK;
}

} // extern "C"
