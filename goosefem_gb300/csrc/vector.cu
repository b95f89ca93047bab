// Vector (dofval / nodevec / elemvec conversions), deterministic CSR assembly and the
// MatrixDiagonal(Partitioned) operations. The reference's serial scatter-adds become
// dof-centric gathers over a CSR whose segments are sorted by flat source index, so every dof is
// summed in the reference's order and results are identical run to run.
#include <vector>

#include "common.cuh"

namespace gfgpu {

__global__ void k_as_element(const int32_t* __restrict__ conn, int64_t nem, int nd,
                             const double* __restrict__ nodevec, double* __restrict__ elemvec)
{
    GF_FOR(t, nem * nd)
    {
        int64_t k = t / nd;
        int i = static_cast<int>(t - k * nd);
        elemvec[t] = __ldg(nodevec + static_cast<int64_t>(__ldg(conn + k)) * nd + i);
    }
}

__global__ void k_as_element_dofval(const int32_t* __restrict__ conn,
                                    const int32_t* __restrict__ dofs, int64_t nem, int nd,
                                    const double* __restrict__ dofval, double* __restrict__ elemvec)
{
    GF_FOR(t, nem * nd)
    {
        int64_t k = t / nd;
        int i = static_cast<int>(t - k * nd);
        int32_t n = __ldg(conn + k);
        elemvec[t] = __ldg(dofval + __ldg(dofs + static_cast<int64_t>(n) * nd + i));
    }
}

__global__ void k_as_node(const int32_t* __restrict__ dofs, int64_t n,
                          const double* __restrict__ dofval, double* __restrict__ nodevec)
{
    GF_FOR(t, n) nodevec[t] = __ldg(dofval + __ldg(dofs + t));
}

__global__ void k_csr_last(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                           int64_t ndof, int32_t* __restrict__ last)
{
    GF_FOR(d, ndof)
    {
        int32_t b = ptr[d], e = ptr[d + 1];
        last[d] = e > b ? idx[e - 1] : -1;
    }
}

__global__ void k_as_dofs(const int32_t* __restrict__ last, int64_t ndof,
                          const double* __restrict__ src, double* __restrict__ dofval)
{
    GF_FOR(d, ndof)
    {
        int32_t l = last[d];
        dofval[d] = l >= 0 ? src[l] : 0.0;
    }
}

// sum of src over the dof's CSR segment, ascending, starting from 0.0 (the reference's fill(0.0))
__device__ __forceinline__ double seg_sum(const int32_t* __restrict__ idx, int32_t b, int32_t e,
                                          const double* __restrict__ src)
{
    double acc = 0.0;
    for (int32_t k = b; k < e; ++k) acc = __dadd_rn(acc, __ldg(src + __ldg(idx + k)));
    return acc;
}

__global__ void k_assemble_dofs(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                int64_t ndof, const double* __restrict__ src,
                                double* __restrict__ dofval)
{
    GF_FOR(d, ndof) dofval[d] = seg_sum(idx, __ldg(ptr + d), __ldg(ptr + d + 1), src);
}

__global__ void k_assemble_node(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                const int32_t* __restrict__ dofs, int64_t n,
                                const double* __restrict__ src, double* __restrict__ nodevec)
{
    GF_FOR(t, n)
    {
        int32_t d = __ldg(dofs + t);
        nodevec[t] = seg_sum(idx, __ldg(ptr + d), __ldg(ptr + d + 1), src);
    }
}

__global__ void k_is_diagonal(const double* __restrict__ elemmat, int64_t nelem, int K,
                              int* __restrict__ flag)
{
    const double eps = 2.220446049250313080847e-16; // DBL_EPSILON
    GF_FOR(t, nelem * K * K)
    {
        int rc = static_cast<int>(t % (static_cast<int64_t>(K) * K));
        int r = rc / K, c = rc - r * K;
        if (r != c && fabs(elemmat[t]) > eps) *flag = 0;
    }
}

__global__ void k_diag_assemble(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                int64_t ndof, int kn, const double* __restrict__ elemmat,
                                double* __restrict__ A)
{
    // flat elemvec index f = e*kn + r  ->  elemmat(e, r, r)
    GF_FOR(d, ndof)
    {
        double acc = 0.0;
        for (int32_t k = ptr[d]; k < ptr[d + 1]; ++k) {
            int64_t f = idx[k];
            int64_t e = f / kn;
            int64_t r = f - e * kn;
            acc = __dadd_rn(acc, elemmat[(e * kn + r) * kn + r]);
        }
        A[d] = acc;
    }
}

__global__ void k_recip(const double* __restrict__ A, int64_t n, double* __restrict__ inv)
{
    GF_FOR(d, n) inv[d] = __ddiv_rn(1.0, A[d]);
}

__global__ void k_diag_solve(const int32_t* __restrict__ dofs, int64_t n, int64_t nnu,
                             const double* __restrict__ inv, const double* __restrict__ b,
                             double* __restrict__ x)
{
    GF_FOR(t, n)
    {
        int32_t d = dofs[t];
        if (d < nnu) x[t] = __dmul_rn(inv[d], b[t]);
    }
}

__global__ void k_diag_dot(const int32_t* __restrict__ dofs, int64_t n,
                           const double* __restrict__ A, const double* __restrict__ x,
                           double* __restrict__ b)
{
    GF_FOR(t, n) b[t] = __dmul_rn(A[dofs[t]], x[t]);
}

__global__ void k_diagp_reaction(const int32_t* __restrict__ part, int64_t n, int64_t nnu,
                                 const double* __restrict__ App, const double* __restrict__ x,
                                 double* __restrict__ b)
{
    GF_FOR(t, n)
    {
        int32_t d = part[t];
        if (d >= nnu) b[t] = __dmul_rn(App[d - nnu], x[t]);
    }
}

__global__ void k_mul(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
                      double* __restrict__ o)
{
    GF_FOR(t, n) o[t] = __dmul_rn(a[t], b[t]);
}

// out[i * k + j] = src[i]: a scalar per entry repeated over k trailing tensor components
__global__ void k_broadcast(const double* __restrict__ src, int64_t n, int64_t k,
                            double* __restrict__ out)
{
    GF_FOR(t, n * k) out[t] = __ldg(src + t / k);
}

// out[t] = [u | p][idx[t]]: the partitioned vector read back through a partitioned index table
__global__ void k_from_partitioned(const int32_t* __restrict__ idx, int64_t n, int64_t nnu,
                                   const double* __restrict__ u, const double* __restrict__ p,
                                   double* __restrict__ out)
{
    GF_FOR(t, n)
    {
        int64_t d = __ldg(idx + t);
        out[t] = d < nnu ? __ldg(u + d) : __ldg(p + (d - nnu));
    }
}

__global__ void k_from_partitioned_elem(const int32_t* __restrict__ conn,
                                        const int32_t* __restrict__ part, int64_t nem, int nd,
                                        int64_t nnu, const double* __restrict__ u,
                                        const double* __restrict__ p, double* __restrict__ elemvec)
{
    GF_FOR(t, nem * nd)
    {
        int64_t k = t / nd;
        int i = static_cast<int>(t - k * nd);
        int64_t d = __ldg(part + static_cast<int64_t>(__ldg(conn + k)) * nd + i);
        elemvec[t] = d < nnu ? __ldg(u + d) : __ldg(p + (d - nnu));
    }
}

__global__ void k_copy_part(const int32_t* __restrict__ part, int64_t n, int64_t lo, int64_t hi,
                            const double* __restrict__ src, double* __restrict__ dest)
{
    GF_FOR(t, n)
    {
        int64_t d = __ldg(part + t);
        if (d >= lo && d < hi) dest[t] = src[t];
    }
}

} // namespace gfgpu

using namespace gfgpu;

extern "C" {

int gfgpu_as_element(const int32_t* conn, int64_t nelem, int32_t nne, int32_t ndim,
                     const double* nodevec, double* elemvec, gfgpu_stream_t stream)
{
    GF_REQUIRE(conn && nodevec && elemvec && nne > 0 && ndim > 0, "bad argument");
    GF_REQUIRE(!too_big(nelem * nne * ndim), "too many elements");
    if (nelem == 0) return GFGPU_OK;
    k_as_element<<<grid_for(nelem * nne * ndim), kBlock, 0, S(stream)>>>(conn, nelem * nne, ndim,
                                                                         nodevec, elemvec);
    return check_launch("as_element");
}

int gfgpu_as_element_dofval(const int32_t* conn, const int32_t* dofs, int64_t nelem, int32_t nne,
                            int32_t ndim, const double* dofval, double* elemvec,
                            gfgpu_stream_t stream)
{
    GF_REQUIRE(conn && dofs && dofval && elemvec && nne > 0 && ndim > 0, "bad argument");
    GF_REQUIRE(!too_big(nelem * nne * ndim), "too many elements");
    if (nelem == 0) return GFGPU_OK;
    k_as_element_dofval<<<grid_for(nelem * nne * ndim), kBlock, 0, S(stream)>>>(
        conn, dofs, nelem * nne, ndim, dofval, elemvec);
    return check_launch("as_element_dofval");
}

int gfgpu_as_node(const int32_t* dofs, int64_t nnode, int32_t ndim, const double* dofval,
                  double* nodevec, gfgpu_stream_t stream)
{
    GF_REQUIRE(dofs && dofval && nodevec && ndim > 0, "bad argument");
    GF_REQUIRE(!too_big(nnode * ndim), "too many nodes");
    if (nnode == 0) return GFGPU_OK;
    k_as_node<<<grid_for(nnode * ndim), kBlock, 0, S(stream)>>>(dofs, nnode * ndim, dofval, nodevec);
    return check_launch("as_node");
}

int gfgpu_csr_last(const int32_t* ptr, const int32_t* idx, int64_t ndof, int32_t* last,
                   gfgpu_stream_t stream)
{
    GF_REQUIRE(ptr && idx && last && !too_big(ndof), "bad argument");
    if (ndof == 0) return GFGPU_OK;
    k_csr_last<<<grid_for(ndof), kBlock, 0, S(stream)>>>(ptr, idx, ndof, last);
    return check_launch("csr_last");
}

int gfgpu_as_dofs(const int32_t* last, int64_t ndof, const double* src, double* dofval,
                  gfgpu_stream_t stream)
{
    GF_REQUIRE(last && src && dofval && !too_big(ndof), "bad argument");
    if (ndof == 0) return GFGPU_OK;
    k_as_dofs<<<grid_for(ndof), kBlock, 0, S(stream)>>>(last, ndof, src, dofval);
    return check_launch("as_dofs");
}

int gfgpu_assemble_dofs(const int32_t* ptr, const int32_t* idx, int64_t ndof, const double* src,
                        double* dofval, gfgpu_stream_t stream)
{
    GF_REQUIRE(ptr && idx && src && dofval && !too_big(ndof), "bad argument");
    if (ndof == 0) return GFGPU_OK;
    k_assemble_dofs<<<grid_for(ndof), kBlock, 0, S(stream)>>>(ptr, idx, ndof, src, dofval);
    return check_launch("assemble_dofs");
}

int gfgpu_assemble_node(const int32_t* ptr, const int32_t* idx, const int32_t* dofs,
                        int64_t nnode, int32_t ndim, const double* elemvec, double* nodevec,
                        gfgpu_stream_t stream)
{
    GF_REQUIRE(ptr && idx && dofs && elemvec && nodevec && ndim > 0, "bad argument");
    GF_REQUIRE(!too_big(nnode * ndim), "too many nodes");
    if (nnode == 0) return GFGPU_OK;
    k_assemble_node<<<grid_for(nnode * ndim), kBlock, 0, S(stream)>>>(ptr, idx, dofs, nnode * ndim,
                                                                      elemvec, nodevec);
    return check_launch("assemble_node");
}

int gfgpu_is_diagonal(const double* elemmat, int64_t nelem, int32_t K, int* is_diag,
                      gfgpu_stream_t stream)
{
    GF_REQUIRE(elemmat && is_diag && K > 0 && !too_big(nelem * K * K), "bad argument");
    int* flag = nullptr;
    GF_TRY(check_cuda(cudaMallocAsync(&flag, sizeof(int), S(stream)), "cudaMallocAsync"));
    int one = 1;
    GF_TRY(check_cuda(cudaMemcpyAsync(flag, &one, sizeof(int), cudaMemcpyHostToDevice, S(stream)),
                      "cudaMemcpyAsync"));
    if (nelem > 0)
        k_is_diagonal<<<grid_for(nelem * K * K), kBlock, 0, S(stream)>>>(elemmat, nelem, K, flag);
    GF_TRY(check_launch("is_diagonal"));
    GF_TRY(check_cuda(cudaMemcpyAsync(is_diag, flag, sizeof(int), cudaMemcpyDeviceToHost, S(stream)),
                      "cudaMemcpyAsync"));
    GF_TRY(check_cuda(cudaFreeAsync(flag, S(stream)), "cudaFreeAsync"));
    return check_cuda(cudaStreamSynchronize(S(stream)), "cudaStreamSynchronize");
}

int gfgpu_diag_assemble(const int32_t* ptr, const int32_t* idx, int64_t ndof, int32_t nne,
                        int32_t ndim, const double* elemmat, double* A, gfgpu_stream_t stream)
{
    GF_REQUIRE(ptr && idx && elemmat && A && nne > 0 && ndim > 0 && !too_big(ndof), "bad argument");
    if (ndof == 0) return GFGPU_OK;
    k_diag_assemble<<<grid_for(ndof), kBlock, 0, S(stream)>>>(ptr, idx, ndof, nne * ndim, elemmat, A);
    return check_launch("diag_assemble");
}

int gfgpu_diag_factorize(const double* A, int64_t n, double* inv, gfgpu_stream_t stream)
{
    GF_REQUIRE(A && inv && !too_big(n), "bad argument");
    if (n == 0) return GFGPU_OK;
    k_recip<<<grid_for(n), kBlock, 0, S(stream)>>>(A, n, inv);
    return check_launch("diag_factorize");
}

int gfgpu_diag_solve_nodevec(const int32_t* dofs, int64_t nnode, int32_t ndim, int64_t nnu,
                             const double* inv, const double* b, double* x, gfgpu_stream_t stream)
{
    GF_REQUIRE(dofs && inv && b && x && ndim > 0 && !too_big(nnode * ndim), "bad argument");
    if (nnode == 0) return GFGPU_OK;
    k_diag_solve<<<grid_for(nnode * ndim), kBlock, 0, S(stream)>>>(dofs, nnode * ndim, nnu, inv, b, x);
    return check_launch("diag_solve_nodevec");
}

int gfgpu_diag_dot_nodevec(const int32_t* dofs, int64_t nnode, int32_t ndim, const double* A,
                           const double* x, double* b, gfgpu_stream_t stream)
{
    GF_REQUIRE(dofs && A && x && b && ndim > 0 && !too_big(nnode * ndim), "bad argument");
    if (nnode == 0) return GFGPU_OK;
    k_diag_dot<<<grid_for(nnode * ndim), kBlock, 0, S(stream)>>>(dofs, nnode * ndim, A, x, b);
    return check_launch("diag_dot_nodevec");
}

int gfgpu_diagp_reaction_nodevec(const int32_t* part, int64_t nnode, int32_t ndim, int64_t nnu,
                                 const double* App, const double* x, double* b,
                                 gfgpu_stream_t stream)
{
    GF_REQUIRE(part && App && x && b && ndim > 0 && !too_big(nnode * ndim), "bad argument");
    if (nnode == 0) return GFGPU_OK;
    k_diagp_reaction<<<grid_for(nnode * ndim), kBlock, 0, S(stream)>>>(part, nnode * ndim, nnu, App,
                                                                       x, b);
    return check_launch("diagp_reaction_nodevec");
}

int gfgpu_dofval_mul(const double* a, const double* b, int64_t n, double* out,
                     gfgpu_stream_t stream)
{
    GF_REQUIRE(a && b && out && !too_big(n), "bad argument");
    if (n == 0) return GFGPU_OK;
    k_mul<<<grid_for(n), kBlock, 0, S(stream)>>>(a, b, n, out);
    return check_launch("dofval_mul");
}

int gfgpu_broadcast(const double* src, int64_t n, int64_t k, double* out, gfgpu_stream_t stream)
{
    GF_REQUIRE(src && out && n >= 0 && k >= 1, "bad argument");
    GF_REQUIRE(!too_big(n * k), "too many values");
    if (n == 0) return GFGPU_OK;
    k_broadcast<<<grid_for(n * k), kBlock, 0, S(stream)>>>(src, n, k, out);
    return check_launch("broadcast");
}

int gfgpu_from_partitioned(const int32_t* idx, int64_t n, int64_t nnu, int64_t nnp,
                           const double* u, const double* p, double* out, gfgpu_stream_t stream)
{
    GF_REQUIRE(idx && out && (u || nnu == 0) && (p || nnp == 0) && nnu >= 0 && nnp >= 0,
               "bad argument");
    GF_REQUIRE(!too_big(n) && !too_big(nnu + nnp), "too many values");
    if (n == 0) return GFGPU_OK;
    k_from_partitioned<<<grid_for(n), kBlock, 0, S(stream)>>>(idx, n, nnu, u, p, out);
    return check_launch("from_partitioned");
}

int gfgpu_from_partitioned_elemvec(const int32_t* conn, const int32_t* part, int64_t nelem,
                                   int32_t nne, int32_t ndim, int64_t nnu, int64_t nnp,
                                   const double* u, const double* p, double* elemvec,
                                   gfgpu_stream_t stream)
{
    GF_REQUIRE(conn && part && elemvec && (u || nnu == 0) && (p || nnp == 0) && nne > 0 &&
                   ndim > 0 && nnu >= 0 && nnp >= 0,
               "bad argument");
    GF_REQUIRE(!too_big(nelem * nne * ndim) && !too_big(nnu + nnp), "too many elements");
    if (nelem == 0) return GFGPU_OK;
    k_from_partitioned_elem<<<grid_for(nelem * nne * ndim), kBlock, 0, S(stream)>>>(
        conn, part, nelem * nne, ndim, nnu, u, p, elemvec);
    return check_launch("from_partitioned_elemvec");
}

int gfgpu_copy_partitioned_nodevec(const int32_t* part, int64_t nnode, int32_t ndim, int64_t lo,
                                   int64_t hi, const double* src, double* dest,
                                   gfgpu_stream_t stream)
{
    GF_REQUIRE(part && src && dest && ndim > 0 && lo >= 0 && hi >= lo, "bad argument");
    GF_REQUIRE(!too_big(nnode * ndim), "too many nodes");
    if (nnode == 0 || hi == lo) return GFGPU_OK;
    k_copy_part<<<grid_for(nnode * ndim), kBlock, 0, S(stream)>>>(part, nnode * ndim, lo, hi, src,
                                                                  dest);
    return check_launch("copy_partitioned_nodevec");
}

} // extern "C"
