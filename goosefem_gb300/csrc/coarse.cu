// Two-level (coarse-grid) correction for the matrix-free static solve on a Regular Quad4 grid.
//
// The coarse space is spanned by bilinear hat functions on a grid of every hc-th node (the last
// interval of each axis may be shorter), one per coarse node and displacement component, with
// the prescribed fine dofs masked out. The Galerkin matrix A_c = P^T A_uu P is a 9-point stencil
// of 2x2 blocks; it is measured by applying the matrix-free operator to 18 colourings of the
// coarse hats (coarse nodes three apart in x and y never share a coarse neighbour), inverted once
// in FP64 by Gauss-Jordan (A_c is SPD, no pivoting) and kept as a dense FP32 inverse. Applying
// the correction is restriction (P^T r) -> dense product -> prolongation (P y); all three are
// fixed-order sums, so results are identical run to run.
#include "common.cuh"

// element-kernel launch shared with the explicit step (dynamics.cu)
int gfgpu_internal_element_forces(const gfgpu_verlet_desc* d, const double* u, double* fe,
                                  cudaStream_t s);

namespace gfgpu {
namespace coarse {

constexpr int kRestrictThreads = 256;
constexpr int64_t kMaxCoarseDofs = 8192; // dense inverse: 256 MB FP32, set-up 512 MB FP64
static_assert(kMaxCoarseDofs * 4 <= 48 * 1024, "k_dense stages v in default shared memory");
constexpr int kRowsPerBlock = 8;         // dense product: one warp per row

inline int64_t a256(int64_t b)
{
    return (b + 255) / 256 * 256;
}

// coarse coordinate of coarse index j along an axis of `nel` elements
__host__ __device__ inline int coarse_x(int j, int hc, int nel)
{
    return min(j * hc, nel);
}

// Interval j of an axis spans [coarse_x(j), coarse_x(j + 1)]: length hc (reciprocal rh) except
// the last one, j = nc - 2 (reciprocal rl). No division on the device. T = double for the set-up
// (the Galerkin matrix), float for the correction inside the solve.
template <typename T>
__device__ inline T rlen(int j, int nc, double rh, double rl)
{
    return static_cast<T>(j == nc - 2 ? rl : rh);
}

// fine node i on an axis: left coarse index j0 and the weight w0 of j0 (1 - w0 for j0 + 1)
template <typename T>
__device__ inline void hat(int i, int hc, int nel, int nc, double rh, double rl, int& j0, T& w0)
{
    int j = i / hc;
    if (j > nc - 2) j = nc - 2;
    j0 = j;
    w0 = static_cast<T>(coarse_x(j + 1, hc, nel) - i) * rlen<T>(j, nc, rh, rl);
}

// weight of coarse index j at fine node i (0 outside its support)
template <typename T>
__device__ inline T hat_w(int j, int i, int hc, int nel, int nc, double rh, double rl)
{
    int x = coarse_x(j, hc, nel);
    if (i == x) return T(1);
    if (i < x) {
        if (j == 0) return T(0);
        int xl = coarse_x(j - 1, hc, nel);
        return i > xl ? static_cast<T>(i - xl) * rlen<T>(j - 1, nc, rh, rl) : T(0);
    }
    if (j == nc - 1) return T(0);
    int xr = coarse_x(j + 1, hc, nel);
    return i < xr ? static_cast<T>(xr - i) * rlen<T>(j, nc, rh, rl) : T(0);
}

template <typename T>
__device__ __forceinline__ T bsum(T v, T* sh)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    if (lane == 0) sh[wi] = v;
    __syncthreads();
    T r = T(0);
    if (wi == 0) {
        r = lane < (blockDim.x >> 5) ? sh[lane] : T(0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;
}

// v[(jy * ncx + jx) * 2 + c] = sum over the hat's support of w(ix) w(iy) f[(iy W + ix) 2 + c] on
// free dofs, accumulated in T; one block per coarse node
template <typename T>
__global__ void __launch_bounds__(kRestrictThreads)
k_restrict(gfgpu_coarse_desc g, const int32_t* __restrict__ part, int64_t nnu,
           const double* __restrict__ f, T* __restrict__ v)
{
    __shared__ T sh[32];
    const int jx = blockIdx.x % g.ncx, jy = blockIdx.x / g.ncx;
    const int x0 = coarse_x(max(jx - 1, 0), g.hc, g.nx), x1 = coarse_x(min(jx + 1, g.ncx - 1), g.hc, g.nx);
    const int y0 = coarse_x(max(jy - 1, 0), g.hc, g.ny), y1 = coarse_x(min(jy + 1, g.ncy - 1), g.hc, g.ny);
    const int sx = x1 - x0 + 1, cnt = sx * (y1 - y0 + 1);
    const int64_t W = g.nx + 1;
    T a0 = T(0), a1 = T(0);
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
        int ix = x0 + k % sx, iy = y0 + k / sx;
        T w = hat_w<T>(jx, ix, g.hc, g.nx, g.ncx, g.rhx, g.rlx) * hat_w<T>(jy, iy, g.hc, g.ny, g.ncy, g.rhy, g.rly);
        int64_t t = (iy * W + ix) * 2;
        int2 pt = __ldg(reinterpret_cast<const int2*>(part + t));
        double2 ft = __ldg(reinterpret_cast<const double2*>(f + t));
        if (pt.x < nnu) a0 += w * static_cast<T>(ft.x);
        if (pt.y < nnu) a1 += w * static_cast<T>(ft.y);
    }
    a0 = bsum(a0, sh);
    a1 = bsum(a1, sh);
    if (threadIdx.x == 0) {
        v[int64_t(blockIdx.x) * 2] = a0;
        v[int64_t(blockIdx.x) * 2 + 1] = a1;
    }
}

// z = (P y)_u  (+ minv * r when minv is given), interpolation in T; 0 on prescribed dofs
template <typename T>
__global__ void k_prolong(gfgpu_coarse_desc g, const int32_t* __restrict__ part, int64_t nnu,
                          const T* __restrict__ y, const double* __restrict__ minv,
                          const double* __restrict__ r, double* __restrict__ z)
{
    const int64_t W = g.nx + 1, nn = W * (g.ny + 1);
    GF_FOR(node, nn)
    {
        int ix = static_cast<int>(node % W), iy = static_cast<int>(node / W);
        int jx, jy;
        T wx, wy;
        hat<T>(ix, g.hc, g.nx, g.ncx, g.rhx, g.rlx, jx, wx);
        hat<T>(iy, g.hc, g.ny, g.ncy, g.rhy, g.rly, jy, wy);
        const T w[4] = {wx * wy, (T(1) - wx) * wy, wx * (T(1) - wy), (T(1) - wx) * (T(1) - wy)};
        const int64_t c[4] = {int64_t(jy) * g.ncx + jx, int64_t(jy) * g.ncx + jx + 1,
                              int64_t(jy + 1) * g.ncx + jx, int64_t(jy + 1) * g.ncx + jx + 1};
        const int64_t t = node * 2;
        const int2 pt = __ldg(reinterpret_cast<const int2*>(part + t));
        T s0 = T(0), s1 = T(0);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            s0 += w[k] * __ldg(y + c[k] * 2);
            s1 += w[k] * __ldg(y + c[k] * 2 + 1);
        }
        double z0 = static_cast<double>(s0), z1 = static_cast<double>(s1);
        if (minv) {
            z0 = fma(minv[t], r[t], z0);
            z1 = fma(minv[t + 1], r[t + 1], z1);
        }
        z[t] = pt.x < nnu ? z0 : 0.0;
        z[t + 1] = pt.y < nnu ? z1 : 0.0;
    }
}

// y = Ainv v (FP32 matrix [nc, ld], FP32 vectors); one warp per row with 16-byte loads, v staged
// in shared memory (zero padded to ld)
__global__ void __launch_bounds__(32 * kRowsPerBlock)
k_dense(const float* __restrict__ ainv, int64_t nc, int64_t ld, const float* __restrict__ v,
        float* __restrict__ y)
{
    extern __shared__ float4 vs4[];
    float* vs = reinterpret_cast<float*>(vs4);
    for (int64_t k = threadIdx.x; k < ld; k += blockDim.x) vs[k] = k < nc ? v[k] : 0.0f;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t row = int64_t(blockIdx.x) * kRowsPerBlock + (threadIdx.x >> 5);
    if (row >= nc) return;
    const float4* a = reinterpret_cast<const float4*>(ainv + row * ld);
    const int64_t n4 = ld / 4;
    float acc0 = 0.0f, acc1 = 0.0f;
#pragma unroll 4
    for (int64_t k = lane; k < n4; k += 32) {
        float4 m = __ldg(a + k), u = vs4[k];
        acc0 = fmaf(m.x, u.x, acc0);
        acc1 = fmaf(m.y, u.y, acc1);
        acc0 = fmaf(m.z, u.z, acc0);
        acc1 = fmaf(m.w, u.w, acc1);
    }
    float acc = acc0 + acc1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) y[row] = acc;
}

// ------------------------------------------------------------------------------ set-up kernels

// coarse indicator of one colouring: e = 1 at coarse dofs (jx % 3 == a, jy % 3 == b, comp)
__global__ void k_probe(gfgpu_coarse_desc g, int a, int b, int comp, double* __restrict__ e)
{
    const int64_t nc = int64_t(g.ncx) * g.ncy * 2;
    GF_FOR(t, nc)
    {
        int64_t node = t / 2;
        int c = static_cast<int>(t - node * 2);
        int jx = static_cast<int>(node % g.ncx), jy = static_cast<int>(node / g.ncx);
        e[t] = (c == comp && jx % 3 == a && jy % 3 == b) ? 1.0 : 0.0;
    }
}

// q = (A p)_u from element forces through the dof CSR (0 on prescribed dofs)
__global__ void k_apply_gather(const int32_t* __restrict__ dofs, const int32_t* __restrict__ ptr,
                               const int32_t* __restrict__ idx, const int32_t* __restrict__ part,
                               int64_t nnu, const double* __restrict__ fe, int64_t n,
                               double* __restrict__ q, RegGrid reg)
{
    GF_FOR(t, n) q[t] = part[t] < nnu ? gather_dof(t, dofs, ptr, idx, fe, reg) : 0.0;
}

// column block of A_c from one probe: row i (coarse node jx, jy) gets v[i] in the column of the
// probed coarse node within one coarse index of (jx, jy) (unique: the probed nodes are 3 apart)
__global__ void k_probe_scatter(gfgpu_coarse_desc g, int a, int b, int comp,
                                const double* __restrict__ v, double* __restrict__ Ac)
{
    const int64_t nc = int64_t(g.ncx) * g.ncy * 2;
    GF_FOR(i, nc)
    {
        int64_t node = i / 2;
        int jx = static_cast<int>(node % g.ncx), jy = static_cast<int>(node / g.ncx);
        int kx = -1, ky = -1;
        for (int o = -1; o <= 1; ++o) {
            int x = jx + o, y = jy + o;
            if (x >= 0 && x < g.ncx && x % 3 == a) kx = x;
            if (y >= 0 && y < g.ncy && y % 3 == b) ky = y;
        }
        if (kx >= 0 && ky >= 0) Ac[i * nc + (int64_t(ky) * g.ncx + kx) * 2 + comp] = v[i];
    }
}

// A_c = (A_c + A_c^T) / 2 (the Galerkin product is symmetric up to rounding); a coarse dof
// without free fine dofs (zero row and column) gets a unit diagonal
__global__ void k_symmetrize(double* __restrict__ Ac, int64_t nc)
{
    GF_FOR(t, nc * nc)
    {
        int64_t i = t / nc, j = t - i * nc;
        if (j > i) {
            double s = 0.5 * (Ac[i * nc + j] + Ac[j * nc + i]);
            Ac[i * nc + j] = s;
            Ac[j * nc + i] = s;
        }
        else if (j == i && Ac[t] == 0.0) {
            Ac[t] = 1.0;
        }
    }
}

// In-place Gauss-Jordan inversion, pivot k: (1) p = 1 / A[k][k], row k scaled by p;
// (2) A[i][j] -= A[i][k] A[k][j] for i, j != k; (3) column k scaled by -p, A[k][k] = p.
__global__ void k_gj_row(double* __restrict__ A, int64_t nc, int64_t k, double* __restrict__ piv)
{
    const double p = 1.0 / A[k * nc + k];
    GF_FOR(j, nc)
    {
        if (j != k) A[k * nc + j] *= p;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        piv[0] = p;
        if (!(p == p) || p == 0.0 || fabs(p) > 1e300) piv[1] = 1.0; // non-finite or singular pivot
    }
}

// grid (ceil(nc / 256), nc): row i = blockIdx.y
__global__ void k_gj_update(double* __restrict__ A, int64_t nc, int64_t k)
{
    const int64_t i = blockIdx.y, j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i == k || j >= nc || j == k) return;
    A[i * nc + j] = fma(-A[i * nc + k], A[k * nc + j], A[i * nc + j]);
}

__global__ void k_gj_col(double* __restrict__ A, int64_t nc, int64_t k, const double* __restrict__ piv)
{
    const double p = piv[0];
    GF_FOR(i, nc)
    {
        if (i != k) A[i * nc + k] *= -p;
        else A[k * nc + k] = p;
    }
}

__global__ void k_to_f32(const double* __restrict__ a, int64_t nc, int64_t ld, float* __restrict__ o)
{
    GF_FOR(t, nc * ld)
    {
        int64_t i = t / ld, j = t - i * ld;
        o[t] = j < nc ? static_cast<float>(a[i * nc + j]) : 0.0f;
    }
}

inline int64_t ncoarse(const gfgpu_coarse_desc* g)
{
    return int64_t(g->ncx) * g->ncy * 2;
}

} // namespace coarse
} // namespace gfgpu

using namespace gfgpu;
using namespace gfgpu::coarse;

// z = P Ainv P^T r (+ minv * r): the correction inside the flexible CG (learned.cu); vc, yc hold
// nc floats each
int gfgpu_internal_coarse_apply(const gfgpu_coarse_desc* g, const int32_t* part, int64_t nnu,
                                const double* minv, const double* r, double* vc, double* yc,
                                double* z, cudaStream_t s)
{
    const int64_t nc = ncoarse(g);
    float* v = reinterpret_cast<float*>(vc);
    float* y = reinterpret_cast<float*>(yc);
    k_restrict<float><<<g->ncx * g->ncy, kRestrictThreads, 0, s>>>(*g, part, nnu, r, v);
    k_dense<<<grid_for(nc, kRowsPerBlock), 32 * kRowsPerBlock, g->ld * sizeof(float), s>>>(g->ainv, nc, g->ld, v, y);
    k_prolong<float><<<grid_for(int64_t(g->nx + 1) * (g->ny + 1)), kBlock, 0, s>>>(*g, part, nnu, y, minv, r, z);
    return check_launch("coarse correction");
}

static int check_grid(const gfgpu_verlet_desc* d, const gfgpu_coarse_desc* g)
{
    GF_REQUIRE(g != nullptr, "bad argument");
    GF_REQUIRE(d && g && d->nne == 4 && d->ndim == 2, "a Quad4 mesh is required");
    GF_REQUIRE(g->nx >= 1 && g->ny >= 1 && g->hc >= 1, "bad coarse grid");
    GF_REQUIRE(int64_t(g->nx + 1) * (g->ny + 1) == d->nnode, "nodes != (nx + 1) (ny + 1)");
    GF_REQUIRE(g->ncx == (g->nx + g->hc - 1) / g->hc + 1 && g->ncy == (g->ny + g->hc - 1) / g->hc + 1,
               "ncx, ncy do not match nx, ny, hc");
    GF_REQUIRE(ncoarse(g) <= kMaxCoarseDofs, "coarse grid too large (more than 8192 coarse dofs)");
    gfgpu_coarse_desc e;
    gfgpu_coarse_grid(g->nx, g->ny, g->hc, &e);
    GF_REQUIRE(g->ld == e.ld && g->rhx == e.rhx && g->rlx == e.rlx && g->rhy == e.rhy && g->rly == e.rly,
               "reciprocal interval lengths do not match nx, ny, hc (use gfgpu_coarse_grid)");
    return GFGPU_OK;
}

extern "C" {

int gfgpu_coarse_grid(int32_t nx, int32_t ny, int32_t hc, gfgpu_coarse_desc* g)
{
    GF_REQUIRE(g && nx >= 1 && ny >= 1 && hc >= 1, "bad argument");
    g->nx = nx;
    g->ny = ny;
    g->hc = hc;
    g->ncx = (nx + hc - 1) / hc + 1;
    g->ncy = (ny + hc - 1) / hc + 1;
    g->ld = static_cast<int32_t>((int64_t(g->ncx) * g->ncy * 2 + 31) / 32 * 32);
    g->ainv = nullptr;
    g->rhx = g->rhy = 1.0 / hc;
    g->rlx = 1.0 / (nx - (g->ncx - 2) * hc);
    g->rly = 1.0 / (ny - (g->ncy - 2) * hc);
    return GFGPU_OK;
}

int64_t gfgpu_coarse_setup_workspace_bytes(const gfgpu_verlet_desc* d, const gfgpu_coarse_desc* g)
{
    if (!d || !g) return 0;
    const int64_t nc = ncoarse(g), n = d->nnode * d->ndim;
    return a256(nc * nc * 8) + 2 * a256(n * 8) + a256(d->nelem * d->nne * d->ndim * 8) + 2 * a256(nc * 8) + 256;
}

int gfgpu_coarse_setup(const gfgpu_verlet_desc* d, const gfgpu_coarse_desc* g, float* ainv,
                       double* ac, void* workspace, gfgpu_stream_t stream)
{
    GF_TRY(check_grid(d, g));
    GF_REQUIRE(ainv && workspace, "bad argument");
    cudaStream_t s = S(stream);
    const int64_t nc = ncoarse(g), n = d->nnode * d->ndim;
    char* c = static_cast<char*>(workspace);
    double* A = reinterpret_cast<double*>(c);
    c += a256(nc * nc * 8);
    double* p = reinterpret_cast<double*>(c);
    c += a256(n * 8);
    double* q = reinterpret_cast<double*>(c);
    c += a256(n * 8);
    double* fe = reinterpret_cast<double*>(c);
    c += a256(d->nelem * d->nne * d->ndim * 8);
    double* e = reinterpret_cast<double*>(c);
    c += a256(nc * 8);
    double* v = reinterpret_cast<double*>(c);
    c += a256(nc * 8);
    double* piv = reinterpret_cast<double*>(c);
    GF_TRY(check_cuda(cudaMemsetAsync(A, 0, nc * nc * 8, s), "cudaMemsetAsync"));
    GF_TRY(check_cuda(cudaMemsetAsync(piv, 0, 16, s), "cudaMemsetAsync"));
    for (int comp = 0; comp < 2; ++comp)
        for (int b = 0; b < 3; ++b)
            for (int a = 0; a < 3; ++a) {
                k_probe<<<grid_for(nc), kBlock, 0, s>>>(*g, a, b, comp, e);
                k_prolong<double><<<grid_for(d->nnode), kBlock, 0, s>>>(*g, d->part, d->nnu, e, nullptr, nullptr,
                                                                        p);
                GF_TRY(gfgpu_internal_element_forces(d, p, fe, s));
                k_apply_gather<<<grid_for(n), kBlock, 0, s>>>(d->dofs, d->csr_ptr, d->csr_idx, d->part,
                                                              d->nnu, fe, n, q, reg_grid(d));
                k_restrict<double><<<g->ncx * g->ncy, kRestrictThreads, 0, s>>>(*g, d->part, d->nnu, q, v);
                k_probe_scatter<<<grid_for(nc), kBlock, 0, s>>>(*g, a, b, comp, v, A);
            }
    k_symmetrize<<<grid_for(nc * nc), kBlock, 0, s>>>(A, nc);
    GF_TRY(check_launch("coarse matrix"));
    if (ac) GF_TRY(check_cuda(cudaMemcpyAsync(ac, A, nc * nc * 8, cudaMemcpyDeviceToDevice, s), "copy"));
    for (int64_t k = 0; k < nc; ++k) {
        k_gj_row<<<grid_for(nc), kBlock, 0, s>>>(A, nc, k, piv);
        k_gj_update<<<dim3(grid_for(nc), static_cast<unsigned>(nc)), kBlock, 0, s>>>(A, nc, k);
        k_gj_col<<<grid_for(nc), kBlock, 0, s>>>(A, nc, k, piv);
    }
    GF_TRY(check_launch("coarse inverse"));
    double flag[2];
    GF_TRY(check_cuda(cudaMemcpyAsync(flag, piv, 16, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync"));
    GF_TRY(check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
    if (flag[1] != 0.0) return fail(GFGPU_ERR_NAN, "gfgpu_coarse_setup: singular coarse matrix");
    k_to_f32<<<grid_for(nc * g->ld), kBlock, 0, s>>>(A, nc, g->ld, ainv);
    return check_launch("coarse inverse f32");
}

int gfgpu_coarse_apply(const gfgpu_verlet_desc* d, const gfgpu_coarse_desc* g, const double* r,
                       double* z, void* workspace, gfgpu_stream_t stream)
{
    GF_TRY(check_grid(d, g));
    GF_REQUIRE(g->ainv && r && z && workspace, "bad argument");
    const int64_t nc = ncoarse(g);
    double* vc = static_cast<double*>(workspace);
    double* yc = vc + a256(nc * 8) / 8;
    return gfgpu_internal_coarse_apply(g, d->part, d->nnu, nullptr, r, vc, yc, z, S(stream));
}

} // extern "C"
