// Host-side set-up of the gfgpu library: error reporting and the integer bookkeeping of
// GooseFEM's Mesh / Vector / partitioned classes (run once per mesh, bit-exact).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gfgpu.h"

namespace gfgpu {

static thread_local std::string g_last_error;
static int g_strict = 0;
static int g_variant_elem = 0;
static int g_variant_node = 0;
static int g_nn_path = 2; // tcgen05 + TMA (the fastest form on GB300)
static int g_pair_kernel = 2; // persistent TMA pipeline, 31 x 15 node tiles

int pair_kernel()
{
    return g_pair_kernel;
}

int nn_tensor_path()
{
    return g_nn_path;
}

int variant_elem()
{
    return g_variant_elem;
}

int variant_node()
{
    return g_variant_node;
}

void set_error(const std::string& msg)
{
    g_last_error = msg;
}

int fail(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

bool strict_mode()
{
    return g_strict != 0;
}

} // namespace gfgpu

using gfgpu::fail;

#define HREQ(cond, msg)                                                                         \
    do {                                                                                        \
        if (!(cond)) return fail(GFGPU_ERR_ARG, std::string(__func__) + ": " + (msg));         \
    } while (0)

static bool fits32(int64_t n)
{
    return n >= 0 && n <= INT32_MAX;
}

extern "C" {

const char* gfgpu_last_error(void)
{
    return gfgpu::g_last_error.c_str();
}

const char* gfgpu_version(void)
{
    return "gfgpu 0.1 (sm_103a)";
}

int gfgpu_set_strict(int strict)
{
    gfgpu::g_strict = strict ? 1 : 0;
    return GFGPU_OK;
}

int gfgpu_set_variant(int elem_variant, int node_variant)
{
    if (elem_variant < 0 || elem_variant > 1 || node_variant < 0 || node_variant > 1)
        return fail(GFGPU_ERR_ARG, "gfgpu_set_variant: variants are 0 or 1");
    gfgpu::g_variant_elem = elem_variant;
    gfgpu::g_variant_node = node_variant;
    return GFGPU_OK;
}

int gfgpu_set_pair_kernel(int kernel)
{
    if (kernel < 0 || kernel > 2) return fail(GFGPU_ERR_ARG, "gfgpu_set_pair_kernel: kernel is 0, 1 or 2");
    gfgpu::g_pair_kernel = kernel;
    return GFGPU_OK;
}

int gfgpu_set_nn_tensor_path(int path)
{
    if (path < 0 || path > 3) return fail(GFGPU_ERR_ARG, "gfgpu_set_nn_tensor_path: path is 0, 1, 2 or 3");
    gfgpu::g_nn_path = path;
    return GFGPU_OK;
}

// xt::linspace(start, stop, num)[i] = start + i * step, step = (stop - start) / (num - 1).
static double linspace_at(double start, double stop, int64_t num, int64_t i)
{
    double step = (stop - start) / static_cast<double>(num - 1);
    return start + step * static_cast<double>(i);
}

int gfgpu_host_quad4_regular(int64_t nx, int64_t ny, double h, double* coor, int32_t* conn)
{
    HREQ(nx >= 1 && ny >= 1, "nelx, nely must be >= 1");
    HREQ(fits32((nx + 1) * (ny + 1)) && fits32(nx * ny * 4), "mesh too large for int32 tables");
    HREQ(coor && conn, "null pointer");
    int64_t inode = 0;
    for (int64_t iy = 0; iy < ny + 1; ++iy) {
        double y = linspace_at(0.0, h * static_cast<double>(ny), ny + 1, iy);
        for (int64_t ix = 0; ix < nx + 1; ++ix) {
            coor[inode * 2 + 0] = linspace_at(0.0, h * static_cast<double>(nx), nx + 1, ix);
            coor[inode * 2 + 1] = y;
            ++inode;
        }
    }
    int64_t e = 0;
    for (int64_t iy = 0; iy < ny; ++iy) {
        for (int64_t ix = 0; ix < nx; ++ix) {
            int32_t* c = conn + e * 4;
            c[0] = static_cast<int32_t>(iy * (nx + 1) + ix);
            c[1] = static_cast<int32_t>(iy * (nx + 1) + ix + 1);
            c[2] = static_cast<int32_t>((iy + 1) * (nx + 1) + ix + 1);
            c[3] = static_cast<int32_t>((iy + 1) * (nx + 1) + ix);
            ++e;
        }
    }
    return GFGPU_OK;
}

int gfgpu_host_hex8_regular(int64_t nx, int64_t ny, int64_t nz, double h, double* coor,
                            int32_t* conn)
{
    HREQ(nx >= 1 && ny >= 1 && nz >= 1, "nelx, nely, nelz must be >= 1");
    HREQ(fits32((nx + 1) * (ny + 1) * (nz + 1)) && fits32(nx * ny * nz * 8),
         "mesh too large for int32 tables");
    HREQ(coor && conn, "null pointer");
    int64_t inode = 0;
    for (int64_t iz = 0; iz < nz + 1; ++iz)
        for (int64_t iy = 0; iy < ny + 1; ++iy)
            for (int64_t ix = 0; ix < nx + 1; ++ix) {
                coor[inode * 3 + 0] = linspace_at(0.0, h * static_cast<double>(nx), nx + 1, ix);
                coor[inode * 3 + 1] = linspace_at(0.0, h * static_cast<double>(ny), ny + 1, iy);
                coor[inode * 3 + 2] = linspace_at(0.0, h * static_cast<double>(nz), nz + 1, iz);
                ++inode;
            }
    int64_t nxy = (nx + 1) * (ny + 1);
    int64_t e = 0;
    for (int64_t iz = 0; iz < nz; ++iz)
        for (int64_t iy = 0; iy < ny; ++iy)
            for (int64_t ix = 0; ix < nx; ++ix) {
                int64_t b = iy * (nx + 1) + ix + iz * nxy;
                int32_t* c = conn + e * 8;
                c[0] = static_cast<int32_t>(b);
                c[1] = static_cast<int32_t>(b + 1);
                c[2] = static_cast<int32_t>(b + (nx + 1) + 1);
                c[3] = static_cast<int32_t>(b + (nx + 1));
                c[4] = static_cast<int32_t>(b + nxy);
                c[5] = static_cast<int32_t>(b + nxy + 1);
                c[6] = static_cast<int32_t>(b + nxy + (nx + 1) + 1);
                c[7] = static_cast<int32_t>(b + nxy + (nx + 1));
                ++e;
            }
    return GFGPU_OK;
}

int gfgpu_host_dofs(int64_t nnode, int32_t ndim, int32_t* dofs)
{
    HREQ(fits32(nnode * ndim) && ndim > 0, "bad size");
    for (int64_t i = 0; i < nnode * ndim; ++i) dofs[i] = static_cast<int32_t>(i);
    return GFGPU_OK;
}

int gfgpu_host_quad4_nodes_periodic(int64_t nx, int64_t ny, int32_t* out, int64_t* nper)
{
    HREQ(nx >= 1 && ny >= 1 && out && nper, "bad argument");
    int64_t n = 0;
    auto put = [&](int64_t a, int64_t b) {
        out[n * 2 + 0] = static_cast<int32_t>(a);
        out[n * 2 + 1] = static_cast<int32_t>(b);
        ++n;
    };
    int64_t bl = 0, br = nx, tl = ny * (nx + 1), tr = ny * (nx + 1) + nx;
    put(bl, br);
    put(bl, tr);
    put(bl, tl);
    for (int64_t i = 1; i < nx; ++i) put(i, i + ny * (nx + 1));
    for (int64_t i = 1; i < ny; ++i) put(i * (nx + 1), i * (nx + 1) + nx);
    *nper = n;
    return GFGPU_OK;
}

int gfgpu_host_hex8_nodes_periodic(int64_t nx, int64_t ny, int64_t nz, int32_t* out, int64_t* nper)
{
    HREQ(nx >= 1 && ny >= 1 && nz >= 1 && out && nper, "bad argument");
    HREQ(fits32((nx + 1) * (ny + 1) * (nz + 1)), "too many nodes");
    const int64_t sy = nx + 1, sz = (nx + 1) * (ny + 1);
    int64_t n = 0;
    auto put = [&](int64_t a, int64_t b) {
        out[n * 2 + 0] = static_cast<int32_t>(a);
        out[n * 2 + 1] = static_cast<int32_t>(b);
        ++n;
    };
    // offsets of the far side along x, y, z
    const int64_t X = nx, Y = ny * sy, Z = nz * sz;
    // corners: every other corner tied to the origin (front-bottom-left)
    for (int64_t c : {X, X + Z, Z, Y, X + Y, X + Y + Z, Y + Z}) put(0, c);
    // open edges along x, then along z, then along y, each tied to the three parallel edges
    for (int64_t dst : {Z, Y + Z, Y})
        for (int64_t i = 1; i < nx; ++i) put(i, i + dst);
    for (int64_t dst : {X, X + Y, Y})
        for (int64_t i = 1; i < nz; ++i) put(i * sz, i * sz + dst);
    for (int64_t dst : {X, X + Z, Z})
        for (int64_t i = 1; i < ny; ++i) put(i * sy, i * sy + dst);
    // open faces: front -> back (iy outer), left -> right (iz outer), bottom -> top (iz outer)
    for (int64_t iy = 1; iy < ny; ++iy)
        for (int64_t ix = 1; ix < nx; ++ix) put(ix + iy * sy, ix + iy * sy + Z);
    for (int64_t iz = 1; iz < nz; ++iz)
        for (int64_t iy = 1; iy < ny; ++iy) put(iy * sy + iz * sz, iy * sy + iz * sz + X);
    for (int64_t iz = 1; iz < nz; ++iz)
        for (int64_t ix = 1; ix < nx; ++ix) put(ix + iz * sz, ix + iz * sz + Y);
    *nper = n;
    return GFGPU_OK;
}

int gfgpu_host_renumber(const int32_t* in, int64_t n, int32_t* out)
{
    HREQ(n >= 0 && (n == 0 || (in && out)), "bad argument");
    if (n == 0) return GFGPU_OK;
    int32_t mn = *std::min_element(in, in + n);
    HREQ(mn >= 0, "negative entry");
    int32_t mx = *std::max_element(in, in + n);
    std::vector<int32_t> renum(static_cast<size_t>(mx) + 1, -1);
    for (int64_t i = 0; i < n; ++i) renum[in[i]] = 0;
    int32_t k = 0;
    for (auto& r : renum)
        if (r == 0) r = k++;
    for (int64_t i = 0; i < n; ++i) out[i] = renum[in[i]];
    return GFGPU_OK;
}

int gfgpu_host_dofs_periodic(int64_t nnode, int32_t ndim, const int32_t* nodes_periodic,
                             int64_t nper, int32_t* dofs)
{
    HREQ(fits32(nnode * ndim) && ndim > 0 && dofs, "bad argument");
    std::vector<int32_t> ret(nnode * ndim);
    for (int64_t i = 0; i < nnode * ndim; ++i) ret[i] = static_cast<int32_t>(i);
    for (int64_t k = 0; k < nper; ++k) {
        int32_t a = nodes_periodic[k * 2 + 0], b = nodes_periodic[k * 2 + 1];
        if (a < 0 || a >= nnode || b < 0 || b >= nnode)
            return fail(GFGPU_ERR_INDEX, "gfgpu_host_dofs_periodic: node index out of range");
    }
    // the right-hand side (dofs of the independent nodes) is read before any assignment
    for (int32_t j = 0; j < ndim; ++j) {
        std::vector<int32_t> rhs(nper);
        for (int64_t k = 0; k < nper; ++k) rhs[k] = ret[nodes_periodic[k * 2 + 0] * ndim + j];
        for (int64_t k = 0; k < nper; ++k) ret[nodes_periodic[k * 2 + 1] * ndim + j] = rhs[k];
    }
    return gfgpu_host_renumber(ret.data(), nnode * ndim, dofs);
}

int gfgpu_host_partition(const int32_t* dofs, int64_t n, const int32_t* iip, int64_t nnp,
                         int32_t* iiu, int32_t* part, int64_t* nnu)
{
    HREQ(n > 0 && dofs && iiu && part && nnu && (nnp == 0 || iip), "bad argument");
    int32_t mx = *std::max_element(dofs, dofs + n);
    std::vector<char> present(static_cast<size_t>(mx) + 1, 0), pres(static_cast<size_t>(mx) + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        if (dofs[i] < 0) return fail(GFGPU_ERR_INDEX, "gfgpu_host_partition: negative dof");
        present[dofs[i]] = 1;
    }
    for (int64_t i = 0; i < nnp; ++i) {
        if (iip[i] < 0 || iip[i] > mx)
            return fail(GFGPU_ERR_INDEX, "gfgpu_host_partition: iip out of range");
        if (pres[iip[i]]) return fail(GFGPU_ERR_ARG, "gfgpu_host_partition: iip is not unique");
        pres[iip[i]] = 1;
    }
    int64_t u = 0;
    for (int32_t j = 0; j <= mx; ++j)
        if (present[j] && !pres[j]) iiu[u++] = j;
    std::vector<int32_t> renum(static_cast<size_t>(mx) + 1, 0);
    int32_t k = 0;
    for (int64_t i = 0; i < u; ++i) renum[iiu[i]] = k++;
    for (int64_t i = 0; i < nnp; ++i) renum[iip[i]] = k++;
    for (int64_t i = 0; i < n; ++i) part[i] = renum[dofs[i]];
    *nnu = u;
    return GFGPU_OK;
}

int gfgpu_host_coordination(const int32_t* conn, int64_t nelem, int32_t nne, int64_t nnode,
                            int32_t* N)
{
    HREQ(conn && N && nne > 0, "bad argument");
    std::fill(N, N + nnode, 0);
    for (int64_t i = 0; i < nelem * nne; ++i) {
        if (conn[i] < 0 || conn[i] >= nnode)
            return fail(GFGPU_ERR_INDEX, "gfgpu_host_coordination: conn out of range");
        N[conn[i]] += 1;
    }
    return GFGPU_OK;
}

int gfgpu_host_elem2node(const int32_t* conn, int64_t nelem, int32_t nne, int64_t nnode,
                         int32_t* ptr, int32_t* idx)
{
    HREQ(conn && ptr && idx && nne > 0 && fits32(nelem * nne), "bad argument");
    std::vector<int32_t> N(nnode);
    int rc = gfgpu_host_coordination(conn, nelem, nne, nnode, N.data());
    if (rc != GFGPU_OK) return rc;
    ptr[0] = 0;
    for (int64_t i = 0; i < nnode; ++i) ptr[i + 1] = ptr[i] + N[i];
    std::vector<int32_t> cur(ptr, ptr + nnode);
    // elements are visited in ascending order, so every row comes out sorted
    for (int64_t e = 0; e < nelem; ++e)
        for (int32_t m = 0; m < nne; ++m) idx[cur[conn[e * nne + m]]++] = static_cast<int32_t>(e);
    return GFGPU_OK;
}

int gfgpu_host_dof_csr(const int32_t* conn, const int32_t* dofs, int64_t nelem, int32_t nne,
                       int64_t nnode, int32_t ndim, int64_t ndof, int32_t* ptr, int32_t* idx)
{
    HREQ(conn && dofs && ptr && idx && nne > 0 && ndim > 0, "bad argument");
    HREQ(fits32(nelem * nne * ndim) && fits32(ndof), "too large for int32 tables");
    std::vector<int32_t> cnt(ndof + 1, 0);
    for (int64_t k = 0; k < nelem * nne; ++k) {
        int32_t n = conn[k];
        if (n < 0 || n >= nnode) return fail(GFGPU_ERR_INDEX, "gfgpu_host_dof_csr: conn out of range");
        for (int32_t i = 0; i < ndim; ++i) {
            int32_t d = dofs[static_cast<int64_t>(n) * ndim + i];
            if (d < 0 || d >= ndof) return fail(GFGPU_ERR_INDEX, "gfgpu_host_dof_csr: dof out of range");
            cnt[d + 1] += 1;
        }
    }
    ptr[0] = 0;
    for (int64_t d = 0; d < ndof; ++d) ptr[d + 1] = ptr[d] + cnt[d + 1];
    std::vector<int32_t> cur(ptr, ptr + ndof);
    // ascending flat index (e, m, i): the serial summation order of Vector.h:724-741
    for (int64_t k = 0; k < nelem * nne; ++k) {
        int32_t n = conn[k];
        for (int32_t i = 0; i < ndim; ++i) {
            int32_t d = dofs[static_cast<int64_t>(n) * ndim + i];
            idx[cur[d]++] = static_cast<int32_t>(k * ndim + i);
        }
    }
    return GFGPU_OK;
}

int gfgpu_host_matrix_pattern(const int32_t* conn, const int32_t* dmap, int64_t nelem, int32_t nne,
                              int64_t nnode, int32_t ndim, int64_t n, int32_t* rowptr,
                              int32_t* col, int32_t* cptr, int32_t* cidx, int64_t* nnz)
{
    HREQ(conn && dmap && rowptr && col && cptr && cidx && nnz && nne > 0 && ndim > 0 && n >= 0,
         "bad argument");
    const int64_t K = int64_t(nne) * ndim;
    const int64_t total = nelem * K * K;
    HREQ(fits32(total) && fits32(n), "too large for int32 tables");
    for (int64_t k = 0; k < nelem * nne; ++k)
        if (conn[k] < 0 || conn[k] >= nnode)
            return fail(GFGPU_ERR_INDEX, "gfgpu_host_matrix_pattern: conn out of range");
    for (int64_t k = 0; k < nnode * ndim; ++k)
        if (dmap[k] < 0 || dmap[k] >= n)
            return fail(GFGPU_ERR_INDEX, "gfgpu_host_matrix_pattern: dof out of range");
    // (row, col) of the triplet with flat elemmat index f = (e K + m ndim + i) K + n ndim + j: the
    // push order of Matrix.h:704-733 / MatrixPartitioned.h:156-200
    auto rc = [&](int64_t f, int32_t& r, int32_t& c) {
        int64_t e = f / (K * K), rem = f % (K * K);
        int64_t a = rem / K, b = rem % K;
        r = dmap[int64_t(conn[e * nne + a / ndim]) * ndim + a % ndim];
        c = dmap[int64_t(conn[e * nne + b / ndim]) * ndim + b % ndim];
    };
    // bucket by row, stable in f
    std::vector<int64_t> start(n + 1, 0);
    for (int64_t f = 0; f < total; ++f) {
        int32_t r, c;
        rc(f, r, c);
        start[r + 1] += 1;
    }
    for (int64_t r = 0; r < n; ++r) start[r + 1] += start[r];
    std::vector<int64_t> cur(start.begin(), start.end() - 1);
    std::vector<int32_t> colof(total);
    for (int64_t f = 0; f < total; ++f) {
        int32_t r, c;
        rc(f, r, c);
        cidx[cur[r]++] = static_cast<int32_t>(f);
        colof[f] = c;
    }
    // within a row: stable by column (triplet order kept among duplicates), then one nonzero per
    // distinct column
    int64_t k = 0;
    rowptr[0] = 0;
    for (int64_t r = 0; r < n; ++r) {
        std::stable_sort(cidx + start[r], cidx + start[r + 1],
                         [&](int32_t a, int32_t b) { return colof[a] < colof[b]; });
        for (int64_t q = start[r]; q < start[r + 1]; ++q) {
            if (q == start[r] || colof[cidx[q]] != colof[cidx[q - 1]]) {
                col[k] = colof[cidx[q]];
                cptr[k] = static_cast<int32_t>(q);
                ++k;
            }
        }
        rowptr[r + 1] = static_cast<int32_t>(k);
    }
    cptr[k] = static_cast<int32_t>(total);
    *nnz = k;
    return GFGPU_OK;
}

int gfgpu_host_tyings_periodic(const int32_t* dofs, int64_t nnode, int32_t ndim,
                               const int32_t* control_dofs, const int32_t* tyings, int64_t nties,
                               const int32_t* iip, int64_t nnp, int32_t* dofs_out,
                               int32_t* control_out, int64_t* counts)
{
    HREQ(dofs && control_dofs && dofs_out && control_out && counts && nnode > 0 && ndim > 0,
         "bad argument");
    HREQ((nties == 0 || tyings) && (nnp == 0 || iip) && nties >= 0 && nnp >= 0, "bad argument");
    const int64_t n = nnode * ndim;
    HREQ(fits32(n), "too large for int32 tables");
    int32_t mn = *std::min_element(dofs, dofs + n), mx = *std::max_element(dofs, dofs + n);
    if (mn < 0) return fail(GFGPU_ERR_INDEX, "gfgpu_host_tyings_periodic: negative dof");
    for (int64_t k = 0; k < int64_t(ndim) * ndim; ++k)
        if (control_dofs[k] < mn || control_dofs[k] > mx)
            return fail(GFGPU_ERR_INDEX, "gfgpu_host_tyings_periodic: control dof out of range");
    for (int64_t k = 0; k < nnp; ++k)
        if (iip[k] < mn || iip[k] > mx)
            return fail(GFGPU_ERR_INDEX, "gfgpu_host_tyings_periodic: iip out of range");
    for (int64_t k = 0; k < 2 * nties; ++k)
        if (tyings[k] < 0 || tyings[k] >= nnode)
            return fail(GFGPU_ERR_INDEX, "gfgpu_host_tyings_periodic: tying node out of range");
    // iid = flatten(dofs[dependent nodes]), iii = setdiff1d(dofs, iid), iiu = setdiff1d(iii, iip)
    // (TyingsPeriodic.h:105-109); Reorder({iiu, iip, iid}) (Mesh.h:2384-2450)
    std::vector<int32_t> iid;
    iid.reserve(static_cast<size_t>(nties) * ndim);
    std::vector<char> dep(static_cast<size_t>(mx) + 1, 0), pre(static_cast<size_t>(mx) + 1, 0),
        present(static_cast<size_t>(mx) + 1, 0);
    for (int64_t t = 0; t < nties; ++t)
        for (int32_t j = 0; j < ndim; ++j) {
            int32_t d = dofs[int64_t(tyings[2 * t + 1]) * ndim + j];
            iid.push_back(d);
            dep[d] = 1;
        }
    for (int64_t k = 0; k < nnp; ++k) pre[iip[k]] = 1;
    for (int64_t k = 0; k < n; ++k) present[dofs[k]] = 1;
    std::vector<int32_t> renum(static_cast<size_t>(mx) + 1, 0);
    int32_t next = 0;
    int64_t nni = 0, nnu = 0;
    for (int32_t d = 0; d <= mx; ++d)
        if (present[d] && !dep[d]) {
            ++nni;
            if (!pre[d]) {
                renum[d] = next++;
                ++nnu;
            }
        }
    for (int64_t k = 0; k < nnp; ++k) renum[iip[k]] = next++;
    for (int32_t d : iid) renum[d] = next++;
    for (int64_t k = 0; k < n; ++k) dofs_out[k] = renum[dofs[k]];
    for (int64_t k = 0; k < int64_t(ndim) * ndim; ++k) control_out[k] = renum[control_dofs[k]];
    counts[0] = nnu;
    counts[1] = nnp;
    counts[2] = nni;
    counts[3] = static_cast<int64_t>(iid.size());
    return GFGPU_OK;
}

int gfgpu_host_tyings_cdi(const double* coor, const int32_t* tdofs, const int32_t* tcontrol,
                          const int32_t* tyings, int64_t nties, int32_t ndim, int32_t* rowptr,
                          int32_t* col, double* val, int64_t* nnz)
{
    HREQ(coor && tdofs && tcontrol && rowptr && col && val && nnz && ndim > 0 && nties >= 0 &&
             (nties == 0 || tyings),
         "bad argument");
    // TyingsPeriodic.h:238-264: row i*ndim+j gets (dofs(ni, j), +1) and, per k,
    // (control(j, k), x(nd, k) - x(ni, k)); setFromTriplets sums equal columns in push order and
    // sorts each row's columns
    int64_t k = 0;
    rowptr[0] = 0;
    std::vector<std::pair<int32_t, double>> row;
    for (int64_t i = 0; i < nties; ++i) {
        int64_t ni = tyings[2 * i], nd = tyings[2 * i + 1];
        for (int32_t j = 0; j < ndim; ++j) {
            row.clear();
            row.emplace_back(tdofs[ni * ndim + j], 1.0);
            for (int32_t q = 0; q < ndim; ++q)
                row.emplace_back(tcontrol[j * ndim + q], coor[nd * ndim + q] - coor[ni * ndim + q]);
            std::stable_sort(row.begin(), row.end(),
                             [](const std::pair<int32_t, double>& a, const std::pair<int32_t, double>& b) {
                                 return a.first < b.first;
                             });
            for (size_t q = 0; q < row.size(); ++q) {
                if (q > 0 && row[q].first == row[q - 1].first) {
                    val[k - 1] = val[k - 1] + row[q].second;
                }
                else {
                    col[k] = row[q].first;
                    val[k] = row[q].second;
                    ++k;
                }
            }
            rowptr[i * ndim + j + 1] = static_cast<int32_t>(k);
        }
    }
    *nnz = k;
    return GFGPU_OK;
}

int gfgpu_host_csr_transpose(const int32_t* rowptr, const int32_t* col, const double* val,
                             int64_t nrow, int64_t ncol, int32_t* trowptr, int32_t* tcol,
                             double* tval)
{
    HREQ(rowptr && col && val && trowptr && tcol && tval && nrow >= 0 && ncol >= 0, "bad argument");
    int64_t nnz = rowptr[nrow];
    std::fill(trowptr, trowptr + ncol + 1, 0);
    for (int64_t k = 0; k < nnz; ++k) {
        if (col[k] < 0 || col[k] >= ncol) return fail(GFGPU_ERR_INDEX, "gfgpu_host_csr_transpose: column out of range");
        trowptr[col[k] + 1] += 1;
    }
    for (int64_t c = 0; c < ncol; ++c) trowptr[c + 1] += trowptr[c];
    std::vector<int32_t> cur(trowptr, trowptr + ncol);
    // rows visited in ascending order: every output row is sorted by the original row
    for (int64_t r = 0; r < nrow; ++r)
        for (int32_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
            int32_t q = cur[col[k]]++;
            tcol[q] = static_cast<int32_t>(r);
            tval[q] = val[k];
        }
    return GFGPU_OK;
}

int gfgpu_host_dof_csr_nodevec(const int32_t* dofs, int64_t nnode, int32_t ndim, int64_t ndof,
                               int32_t* ptr, int32_t* idx)
{
    HREQ(dofs && ptr && idx && ndim > 0 && fits32(nnode * ndim), "bad argument");
    std::vector<int32_t> cnt(ndof + 1, 0);
    for (int64_t k = 0; k < nnode * ndim; ++k) {
        if (dofs[k] < 0 || dofs[k] >= ndof)
            return fail(GFGPU_ERR_INDEX, "gfgpu_host_dof_csr_nodevec: dof out of range");
        cnt[dofs[k] + 1] += 1;
    }
    ptr[0] = 0;
    for (int64_t d = 0; d < ndof; ++d) ptr[d + 1] = ptr[d] + cnt[d + 1];
    std::vector<int32_t> cur(ptr, ptr + ndof);
    for (int64_t k = 0; k < nnode * ndim; ++k) idx[cur[dofs[k]]++] = static_cast<int32_t>(k);
    return GFGPU_OK;
}

} // extern "C"
