// CPU ORACLE — test infrastructure only.
//
// A plain C++17 restatement of GooseFEM's element hot path, used by the tests,
// by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
// It is never part of the shipped GPU path.
//
// Every function restates the reference loop nest and summation order of the
// file:line it cites (paths relative to the GooseFEM source tree). Built with
// -O3 -ffp-contract=off so that x86_64 and aarch64 give identical bits.
// Compiled twice: serial (the reference as shipped, whose OpenMP pragmas are
// inert) and with -fopenmp (the reference's element-loop pragmas enabled; the
// assembly loops stay serial exactly as in the reference).
//
// The reference itself cannot be compiled here: it needs xtensor (and Eigen for
// Matrix*.h), neither of which is installed. Parity of this restatement is
// pinned instead against the golden arrays and known-answer tests of the
// reference's own test-suite (tests/basic/*.cpp), extracted into tests/golden/.
//
// Index arrays are int64 (the reference's size_t), values are double.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iterator>
#include <limits>
#include <map>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#define GF_OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define GF_OMP_FOR
#endif

typedef int64_t idx;

extern "C" {

int ref_num_threads()
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// ------------------------------------------------------------------------------------------------
// Mesh
// ------------------------------------------------------------------------------------------------

// xt::linspace(start, stop, num): start + i * step, step = (stop - start) / (num - 1).
static inline double linspace_at(double start, double stop, idx num, idx i)
{
    double step = (stop - start) / static_cast<double>(num - 1);
    return start + step * static_cast<double>(i);
}

// MeshQuad4.h:87-107 (coor_impl) and :109-126 (conn_impl).
void ref_quad4_regular(idx nx, idx ny, double h, double* coor, idx* conn)
{
    idx inode = 0;
    for (idx iy = 0; iy < ny + 1; ++iy) {
        for (idx ix = 0; ix < nx + 1; ++ix) {
            coor[inode * 2 + 0] = linspace_at(0.0, h * static_cast<double>(nx), nx + 1, ix);
            coor[inode * 2 + 1] = linspace_at(0.0, h * static_cast<double>(ny), ny + 1, iy);
            ++inode;
        }
    }
    idx ielem = 0;
    for (idx iy = 0; iy < ny; ++iy) {
        for (idx ix = 0; ix < nx; ++ix) {
            conn[ielem * 4 + 0] = iy * (nx + 1) + ix;
            conn[ielem * 4 + 1] = iy * (nx + 1) + (ix + 1);
            conn[ielem * 4 + 3] = (iy + 1) * (nx + 1) + ix;
            conn[ielem * 4 + 2] = (iy + 1) * (nx + 1) + (ix + 1);
            ++ielem;
        }
    }
}

// MeshHex8.h:77-102 (coor_impl) and :104-130 (conn_impl).
void ref_hex8_regular(idx nx, idx ny, idx nz, double h, double* coor, idx* conn)
{
    idx inode = 0;
    for (idx iz = 0; iz < nz + 1; ++iz) {
        for (idx iy = 0; iy < ny + 1; ++iy) {
            for (idx ix = 0; ix < nx + 1; ++ix) {
                coor[inode * 3 + 0] = linspace_at(0.0, h * static_cast<double>(nx), nx + 1, ix);
                coor[inode * 3 + 1] = linspace_at(0.0, h * static_cast<double>(ny), ny + 1, iy);
                coor[inode * 3 + 2] = linspace_at(0.0, h * static_cast<double>(nz), nz + 1, iz);
                ++inode;
            }
        }
    }
    idx ielem = 0;
    idx nxy = (ny + 1) * (nx + 1);
    for (idx iz = 0; iz < nz; ++iz) {
        for (idx iy = 0; iy < ny; ++iy) {
            for (idx ix = 0; ix < nx; ++ix) {
                idx* c = conn + ielem * 8;
                c[0] = iy * (nx + 1) + ix + iz * nxy;
                c[1] = iy * (nx + 1) + (ix + 1) + iz * nxy;
                c[3] = (iy + 1) * (nx + 1) + ix + iz * nxy;
                c[2] = (iy + 1) * (nx + 1) + (ix + 1) + iz * nxy;
                c[4] = iy * (nx + 1) + ix + (iz + 1) * nxy;
                c[5] = iy * (nx + 1) + (ix + 1) + (iz + 1) * nxy;
                c[7] = (iy + 1) * (nx + 1) + ix + (iz + 1) * nxy;
                c[6] = (iy + 1) * (nx + 1) + (ix + 1) + (iz + 1) * nxy;
                ++ielem;
            }
        }
    }
}

// Mesh.h:511-540 (RegularBase2d::nodesPeriodic_impl) with the Quad4 edge sets of
// MeshQuad4.h:128-186. Output: [(nx-1) + (ny-1) + 3, 2] (independent, dependent).
idx ref_quad4_nodes_periodic(idx nx, idx ny, idx* out)
{
    idx n = 0;
    idx bl = 0, br = nx, tl = ny * (nx + 1), tr = ny * (nx + 1) + nx;
    out[n * 2 + 0] = bl; out[n * 2 + 1] = br; ++n;
    out[n * 2 + 0] = bl; out[n * 2 + 1] = tr; ++n;
    out[n * 2 + 0] = bl; out[n * 2 + 1] = tl; ++n;
    for (idx i = 1; i < nx; ++i) { // bottom open edge -> top open edge
        out[n * 2 + 0] = i;
        out[n * 2 + 1] = i + ny * (nx + 1);
        ++n;
    }
    for (idx i = 1; i < ny; ++i) { // left open edge -> right open edge
        out[n * 2 + 0] = i * (nx + 1);
        out[n * 2 + 1] = i * (nx + 1) + nx;
        ++n;
    }
    return n;
}

// Mesh.h:1577-1692 (RegularBase3d::nodesPeriodic_impl) with the Hex8 face, open-edge and corner
// sets of MeshHex8.h:214-600, written as the reference lists them: 7 corners tied to the origin,
// then the open edges of each axis direction, then the open faces.
idx ref_hex8_nodes_periodic(idx nx, idx ny, idx nz, idx* out)
{
    idx nxy = (nx + 1) * (ny + 1);
    auto node = [&](idx ix, idx iy, idx iz) { return ix + iy * (nx + 1) + iz * nxy; };
    std::vector<idx> froBot, bckBot, bckTop, froTop, botLft, botRgt, topRgt, topLft, froLft, froRgt,
        bckRgt, bckLft, fro, bck, lft, rgt, bot, top;
    for (idx ix = 1; ix < nx; ++ix) {
        froBot.push_back(node(ix, 0, 0));
        froTop.push_back(node(ix, ny, 0));
        bckBot.push_back(node(ix, 0, nz));
        bckTop.push_back(node(ix, ny, nz));
    }
    for (idx iz = 1; iz < nz; ++iz) {
        botLft.push_back(node(0, 0, iz));
        botRgt.push_back(node(nx, 0, iz));
        topLft.push_back(node(0, ny, iz));
        topRgt.push_back(node(nx, ny, iz));
    }
    for (idx iy = 1; iy < ny; ++iy) {
        froLft.push_back(node(0, iy, 0));
        froRgt.push_back(node(nx, iy, 0));
        bckLft.push_back(node(0, iy, nz));
        bckRgt.push_back(node(nx, iy, nz));
    }
    for (idx iy = 1; iy < ny; ++iy)
        for (idx ix = 1; ix < nx; ++ix) {
            fro.push_back(node(ix, iy, 0));
            bck.push_back(node(ix, iy, nz));
        }
    for (idx iz = 1; iz < nz; ++iz)
        for (idx iy = 1; iy < ny; ++iy) {
            lft.push_back(node(0, iy, iz));
            rgt.push_back(node(nx, iy, iz));
        }
    for (idx iz = 1; iz < nz; ++iz)
        for (idx ix = 1; ix < nx; ++ix) {
            bot.push_back(node(ix, 0, iz));
            top.push_back(node(ix, ny, iz));
        }
    idx n = 0;
    auto put = [&](idx a, idx b) {
        out[n * 2 + 0] = a;
        out[n * 2 + 1] = b;
        ++n;
    };
    idx o = node(0, 0, 0);
    put(o, node(nx, 0, 0));
    put(o, node(nx, 0, nz));
    put(o, node(0, 0, nz));
    put(o, node(0, ny, 0));
    put(o, node(nx, ny, 0));
    put(o, node(nx, ny, nz));
    put(o, node(0, ny, nz));
    auto pairs = [&](const std::vector<idx>& a, const std::vector<idx>& b) {
        for (size_t j = 0; j < a.size(); ++j) put(a[j], b[j]);
    };
    pairs(froBot, bckBot);
    pairs(froBot, bckTop);
    pairs(froBot, froTop);
    pairs(botLft, botRgt);
    pairs(botLft, topRgt);
    pairs(botLft, topLft);
    pairs(froLft, froRgt);
    pairs(froLft, bckRgt);
    pairs(froLft, bckLft);
    pairs(fro, bck);
    pairs(lft, rgt);
    pairs(bot, top);
    return n;
}

// Mesh.h:114-166 (Renumber): ret = index-in-sorted-unique-list of each entry.
void ref_renumber(const idx* in, idx n, idx* out)
{
    if (n == 0) return;
    idx mx = *std::max_element(in, in + n);
    std::vector<char> present(mx + 1, 0);
    for (idx i = 0; i < n; ++i) present[in[i]] = 1;
    std::vector<idx> renum(mx + 1, 0);
    idx k = 0;
    for (idx j = 0; j <= mx; ++j) {
        if (present[j]) renum[j] = k++;
    }
    for (idx i = 0; i < n; ++i) out[i] = renum[in[i]];
}

// Mesh.h:93-96 (dofs) then Mesh.h:291-306 (dofsPeriodic): the dependent node takes the
// dofs of its independent node (the right-hand side is evaluated before assignment,
// as xtensor does for non-noalias view assignment), then renumber.
void ref_dofs_periodic(idx nnode, idx ndim, const idx* nodes_periodic, idx nper, idx* dofs)
{
    std::vector<idx> base(nnode * ndim);
    for (idx i = 0; i < nnode * ndim; ++i) base[i] = i;
    std::vector<idx> ret = base;
    for (idx j = 0; j < ndim; ++j) {
        std::vector<idx> rhs(nper);
        for (idx k = 0; k < nper; ++k) rhs[k] = ret[nodes_periodic[k * 2 + 0] * ndim + j];
        for (idx k = 0; k < nper; ++k) ret[nodes_periodic[k * 2 + 1] * ndim + j] = rhs[k];
    }
    ref_renumber(ret.data(), nnode * ndim, dofs);
}

// VectorPartitioned.h:72-88 / MatrixDiagonalPartitioned.h:42-70:
// iiu = setdiff1d(dofs, iip) (sorted unique), part = Reorder({iiu, iip}).apply(dofs)
// (Mesh.h:2384-2450). Returns nnu.
idx ref_partition(const idx* dofs, idx n, const idx* iip, idx nnp, idx* iiu, idx* part)
{
    idx mx = 0;
    for (idx i = 0; i < n; ++i) mx = std::max(mx, dofs[i]);
    for (idx i = 0; i < nnp; ++i) mx = std::max(mx, iip[i]);
    std::vector<char> present(mx + 1, 0), pres(mx + 1, 0);
    for (idx i = 0; i < n; ++i) present[dofs[i]] = 1;
    for (idx i = 0; i < nnp; ++i) pres[iip[i]] = 1;
    idx nnu = 0;
    for (idx j = 0; j <= mx; ++j) {
        if (present[j] && !pres[j]) iiu[nnu++] = j;
    }
    std::vector<idx> renum(mx + 1, 0);
    idx k = 0;
    for (idx i = 0; i < nnu; ++i) renum[iiu[i]] = k++;
    for (idx i = 0; i < nnp; ++i) renum[iip[i]] = k++;
    for (idx i = 0; i < n; ++i) part[i] = renum[dofs[i]];
    return nnu;
}

// Mesh.h:2462-2477 (coordination).
void ref_coordination(const idx* conn, idx nelem, idx nne, idx nnode, idx* N)
{
    for (idx i = 0; i < nnode; ++i) N[i] = 0;
    for (idx i = 0; i < nelem * nne; ++i) N[conn[i]] += 1;
}

// Mesh.h:2485-2513 (elem2node, sorted): CSR (ptr [nnode+1], idx [nelem*nne]).
void ref_elem2node(const idx* conn, idx nelem, idx nne, idx nnode, idx* ptr, idx* out)
{
    std::vector<idx> N(nnode, 0);
    for (idx i = 0; i < nelem * nne; ++i) N[conn[i]] += 1;
    ptr[0] = 0;
    for (idx i = 0; i < nnode; ++i) ptr[i + 1] = ptr[i] + N[i];
    std::vector<idx> cur(ptr, ptr + nnode);
    for (idx e = 0; e < nelem; ++e) {
        for (idx m = 0; m < nne; ++m) out[cur[conn[e * nne + m]]++] = e;
    }
    for (idx i = 0; i < nnode; ++i) std::sort(out + ptr[i], out + ptr[i + 1]);
}

// ------------------------------------------------------------------------------------------------
// Quadrature: shape functions and compute_dN
// ------------------------------------------------------------------------------------------------

// ElementQuad4.h:36-93 (Gauss) and :103-163 (Nodal).
void ref_quad4_gauss(double* xi, double* w)
{
    double g = 1.0 / std::sqrt(3.0);
    const double s[4][2] = {{-1, -1}, {+1, -1}, {+1, +1}, {-1, +1}};
    for (int q = 0; q < 4; ++q) {
        xi[q * 2 + 0] = s[q][0] * g;
        xi[q * 2 + 1] = s[q][1] * g;
        w[q] = 1.0;
    }
}

void ref_quad4_nodal(double* xi, double* w)
{
    const double s[4][2] = {{-1, -1}, {+1, -1}, {+1, +1}, {-1, +1}};
    for (int q = 0; q < 4; ++q) {
        xi[q * 2 + 0] = s[q][0];
        xi[q * 2 + 1] = s[q][1];
        w[q] = 1.0;
    }
}

// ElementHex8.h:26-110 (Gauss) and :116-200 (Nodal).
void ref_hex8_gauss(double* xi, double* w)
{
    double g = 1.0 / std::sqrt(3.0);
    const double s[8][3] = {{-1, -1, -1}, {+1, -1, -1}, {+1, +1, -1}, {-1, +1, -1},
                            {-1, -1, +1}, {+1, -1, +1}, {+1, +1, +1}, {-1, +1, +1}};
    for (int q = 0; q < 8; ++q) {
        for (int d = 0; d < 3; ++d) xi[q * 3 + d] = s[q][d] * g;
        w[q] = 1.0;
    }
}

void ref_hex8_nodal(double* xi, double* w)
{
    const double s[8][3] = {{-1, -1, -1}, {+1, -1, -1}, {+1, +1, -1}, {-1, +1, -1},
                            {-1, -1, +1}, {+1, -1, +1}, {+1, +1, +1}, {-1, +1, +1}};
    for (int q = 0; q < 8; ++q) {
        for (int d = 0; d < 3; ++d) xi[q * 3 + d] = s[q][d];
        w[q] = 1.0;
    }
}

// ElementQuad4.h:277-300: N [nip,4], dNxi [nip,4,2].
void ref_quad4_shape(const double* xi, idx nip, double* N, double* dNxi)
{
    for (idx q = 0; q < nip; ++q) {
        double x0 = xi[q * 2 + 0], x1 = xi[q * 2 + 1];
        N[q * 4 + 0] = 0.25 * (1.0 - x0) * (1.0 - x1);
        N[q * 4 + 1] = 0.25 * (1.0 + x0) * (1.0 - x1);
        N[q * 4 + 2] = 0.25 * (1.0 + x0) * (1.0 + x1);
        N[q * 4 + 3] = 0.25 * (1.0 - x0) * (1.0 + x1);
        double* d = dNxi + q * 8;
        d[0 * 2 + 0] = -0.25 * (1.0 - x1);
        d[1 * 2 + 0] = +0.25 * (1.0 - x1);
        d[2 * 2 + 0] = +0.25 * (1.0 + x1);
        d[3 * 2 + 0] = -0.25 * (1.0 + x1);
        d[0 * 2 + 1] = -0.25 * (1.0 - x0);
        d[1 * 2 + 1] = -0.25 * (1.0 + x0);
        d[2 * 2 + 1] = +0.25 * (1.0 + x0);
        d[3 * 2 + 1] = +0.25 * (1.0 - x0);
    }
}

// ElementHex8.h:255-295: N [nip,8], dNxi [nip,8,3].
void ref_hex8_shape(const double* xi, idx nip, double* N, double* dNxi)
{
    const double sx[8] = {-1, +1, +1, -1, -1, +1, +1, -1};
    const double sy[8] = {-1, -1, +1, +1, -1, -1, +1, +1};
    const double sz[8] = {-1, -1, -1, -1, +1, +1, +1, +1};
    for (idx q = 0; q < nip; ++q) {
        double a = xi[q * 3 + 0], b = xi[q * 3 + 1], c = xi[q * 3 + 2];
        for (int m = 0; m < 8; ++m) {
            // 0.125 * (1 +/- xi0) * (1 +/- xi1) * (1 +/- xi2), evaluated left to right
            double fa = sx[m] < 0 ? (1.0 - a) : (1.0 + a);
            double fb = sy[m] < 0 ? (1.0 - b) : (1.0 + b);
            double fc = sz[m] < 0 ? (1.0 - c) : (1.0 + c);
            N[q * 8 + m] = 0.125 * fa * fb * fc;
            double* d = dNxi + (q * 8 + m) * 3;
            d[0] = (sx[m] < 0 ? -0.125 : +0.125) * fb * fc;
            d[1] = (sy[m] < 0 ? -0.125 : +0.125) * fa * fc;
            d[2] = (sz[m] < 0 ? -0.125 : +0.125) * fa * fb;
        }
    }
}

// ElementQuad4.h:493-532 (compute_dN_impl) with detail.h:26-36 (2x2 inverse).
void ref_quad4_compute_dN(const double* x, idx nelem, const double* xi, const double* w, idx nip,
                          double* dNx, double* vol)
{
    std::vector<double> N(nip * 4), dNxi(nip * 8);
    ref_quad4_shape(xi, nip, N.data(), dNxi.data());
    GF_OMP_FOR
    for (idx e = 0; e < nelem; ++e) {
        const double* xe = x + e * 8;
        for (idx q = 0; q < nip; ++q) {
            const double* dn = dNxi.data() + q * 8;
            double J00 = dn[0] * xe[0] + dn[2] * xe[2] + dn[4] * xe[4] + dn[6] * xe[6];
            double J01 = dn[0] * xe[1] + dn[2] * xe[3] + dn[4] * xe[5] + dn[6] * xe[7];
            double J10 = dn[1] * xe[0] + dn[3] * xe[2] + dn[5] * xe[4] + dn[7] * xe[6];
            double J11 = dn[1] * xe[1] + dn[3] * xe[3] + dn[5] * xe[5] + dn[7] * xe[7];
            double det = J00 * J11 - J01 * J10;
            double i00 = J11 / det;
            double i01 = -1.0 * J01 / det;
            double i10 = -1.0 * J10 / det;
            double i11 = J00 / det;
            double* o = dNx + (e * nip + q) * 8;
            for (int m = 0; m < 4; ++m) {
                o[m * 2 + 0] = i00 * dn[m * 2 + 0] + i01 * dn[m * 2 + 1];
                o[m * 2 + 1] = i10 * dn[m * 2 + 0] + i11 * dn[m * 2 + 1];
            }
            vol[e * nip + q] = w[q] * det;
        }
    }
}

// Element.h:1178-1229 (generic compute_dN_impl, used by Hex8) with detail.h:49-69.
// Restated as written, including the accumulation dNx(m,i) += Jinv(i,j) * dNxi(m,i)
// (index i, not j; Element.h:1220). On axis-aligned elements J is diagonal and the
// result equals the textbook Jinv . dNxi.
void ref_hex8_compute_dN(const double* x, idx nelem, const double* xi, const double* w, idx nip,
                         double* dNx, double* vol)
{
    std::vector<double> N(nip * 8), dNxi(nip * 24);
    ref_hex8_shape(xi, nip, N.data(), dNxi.data());
    GF_OMP_FOR
    for (idx e = 0; e < nelem; ++e) {
        const double* xe = x + e * 24;
        for (idx q = 0; q < nip; ++q) {
            const double* dn = dNxi.data() + q * 24;
            double* o = dNx + (e * nip + q) * 24;
            for (int k = 0; k < 24; ++k) o[k] = 0.0;
            double A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int m = 0; m < 8; ++m)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) A[i][j] += dn[m * 3 + i] * xe[m * 3 + j];
            double det = (A[0][0] * A[1][1] * A[2][2] + A[0][1] * A[1][2] * A[2][0] +
                          A[0][2] * A[1][0] * A[2][1]) -
                         (A[0][2] * A[1][1] * A[2][0] + A[0][1] * A[1][0] * A[2][2] +
                          A[0][0] * A[1][2] * A[2][1]);
            double B[3][3];
            B[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) / det;
            B[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / det;
            B[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / det;
            B[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) / det;
            B[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) / det;
            B[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / det;
            B[2][0] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) / det;
            B[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / det;
            B[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / det;
            for (int m = 0; m < 8; ++m)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) o[m * 3 + i] += B[i][j] * dn[m * 3 + i];
            vol[e * nip + q] = w[q] * det;
        }
    }
}

// ------------------------------------------------------------------------------------------------
// Quadrature operators. nne=4,ndim=2 selects the Quad4 overrides (ElementQuad4.h), nne=8,ndim=3
// the Hex8 path (ElementHex8.h overrides + Element.h generic loops).
// ------------------------------------------------------------------------------------------------

// ElementQuad4.h:325-346 (Quad4) / Element.h:893-922 (generic, Hex8). n = vector length.
void ref_interp_quad_vector(const double* N, const double* elemvec, idx nelem, idx nne, idx nip,
                            idx n, double* qvector)
{
    for (idx i = 0; i < nelem * nip * n; ++i) qvector[i] = 0.0;
    GF_OMP_FOR
    for (idx e = 0; e < nelem; ++e) {
        const double* u = elemvec + e * nne * n;
        for (idx q = 0; q < nip; ++q) {
            const double* Nq = N + q * nne;
            double* tq = qvector + (e * nip + q) * n;
            if (nne == 4 && n == 2) {
                tq[0] = Nq[0] * u[0] + Nq[1] * u[2] + Nq[2] * u[4] + Nq[3] * u[6];
                tq[1] = Nq[0] * u[1] + Nq[1] * u[3] + Nq[2] * u[5] + Nq[3] * u[7];
            }
            else {
                for (idx m = 0; m < nne; ++m)
                    for (idx i = 0; i < n; ++i) tq[i] += Nq[m] * u[m * n + i];
            }
        }
    }
}

// mode 0: gradN_vector (ElementQuad4.h:349-375 / Element.h:925-955)
// mode 1: gradN_vector_T (ElementQuad4.h:378-404 / Element.h:958-988)
// mode 2: symGradN_vector (ElementQuad4.h:407-434 / Element.h:991-1022)
void ref_grad_n_vector(const double* dNx, const double* elemvec, idx nelem, idx nne, idx nip,
                       idx nd, int mode, double* qtensor)
{
    GF_OMP_FOR
    for (idx e = 0; e < nelem; ++e) {
        const double* u = elemvec + e * nne * nd;
        for (idx q = 0; q < nip; ++q) {
            const double* g = dNx + (e * nip + q) * nne * nd;
            double* t = qtensor + (e * nip + q) * nd * nd;
            if (nne == 4 && nd == 2) {
                // hand-unrolled Quad4 overrides
                double g00 = g[0] * u[0] + g[2] * u[2] + g[4] * u[4] + g[6] * u[6];
                double g01 = g[0] * u[1] + g[2] * u[3] + g[4] * u[5] + g[6] * u[7];
                double g10 = g[1] * u[0] + g[3] * u[2] + g[5] * u[4] + g[7] * u[6];
                double g11 = g[1] * u[1] + g[3] * u[3] + g[5] * u[5] + g[7] * u[7];
                if (mode == 0) {
                    t[0] = g00; t[1] = g01; t[2] = g10; t[3] = g11;
                }
                else if (mode == 1) {
                    t[0] = g00; t[2] = g01; t[1] = g10; t[3] = g11;
                }
                else {
                    t[0] = g00;
                    t[3] = g11;
                    t[1] = 0.5 * (g[0] * u[1] + g[2] * u[3] + g[4] * u[5] + g[6] * u[7] +
                                  g[1] * u[0] + g[3] * u[2] + g[5] * u[4] + g[7] * u[6]);
                    t[2] = t[1];
                }
            }
            else {
                for (idx k = 0; k < nd * nd; ++k) t[k] = 0.0;
                for (idx m = 0; m < nne; ++m) {
                    for (idx i = 0; i < nd; ++i) {
                        for (idx j = 0; j < nd; ++j) {
                            if (mode == 0) {
                                t[i * nd + j] += g[m * nd + i] * u[m * nd + j];
                            }
                            else if (mode == 1) {
                                t[j * nd + i] += g[m * nd + i] * u[m * nd + j];
                            }
                            else {
                                t[i * nd + j] += 0.5 * g[m * nd + i] * u[m * nd + j];
                                t[j * nd + i] += 0.5 * g[m * nd + i] * u[m * nd + j];
                            }
                        }
                    }
                }
            }
        }
    }
}

// Element.h:1025-1056 (generic int_N_vector_dV; no Quad4/Hex8 override).
void ref_int_n_vector_dv(const double* N, const double* vol, const double* qvector, idx nelem,
                         idx nne, idx nip, idx n, double* elemvec)
{
    for (idx i = 0; i < nelem * nne * n; ++i) elemvec[i] = 0.0;
    GF_OMP_FOR
    for (idx e = 0; e < nelem; ++e) {
        double* f = elemvec + e * nne * n;
        for (idx q = 0; q < nip; ++q) {
            const double* Ne = N + q * nne;
            const double* tq = qvector + (e * nip + q) * n;
            double volq = vol[e * nip + q];
            for (idx m = 0; m < nne; ++m)
                for (idx i = 0; i < n; ++i) f[m * n + i] += Ne[m] * tq[i] * volq;
        }
    }
}

// ElementQuad4.h:437-464 / ElementHex8.h:324-352 (int_N_scalar_NT_dV): full elemmat.
void ref_int_n_scalar_nt_dv(const double* N, const double* vol, const double* qscalar, idx nelem,
                            idx nne, idx nip, idx nd, double* elemmat)
{
    idx K = nne * nd;
    for (idx i = 0; i < nelem * K * K; ++i) elemmat[i] = 0.0;
    GF_OMP_FOR
    for (idx e = 0; e < nelem; ++e) {
        double* M = elemmat + e * K * K;
        for (idx q = 0; q < nip; ++q) {
            const double* Nq = N + q * nne;
            double v = vol[e * nip + q];
            double rho = qscalar[e * nip + q];
            for (idx m = 0; m < nne; ++m)
                for (idx n = 0; n < nne; ++n)
                    for (idx i = 0; i < nd; ++i)
                        M[(m * nd + i) * K + n * nd + i] += Nq[m] * rho * Nq[n] * v;
        }
    }
}

// ElementQuad4.h:467-491 / ElementHex8.h:355-383 (int_gradN_dot_tensor2_dV).
void ref_int_grad_n_dot_tensor2_dv(const double* dNx, const double* vol, const double* qtensor,
                                   idx nelem, idx nne, idx nip, idx nd, double* elemvec)
{
    for (idx i = 0; i < nelem * nne * nd; ++i) elemvec[i] = 0.0;
    GF_OMP_FOR
    for (idx e = 0; e < nelem; ++e) {
        double* f = elemvec + e * nne * nd;
        for (idx q = 0; q < nip; ++q) {
            const double* g = dNx + (e * nip + q) * nne * nd;
            const double* s = qtensor + (e * nip + q) * nd * nd;
            double v = vol[e * nip + q];
            for (idx m = 0; m < nne; ++m) {
                if (nd == 2) {
                    f[m * 2 + 0] += (g[m * 2 + 0] * s[0] + g[m * 2 + 1] * s[2]) * v;
                    f[m * 2 + 1] += (g[m * 2 + 0] * s[1] + g[m * 2 + 1] * s[3]) * v;
                }
                else {
                    for (idx j = 0; j < 3; ++j)
                        f[m * 3 + j] += (g[m * 3 + 0] * s[0 * 3 + j] + g[m * 3 + 1] * s[1 * 3 + j] +
                                         g[m * 3 + 2] * s[2 * 3 + j]) *
                                        v;
                }
            }
        }
    }
}

// Element.h:1132-1176 (int_gradN_dot_tensor4_dot_gradNT_dV).
void ref_int_grad_n_dot_tensor4_dot_grad_nt_dv(const double* dNx, const double* vol,
                                               const double* qtensor, idx nelem, idx nne, idx nip,
                                               idx nd, double* elemmat)
{
    idx K = nne * nd;
    for (idx i = 0; i < nelem * K * K; ++i) elemmat[i] = 0.0;
    GF_OMP_FOR
    for (idx e = 0; e < nelem; ++e) {
        double* Ke = elemmat + e * K * K;
        for (idx q = 0; q < nip; ++q) {
            const double* g = dNx + (e * nip + q) * nne * nd;
            const double* C = qtensor + (e * nip + q) * nd * nd * nd * nd;
            double v = vol[e * nip + q];
            for (idx m = 0; m < nne; ++m)
                for (idx n = 0; n < nne; ++n)
                    for (idx i = 0; i < nd; ++i)
                        for (idx j = 0; j < nd; ++j)
                            for (idx k = 0; k < nd; ++k)
                                for (idx l = 0; l < nd; ++l)
                                    Ke[(m * nd + j) * K + n * nd + k] +=
                                        g[m * nd + i] * C[((i * nd + j) * nd + k) * nd + l] *
                                        g[n * nd + l] * v;
        }
    }
}

// ------------------------------------------------------------------------------------------------
// Element::Quad4::QuadraturePlanar (ElementQuad4Planar.h): the Quad4 operators with 3x3
// quadrature-point tensors (plane strain) and the out-of-plane thickness in the volume.
// ------------------------------------------------------------------------------------------------

// ElementQuad4Planar.h:81-123 + compute_dN_impl :280-318: the Quad4 Jacobian, inverse and dNx,
// vol = w * det(J) * thick (:315), evaluated left to right.
void ref_quad4_planar_compute_dN(const double* x, idx nelem, const double* xi, const double* w,
                                 idx nip, double thick, double* dNx, double* vol)
{
    ref_quad4_compute_dN(x, nelem, xi, w, nip, dNx, vol);
    for (idx t = 0; t < nelem * nip; ++t) vol[t] = vol[t] * thick;
}

// ElementQuad4Planar.h:130-221 (gradN_vector / gradN_vector_T / symGradN_vector): the output is
// zero-filled [nelem, nip, 3, 3] and only the in-plane 2x2 block is written, with the Quad4
// expressions (mode as in ref_grad_n_vector).
void ref_grad_n_vector_planar(const double* dNx, const double* elemvec, idx nelem, idx nip,
                              int mode, double* qtensor)
{
    std::vector<double> t2(static_cast<size_t>(nelem * nip * 4));
    ref_grad_n_vector(dNx, elemvec, nelem, 4, nip, 2, mode, t2.data());
    for (idx t = 0; t < nelem * nip; ++t) {
        double* o = qtensor + t * 9;
        for (int k = 0; k < 9; ++k) o[k] = 0.0;
        o[0] = t2[t * 4 + 0];
        o[1] = t2[t * 4 + 1];
        o[3] = t2[t * 4 + 2];
        o[4] = t2[t * 4 + 3];
    }
}

// ElementQuad4Planar.h:254-277 (int_gradN_dot_tensor2_dV): reads sig(0,0), sig(1,0), sig(0,1),
// sig(1,1) of each 3x3 tensor, with the Quad4 expression.
void ref_int_grad_n_dot_tensor2_dv_planar(const double* dNx, const double* vol,
                                          const double* qtensor, idx nelem, idx nip,
                                          double* elemvec)
{
    std::vector<double> t2(static_cast<size_t>(nelem * nip * 4));
    for (idx t = 0; t < nelem * nip; ++t) {
        t2[t * 4 + 0] = qtensor[t * 9 + 0];
        t2[t * 4 + 1] = qtensor[t * 9 + 1];
        t2[t * 4 + 2] = qtensor[t * 9 + 3];
        t2[t * 4 + 3] = qtensor[t * 9 + 4];
    }
    ref_int_grad_n_dot_tensor2_dv(dNx, vol, t2.data(), nelem, 4, nip, 2, elemvec);
}

// Element.h:1132-1176 (base int_gradN_dot_tensor4_dot_gradNT_dV) for QuadraturePlanar: the
// tensor is viewed as [3,3,3,3] and i, j, k, l run over the two in-plane indices.
void ref_int_grad_n_dot_tensor4_dot_grad_nt_dv_planar(const double* dNx, const double* vol,
                                                      const double* qtensor, idx nelem, idx nip,
                                                      double* elemmat)
{
    std::vector<double> t2(static_cast<size_t>(nelem * nip * 16));
    for (idx t = 0; t < nelem * nip; ++t)
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k)
                    for (int l = 0; l < 2; ++l)
                        t2[t * 16 + ((i * 2 + j) * 2 + k) * 2 + l] =
                            qtensor[t * 81 + ((i * 3 + j) * 3 + k) * 3 + l];
    ref_int_grad_n_dot_tensor4_dot_grad_nt_dv(dNx, vol, t2.data(), nelem, 4, nip, 2, elemmat);
}

// ------------------------------------------------------------------------------------------------
// Assembled sparse matrices (Matrix.h, MatrixPartitioned.h). Eigen's setFromTriplets sums the
// triplets of one (row, col) in the order they were pushed and stores every row's columns in
// ascending order; restated with an ordered map. The matrix is returned as CSR.
// ------------------------------------------------------------------------------------------------

// Matrix::assemble_impl (Matrix.h:704-733) with dmap = dofs, or MatrixPartitioned::assemble_impl
// (MatrixPartitioned.h:156-200) with dmap = part (the four blocks are the index ranges of the one
// partitioned matrix: the triplet order within each block is the global order). First call with
// rowptr == nullptr returns nnz; the second fills rowptr [n+1], col [nnz], val [nnz].
idx ref_matrix_assemble(const idx* conn, const idx* dmap, idx nelem, idx nne, idx nd, idx n,
                        const double* elemmat, idx* rowptr, idx* col, double* val)
{
    std::map<std::pair<idx, idx>, double> A;
    idx K = nne * nd;
    for (idx e = 0; e < nelem; ++e)
        for (idx m = 0; m < nne; ++m)
            for (idx i = 0; i < nd; ++i)
                for (idx nn = 0; nn < nne; ++nn)
                    for (idx j = 0; j < nd; ++j) {
                        idx r = dmap[conn[e * nne + m] * nd + i];
                        idx c = dmap[conn[e * nne + nn] * nd + j];
                        double v = elemmat[(e * K + m * nd + i) * K + nn * nd + j];
                        auto it = A.find({r, c});
                        if (it == A.end()) A.emplace(std::make_pair(r, c), v);
                        else it->second = it->second + v;
                    }
    if (!rowptr) return static_cast<idx>(A.size());
    for (idx r = 0; r <= n; ++r) rowptr[r] = 0;
    idx k = 0;
    for (auto& kv : A) {
        rowptr[kv.first.first + 1] += 1;
        col[k] = kv.first.second;
        val[k] = kv.second;
        ++k;
    }
    for (idx r = 0; r < n; ++r) rowptr[r + 1] += rowptr[r];
    return k;
}

// Matrix::dot_dofval_impl (Matrix.h:810-815): b = A x with Eigen's column-major product, i.e.
// per row a sum from 0 of A(r,c) x(c) over ascending c.
void ref_matrix_dot(const idx* rowptr, const idx* col, const double* val, idx n, const double* x,
                    double* b)
{
    for (idx r = 0; r < n; ++r) {
        double acc = 0.0;
        for (idx k = rowptr[r]; k < rowptr[r + 1]; ++k) acc = acc + val[k] * x[col[k]];
        b[r] = acc;
    }
}

// MatrixPartitioned::dot_dofval_impl (MatrixPartitioned.h:378-398) on the partitioned CSR
// (rows / columns < nnu: unknown): B = A_.u X_u + A_.p X_p (each product summed from 0, then
// added); x and b dofval in the original numbering, part1d [ndof] the partitioned index of dof d.
void ref_matrixp_dot(const idx* rowptr, const idx* col, const double* val, idx ndof, idx nnu,
                     const idx* part1d, const double* x, double* b)
{
    std::vector<double> xp(ndof), bp(ndof);
    for (idx d = 0; d < ndof; ++d) xp[part1d[d]] = x[d];
    for (idx r = 0; r < ndof; ++r) {
        double su = 0.0, sp = 0.0;
        for (idx k = rowptr[r]; k < rowptr[r + 1]; ++k) {
            if (col[k] < nnu) su = su + val[k] * xp[col[k]];
            else sp = sp + val[k] * xp[col[k]];
        }
        bp[r] = su + sp;
    }
    for (idx d = 0; d < ndof; ++d) b[d] = bp[part1d[d]];
}

// ------------------------------------------------------------------------------------------------
// Periodic tyings (TyingsPeriodic.h, VectorPartitionedTyings.h)
// ------------------------------------------------------------------------------------------------

// TyingsPeriodic.h:85-122: iid = flatten(dofs[dependent]), iii = setdiff1d(dofs, iid),
// iiu = setdiff1d(iii, iip) (sorted unique), renumbering Reorder({iiu, iip, iid}) (Mesh.h:2384-2450)
// applied to dofs and control_dofs. counts = (nnu, nnp, nni, nnd).
void ref_tyings_periodic(const idx* dofs, idx nnode, idx nd, const idx* control, const idx* tyings,
                         idx nties, const idx* iip, idx nnp, idx* dofs_out, idx* control_out,
                         idx* counts)
{
    std::vector<idx> iid;
    for (idx t = 0; t < nties; ++t)
        for (idx j = 0; j < nd; ++j) iid.push_back(dofs[tyings[t * 2 + 1] * nd + j]);
    std::vector<idx> all(dofs, dofs + nnode * nd);
    std::sort(all.begin(), all.end());
    all.erase(std::unique(all.begin(), all.end()), all.end());
    std::vector<idx> sid(iid), sip(iip, iip + nnp);
    std::sort(sid.begin(), sid.end());
    std::sort(sip.begin(), sip.end());
    std::vector<idx> iii, iiu;
    std::set_difference(all.begin(), all.end(), sid.begin(), sid.end(), std::back_inserter(iii));
    std::set_difference(iii.begin(), iii.end(), sip.begin(), sip.end(), std::back_inserter(iiu));
    idx mx = all.empty() ? 0 : all.back();
    std::vector<idx> renum(mx + 1, 0);
    idx i = 0;
    for (idx v : iiu) renum[v] = i++;
    for (idx k = 0; k < nnp; ++k) renum[iip[k]] = i++;
    for (idx v : iid) renum[v] = i++;
    for (idx k = 0; k < nnode * nd; ++k) dofs_out[k] = renum[dofs[k]];
    for (idx k = 0; k < nd * nd; ++k) control_out[k] = renum[control[k]];
    counts[0] = static_cast<idx>(iiu.size());
    counts[1] = nnp;
    counts[2] = static_cast<idx>(iii.size());
    counts[3] = static_cast<idx>(iid.size());
}

// TyingsPeriodic.h:238-264 (Cdi) through setFromTriplets; dense [nnd, nni] output.
void ref_tyings_cdi_dense(const double* coor, const idx* tdofs, const idx* tcontrol,
                          const idx* tyings, idx nties, idx nd, idx nni, double* Cdi)
{
    std::map<std::pair<idx, idx>, double> A;
    auto push = [&](idx r, idx c, double v) {
        auto it = A.find({r, c});
        if (it == A.end()) A.emplace(std::make_pair(r, c), v);
        else it->second = it->second + v;
    };
    for (idx i = 0; i < nties; ++i)
        for (idx j = 0; j < nd; ++j) {
            idx ni = tyings[i * 2], ndn = tyings[i * 2 + 1];
            push(i * nd + j, tdofs[ni * nd + j], +1.0);
            for (idx k = 0; k < nd; ++k)
                push(i * nd + j, tcontrol[j * nd + k], coor[ndn * nd + k] - coor[ni * nd + k]);
        }
    for (idx k = 0; k < nties * nd * nni; ++k) Cdi[k] = 0.0;
    for (auto& kv : A) Cdi[kv.first.first * nni + kv.first.second] = kv.second;
}

// VectorPartitionedTyings.h:208-239 (asDofs_i): the independent entries, then + C_id u_d with
// Eigen's column-major product (per entry i a sum from 0 over ascending d of Cdi(d, i) u_d).
void ref_tyings_as_dofs_i(const idx* tdofs, idx nnode, idx nd, idx nni, idx nnd,
                          const double* Cdi_dense, const double* nodevec, int apply,
                          double* dofval_i)
{
    for (idx i = 0; i < nni; ++i) dofval_i[i] = 0.0;
    std::vector<double> ud(nnd, 0.0);
    for (idx k = 0; k < nnode * nd; ++k) {
        if (tdofs[k] < nni) dofval_i[tdofs[k]] = nodevec[k];
        else ud[tdofs[k] - nni] = nodevec[k];
    }
    if (!apply) return;
    for (idx i = 0; i < nni; ++i) {
        double acc = 0.0;
        for (idx d = 0; d < nnd; ++d) {
            double c = Cdi_dense[d * nni + i];
            if (c != 0.0) acc = acc + c * ud[d];
        }
        dofval_i[i] = dofval_i[i] + acc;
    }
}

// ------------------------------------------------------------------------------------------------
// Vector (Vector.h)
// ------------------------------------------------------------------------------------------------

// Vector.h:681-697 (asElement_impl_nodevec); Element.h:31-52 (asElementVector).
void ref_as_element_nodevec(const idx* conn, idx nelem, idx nne, idx nd, const double* nodevec,
                            double* elemvec)
{
    GF_OMP_FOR
    for (idx e = 0; e < nelem; ++e)
        for (idx m = 0; m < nne; ++m)
            for (idx i = 0; i < nd; ++i)
                elemvec[(e * nne + m) * nd + i] = nodevec[conn[e * nne + m] * nd + i];
}

// Vector.h:659-675 (asElement_impl_dofval).
void ref_as_element_dofval(const idx* conn, const idx* dofs, idx nelem, idx nne, idx nd,
                           const double* dofval, double* elemvec)
{
    GF_OMP_FOR
    for (idx e = 0; e < nelem; ++e)
        for (idx m = 0; m < nne; ++m)
            for (idx i = 0; i < nd; ++i)
                elemvec[(e * nne + m) * nd + i] = dofval[dofs[conn[e * nne + m] * nd + i]];
}

// Vector.h:569-585 (asDofs_impl_nodevec; last writer wins).
void ref_as_dofs_nodevec(const idx* dofs, idx nnode, idx nd, idx ndof, const double* nodevec,
                         double* dofval)
{
    for (idx d = 0; d < ndof; ++d) dofval[d] = 0.0;
    for (idx m = 0; m < nnode; ++m)
        for (idx i = 0; i < nd; ++i) dofval[dofs[m * nd + i]] = nodevec[m * nd + i];
}

// Vector.h:591-608 (asDofs_impl_elemvec; last writer wins).
void ref_as_dofs_elemvec(const idx* conn, const idx* dofs, idx nelem, idx nne, idx nd, idx ndof,
                         const double* elemvec, double* dofval)
{
    for (idx d = 0; d < ndof; ++d) dofval[d] = 0.0;
    for (idx e = 0; e < nelem; ++e)
        for (idx m = 0; m < nne; ++m)
            for (idx i = 0; i < nd; ++i)
                dofval[dofs[conn[e * nne + m] * nd + i]] = elemvec[(e * nne + m) * nd + i];
}

// Vector.h:615-629 (asNode_impl_dofval).
void ref_as_node_dofval(const idx* dofs, idx nnode, idx nd, const double* dofval, double* nodevec)
{
    GF_OMP_FOR
    for (idx m = 0; m < nnode; ++m)
        for (idx i = 0; i < nd; ++i) nodevec[m * nd + i] = dofval[dofs[m * nd + i]];
}

// Vector.h:703-718 (assembleDofs_impl_nodevec, serial).
void ref_assemble_dofs_nodevec(const idx* dofs, idx nnode, idx nd, idx ndof, const double* nodevec,
                               double* dofval)
{
    for (idx d = 0; d < ndof; ++d) dofval[d] = 0.0;
    for (idx m = 0; m < nnode; ++m)
        for (idx i = 0; i < nd; ++i) dofval[dofs[m * nd + i]] += nodevec[m * nd + i];
}

// Vector.h:724-741 (assembleDofs_impl_elemvec, serial, ascending (e, m, i)).
void ref_assemble_dofs_elemvec(const idx* conn, const idx* dofs, idx nelem, idx nne, idx nd,
                               idx ndof, const double* elemvec, double* dofval)
{
    for (idx d = 0; d < ndof; ++d) dofval[d] = 0.0;
    for (idx e = 0; e < nelem; ++e)
        for (idx m = 0; m < nne; ++m)
            for (idx i = 0; i < nd; ++i)
                dofval[dofs[conn[e * nne + m] * nd + i]] += elemvec[(e * nne + m) * nd + i];
}

// Vector.h:747-757 (assembleNode_impl_elemvec = AssembleDofs then asNode).
void ref_assemble_node(const idx* conn, const idx* dofs, idx nelem, idx nne, idx nnode, idx nd,
                       idx ndof, const double* elemvec, double* nodevec)
{
    std::vector<double> dofval(ndof);
    ref_assemble_dofs_elemvec(conn, dofs, nelem, nne, nd, ndof, elemvec, dofval.data());
    ref_as_node_dofval(dofs, nnode, nd, dofval.data(), nodevec);
}

// ------------------------------------------------------------------------------------------------
// MatrixDiagonal (MatrixDiagonal.h) and MatrixDiagonalPartitioned (MatrixDiagonalPartitioned.h)
// ------------------------------------------------------------------------------------------------

// Element.h:122-145 (isDiagonal): |offdiag| > DBL_EPSILON -> not diagonal.
int ref_is_diagonal(const double* elemmat, idx nelem, idx K)
{
    double eps = std::numeric_limits<double>::epsilon();
    for (idx e = 0; e < nelem; ++e)
        for (idx i = 0; i < K; ++i)
            for (idx j = 0; j < K; ++j)
                if (i != j && std::abs(elemmat[(e * K + i) * K + j]) > eps) return 0;
    return 1;
}

// MatrixDiagonal.h:151-167 (assemble_impl, serial diagonal scatter).
void ref_diag_assemble(const idx* conn, const idx* dofs, idx nelem, idx nne, idx nd, idx ndof,
                       const double* elemmat, double* A)
{
    idx K = nne * nd;
    for (idx d = 0; d < ndof; ++d) A[d] = 0.0;
    for (idx e = 0; e < nelem; ++e)
        for (idx m = 0; m < nne; ++m)
            for (idx i = 0; i < nd; ++i)
                A[dofs[conn[e * nne + m] * nd + i]] +=
                    elemmat[(e * K + m * nd + i) * K + m * nd + i];
}

// MatrixDiagonal.h:268-280 (factorize) + :237-250 (solve_nodevec_impl).
void ref_diag_solve_nodevec(const idx* dofs, idx nnode, idx nd, idx ndof, const double* A,
                            const double* b, double* x)
{
    std::vector<double> inv(ndof);
    for (idx d = 0; d < ndof; ++d) inv[d] = 1.0 / A[d];
    for (idx m = 0; m < nnode; ++m)
        for (idx i = 0; i < nd; ++i) x[m * nd + i] = inv[dofs[m * nd + i]] * b[m * nd + i];
}

// MatrixDiagonal.h:213-222 (dot_nodevec_impl).
void ref_diag_dot_nodevec(const idx* dofs, idx nnode, idx nd, const double* A, const double* x,
                          double* b)
{
    for (idx m = 0; m < nnode; ++m)
        for (idx i = 0; i < nd; ++i) b[m * nd + i] = A[dofs[m * nd + i]] * x[m * nd + i];
}

// MatrixDiagonalPartitioned.h:73-98 (assemble_impl into uu / pp).
void ref_diagp_assemble(const idx* conn, const idx* part, idx nelem, idx nne, idx nd, idx nnu,
                        idx nnp, const double* elemmat, double* Auu, double* App)
{
    idx K = nne * nd;
    for (idx d = 0; d < nnu; ++d) Auu[d] = 0.0;
    for (idx d = 0; d < nnp; ++d) App[d] = 0.0;
    for (idx e = 0; e < nelem; ++e)
        for (idx m = 0; m < nne; ++m)
            for (idx i = 0; i < nd; ++i) {
                idx d = part[conn[e * nne + m] * nd + i];
                double v = elemmat[(e * K + m * nd + i) * K + m * nd + i];
                if (d < nnu) Auu[d] += v;
                else App[d - nnu] += v;
            }
}

// MatrixDiagonalPartitioned.h:306-322 (solve_nodevec_impl: unknown DOFs only) + :439-451.
void ref_diagp_solve_nodevec(const idx* part, idx nnode, idx nd, idx nnu, const double* Auu,
                             const double* b, double* x)
{
    std::vector<double> inv(nnu);
    for (idx d = 0; d < nnu; ++d) inv[d] = 1.0 / Auu[d];
    for (idx m = 0; m < nnode; ++m)
        for (idx i = 0; i < nd; ++i)
            if (part[m * nd + i] < nnu) x[m * nd + i] = inv[part[m * nd + i]] * b[m * nd + i];
}

// MatrixDiagonalPartitioned.h:378-392 (reaction_nodevec_impl: prescribed DOFs only).
void ref_diagp_reaction_nodevec(const idx* part, idx nnode, idx nd, idx nnu, const double* App,
                                const double* x, double* b)
{
    for (idx m = 0; m < nnode; ++m)
        for (idx i = 0; i < nd; ++i)
            if (part[m * nd + i] >= nnu) b[m * nd + i] = App[part[m * nd + i] - nnu] * x[m * nd + i];
}

// ------------------------------------------------------------------------------------------------
// Linear elasticity (external GMat in the reference; convention of
// docs/theory/examples/cartesian_linear-elasticity.py:146-186: sigma = K tr(eps) I + 2G dev(eps),
// with a 3-d trace; nd=2 is plane strain). K, G per element, broadcast over the Gauss points.
// ------------------------------------------------------------------------------------------------

void ref_elastic_stress(const double* eps, const double* K, const double* G, idx nelem, idx nip,
                        idx nd, double* sig)
{
    GF_OMP_FOR
    for (idx e = 0; e < nelem; ++e) {
        double g2 = 2.0 * G[e];
        for (idx q = 0; q < nip; ++q) {
            const double* s = eps + (e * nip + q) * nd * nd;
            double* o = sig + (e * nip + q) * nd * nd;
            double tr = 0.0;
            for (idx i = 0; i < nd; ++i) tr += s[i * nd + i];
            double Kt = K[e] * tr;
            double m = tr / 3.0;
            for (idx i = 0; i < nd; ++i)
                for (idx j = 0; j < nd; ++j)
                    o[i * nd + j] = (i == j) ? Kt + g2 * (s[i * nd + j] - m) : g2 * s[i * nd + j];
        }
    }
}

// ------------------------------------------------------------------------------------------------
// Explicit velocity-Verlet (docs/examples/dynamics/Elastic-VelocityVerlet/main.cpp:110-157 and
// docs/examples/dynamics_inertia-damping.rst:6-66), with a nodal viscous damping force -eta*v in
// the residual and the lumped solve of MatrixDiagonal(Partitioned) (diagonal inverse per node,
// fixed DOFs left untouched: minv_mask[m*nd+i] == 0 marks a fixed DOF).
// Force chain per increment: asElement -> symGradN_vector -> stress -> int_gradN_dot_tensor2_dV
// -> assembleNode.
// ------------------------------------------------------------------------------------------------

void ref_verlet_run(const idx* conn, const idx* dofs, idx nelem, idx nne, idx nnode, idx nd,
                    idx ndof, const double* dNx, const double* vol, idx nip, const double* K,
                    const double* G, const double* Adiag, const unsigned char* free_mask,
                    const double* fext, double dt, double eta, idx nsteps, double* u, double* v,
                    double* a)
{
    idx nn = nnode * nd;
    std::vector<double> v_n(nn), a_n(nn), fint(nn), fres(nn), ue(nelem * nne * nd),
        fe(nelem * nne * nd), Eps(nelem * nip * nd * nd), Sig(nelem * nip * nd * nd), inv(ndof);
    for (idx d = 0; d < ndof; ++d) inv[d] = 1.0 / Adiag[d];
    double c = 0.5 * std::pow(dt, 2.0);
    double h = 0.5 * dt;
    auto solve = [&]() {
        for (idx k = 0; k < nn; ++k)
            if (free_mask[k]) a[k] = inv[dofs[k]] * fres[k];
    };
    auto residual = [&]() {
        for (idx k = 0; k < nn; ++k) fres[k] = ((fext ? fext[k] : 0.0) - fint[k]) - eta * v[k];
    };
    for (idx inc = 0; inc < nsteps; ++inc) {
        for (idx k = 0; k < nn; ++k) {
            v_n[k] = v[k];
            a_n[k] = a[k];
        }
        for (idx k = 0; k < nn; ++k) u[k] = (u[k] + dt * v[k]) + c * a[k];
        ref_as_element_nodevec(conn, nelem, nne, nd, u, ue.data());
        ref_grad_n_vector(dNx, ue.data(), nelem, nne, nip, nd, 2, Eps.data());
        ref_elastic_stress(Eps.data(), K, G, nelem, nip, nd, Sig.data());
        ref_int_grad_n_dot_tensor2_dv(dNx, vol, Sig.data(), nelem, nne, nip, nd, fe.data());
        ref_assemble_node(conn, dofs, nelem, nne, nnode, nd, ndof, fe.data(), fint.data());
        for (idx k = 0; k < nn; ++k) v[k] = v_n[k] + dt * a_n[k];
        residual();
        solve();
        for (idx k = 0; k < nn; ++k) v[k] = v_n[k] + h * (a_n[k] + a[k]);
        residual();
        solve();
        for (idx k = 0; k < nn; ++k) v[k] = v_n[k] + h * (a_n[k] + a[k]);
        residual();
        solve();
    }
}

} // extern "C"
