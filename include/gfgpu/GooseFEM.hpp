/*
 * GooseFEM-compatible C++ interface of the element hot path, running on the GPU through the
 * C ABI of gfgpu.h (libgfgpu.so). Header-only; needs no CUDA headers.
 *
 * Names and semantics follow GooseFEM (the headers in include/GooseFEM of the reference):
 *   gfgpu::Mesh::Quad4::Regular / Mesh::Hex8::Regular          (MeshQuad4.h, MeshHex8.h)
 *   gfgpu::Vector, gfgpu::VectorPartitioned                    (Vector.h, VectorPartitioned.h)
 *   gfgpu::Element::Quad4::Quadrature / Element::Hex8::Quadrature  (ElementQuad4.h, ElementHex8.h)
 *   gfgpu::MatrixDiagonal, gfgpu::MatrixDiagonalPartitioned   (MatrixDiagonal*.h)
 * Capitalised methods allocate and return, lower-case methods write into a caller-provided
 * array (the reference's convention). Mesh tables are host arrays (gfgpu::host::array); nodal,
 * element and integration-point fields are device arrays (gfgpu::array). Errors throw
 * std::runtime_error with the library's message (GOOSEFEM_ASSERT style).
 */
#ifndef GFGPU_GOOSEFEM_HPP
#define GFGPU_GOOSEFEM_HPP

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../gfgpu.h"

namespace gfgpu {

inline void check(int rc, const char* what)
{
    if (rc != GFGPU_OK)
        throw std::runtime_error(std::string(what) + ": " + gfgpu_last_error());
}

using shape_t = std::vector<int64_t>;

inline int64_t numel(const shape_t& s)
{
    return std::accumulate(s.begin(), s.end(), int64_t(1), std::multiplies<int64_t>());
}

namespace host {

/* Row-major host array (the role of array_type::tensor for mesh tables). */
template <class T>
class array {
public:
    array() = default;
    explicit array(shape_t shape, T val = T()) : m_shape(std::move(shape)), m_data(numel(m_shape), val)
    {
    }
    static array from_shape(shape_t shape) { return array(std::move(shape)); }
    const shape_t& shape() const { return m_shape; }
    int64_t shape(size_t i) const { return m_shape.at(i); }
    size_t dimension() const { return m_shape.size(); }
    int64_t size() const { return static_cast<int64_t>(m_data.size()); }
    T* data() { return m_data.data(); }
    const T* data() const { return m_data.data(); }
    T& operator[](int64_t i) { return m_data[i]; }
    const T& operator[](int64_t i) const { return m_data[i]; }
    T& operator()(int64_t i, int64_t j) { return m_data[i * m_shape[1] + j]; }
    const T& operator()(int64_t i, int64_t j) const { return m_data[i * m_shape[1] + j]; }
    void fill(T v) { std::fill(m_data.begin(), m_data.end(), v); }

private:
    shape_t m_shape;
    std::vector<T> m_data;
};

} // namespace host

/* Owning device array (FP64 fields and int32 tables). Move-only. */
template <class T>
class array {
public:
    array() = default;
    explicit array(shape_t shape) : m_shape(std::move(shape))
    {
        void* p = nullptr;
        check(gfgpu_malloc(&p, numel(m_shape) * sizeof(T)), "gfgpu_malloc");
        m_ptr = static_cast<T*>(p);
    }
    static array from_shape(shape_t shape) { return array(std::move(shape)); }
    static array from_host(const host::array<T>& h)
    {
        array a(h.shape());
        check(gfgpu_memcpy_h2d(a.m_ptr, h.data(), h.size() * sizeof(T)), "gfgpu_memcpy_h2d");
        return a;
    }
    static array from_host(const T* p, shape_t shape)
    {
        array a(std::move(shape));
        check(gfgpu_memcpy_h2d(a.m_ptr, p, a.size() * sizeof(T)), "gfgpu_memcpy_h2d");
        return a;
    }
    host::array<T> to_host() const
    {
        host::array<T> h(m_shape);
        check(gfgpu_memcpy_d2h(h.data(), m_ptr, size() * sizeof(T)), "gfgpu_memcpy_d2h");
        return h;
    }
    array copy() const
    {
        array a(m_shape);
        check(gfgpu_memcpy_d2d(a.m_ptr, m_ptr, size() * sizeof(T)), "gfgpu_memcpy_d2d");
        return a;
    }
    void fill_zero() { check(gfgpu_memset(m_ptr, 0, size() * sizeof(T)), "gfgpu_memset"); }
    ~array() { gfgpu_free(m_ptr); }
    array(const array&) = delete;
    array& operator=(const array&) = delete;
    array(array&& o) noexcept : m_shape(std::move(o.m_shape)), m_ptr(o.m_ptr) { o.m_ptr = nullptr; }
    array& operator=(array&& o) noexcept
    {
        std::swap(m_shape, o.m_shape);
        std::swap(m_ptr, o.m_ptr);
        return *this;
    }
    const shape_t& shape() const { return m_shape; }
    int64_t shape(size_t i) const { return m_shape.at(i); }
    size_t dimension() const { return m_shape.size(); }
    int64_t size() const { return numel(m_shape); }
    T* data() { return m_ptr; }
    const T* data() const { return m_ptr; }

private:
    shape_t m_shape;
    T* m_ptr = nullptr;
};

inline void require_shape(const shape_t& a, const shape_t& b, const char* what)
{
    if (a != b) throw std::runtime_error(std::string(what) + ": shape mismatch");
}

// ------------------------------------------------------------------------------------- Mesh

namespace Mesh {

/* Mesh::dofs (Mesh.h:93-96). */
inline host::array<int32_t> dofs(int64_t nnode, int32_t ndim)
{
    host::array<int32_t> out({nnode, ndim});
    check(gfgpu_host_dofs(nnode, ndim, out.data()), "Mesh::dofs");
    return out;
}

/* Mesh::renumber (Mesh.h:114-175). */
inline host::array<int32_t> renumber(const host::array<int32_t>& in)
{
    host::array<int32_t> out(in.shape());
    check(gfgpu_host_renumber(in.data(), in.size(), out.data()), "Mesh::renumber");
    return out;
}

namespace Quad4 {

/* Mesh::Quad4::Regular (MeshQuad4.h:32-195). */
class Regular {
public:
    Regular(int64_t nelx, int64_t nely, double h = 1.0) : m_nx(nelx), m_ny(nely), m_h(h)
    {
        if (nelx < 1 || nely < 1) throw std::runtime_error("Mesh::Quad4::Regular: nel < 1");
    }
    int64_t nelem() const { return m_nx * m_ny; }
    int64_t nnode() const { return (m_nx + 1) * (m_ny + 1); }
    int32_t nne() const { return 4; }
    int32_t ndim() const { return 2; }
    int64_t nelx() const { return m_nx; }
    int64_t nely() const { return m_ny; }
    double h() const { return m_h; }
    host::array<double> coor() const
    {
        host::array<double> c({nnode(), 2});
        host::array<int32_t> n({nelem(), 4});
        check(gfgpu_host_quad4_regular(m_nx, m_ny, m_h, c.data(), n.data()), "Regular::coor");
        return c;
    }
    host::array<int32_t> conn() const
    {
        host::array<double> c({nnode(), 2});
        host::array<int32_t> n({nelem(), 4});
        check(gfgpu_host_quad4_regular(m_nx, m_ny, m_h, c.data(), n.data()), "Regular::conn");
        return n;
    }
    host::array<int32_t> dofs() const { return Mesh::dofs(nnode(), 2); }
    host::array<int32_t> nodesBottomEdge() const { return range(0, m_nx + 1, 1); }
    host::array<int32_t> nodesTopEdge() const
    {
        return range(m_ny * (m_nx + 1), m_ny * (m_nx + 1) + m_nx + 1, 1);
    }
    host::array<int32_t> nodesLeftEdge() const
    {
        return range(0, (m_ny + 1) * (m_nx + 1), m_nx + 1);
    }
    host::array<int32_t> nodesRightEdge() const
    {
        return range(m_nx, (m_ny + 1) * (m_nx + 1), m_nx + 1);
    }
    /* edges without their corners (MeshQuad4.h:148-166) */
    host::array<int32_t> nodesBottomOpenEdge() const { return range(1, m_nx, 1); }
    host::array<int32_t> nodesTopOpenEdge() const
    {
        return range(m_ny * (m_nx + 1) + 1, m_ny * (m_nx + 1) + m_nx, 1);
    }
    host::array<int32_t> nodesLeftOpenEdge() const
    {
        return range(m_nx + 1, m_ny * (m_nx + 1), m_nx + 1);
    }
    host::array<int32_t> nodesRightOpenEdge() const
    {
        return range(2 * m_nx + 1, m_ny * (m_nx + 1), m_nx + 1);
    }
    int64_t nodesBottomLeftCorner() const { return 0; }
    int64_t nodesBottomRightCorner() const { return m_nx; }
    int64_t nodesTopLeftCorner() const { return m_ny * (m_nx + 1); }
    int64_t nodesTopRightCorner() const { return m_ny * (m_nx + 1) + m_nx; }
    int64_t nodesOrigin() const { return 0; }
    host::array<int32_t> nodesPeriodic() const
    {
        host::array<int32_t> out({(m_nx - 1) + (m_ny - 1) + 3, 2});
        int64_t n = 0;
        check(gfgpu_host_quad4_nodes_periodic(m_nx, m_ny, out.data(), &n), "nodesPeriodic");
        return out;
    }
    host::array<int32_t> dofsPeriodic() const
    {
        auto npr = nodesPeriodic();
        host::array<int32_t> out({nnode(), 2});
        check(gfgpu_host_dofs_periodic(nnode(), 2, npr.data(), npr.shape(0), out.data()),
              "dofsPeriodic");
        return out;
    }

private:
    static host::array<int32_t> range(int64_t a, int64_t b, int64_t s)
    {
        host::array<int32_t> r({(b - a + s - 1) / s});
        for (int64_t i = 0; i < r.size(); ++i) r[i] = static_cast<int32_t>(a + i * s);
        return r;
    }
    int64_t m_nx, m_ny;
    double m_h;
};

} // namespace Quad4

namespace Hex8 {

/* Mesh::Hex8::Regular (MeshHex8.h:26-608). */
class Regular {
public:
    Regular(int64_t nelx, int64_t nely, int64_t nelz, double h = 1.0)
        : m_nx(nelx), m_ny(nely), m_nz(nelz), m_h(h)
    {
        if (nelx < 1 || nely < 1 || nelz < 1) throw std::runtime_error("Mesh::Hex8::Regular");
    }
    int64_t nelem() const { return m_nx * m_ny * m_nz; }
    int64_t nnode() const { return (m_nx + 1) * (m_ny + 1) * (m_nz + 1); }
    int32_t nne() const { return 8; }
    int32_t ndim() const { return 3; }
    host::array<double> coor() const { return build().first; }
    host::array<int32_t> conn() const { return build().second; }
    host::array<int32_t> dofs() const { return Mesh::dofs(nnode(), 3); }
    host::array<int32_t> nodesFront() const
    {
        host::array<int32_t> r({(m_nx + 1) * (m_ny + 1)});
        for (int64_t i = 0; i < r.size(); ++i) r[i] = static_cast<int32_t>(i);
        return r;
    }
    host::array<int32_t> nodesBack() const
    {
        host::array<int32_t> r({(m_nx + 1) * (m_ny + 1)});
        for (int64_t i = 0; i < r.size(); ++i) r[i] = static_cast<int32_t>(i + m_nz * r.size());
        return r;
    }
    /* RegularBase3d::nodesPeriodic / dofsPeriodic (Mesh.h:1577-1692, 291-306) */
    host::array<int32_t> nodesPeriodic() const
    {
        int64_t n = 7 + 3 * (m_nx - 1 + m_ny - 1 + m_nz - 1) + (m_nx - 1) * (m_ny - 1) +
                    (m_ny - 1) * (m_nz - 1) + (m_nx - 1) * (m_nz - 1);
        host::array<int32_t> out({n, 2});
        int64_t k = 0;
        check(gfgpu_host_hex8_nodes_periodic(m_nx, m_ny, m_nz, out.data(), &k), "nodesPeriodic");
        return out;
    }
    host::array<int32_t> dofsPeriodic() const
    {
        auto npr = nodesPeriodic();
        host::array<int32_t> out({nnode(), 3});
        check(gfgpu_host_dofs_periodic(nnode(), 3, npr.data(), npr.shape(0), out.data()),
              "dofsPeriodic");
        return out;
    }
    int64_t nodesOrigin() const { return 0; }

private:
    std::pair<host::array<double>, host::array<int32_t>> build() const
    {
        host::array<double> c({nnode(), 3});
        host::array<int32_t> n({nelem(), 8});
        check(gfgpu_host_hex8_regular(m_nx, m_ny, m_nz, m_h, c.data(), n.data()), "Hex8::Regular");
        return {std::move(c), std::move(n)};
    }
    int64_t m_nx, m_ny, m_nz;
    double m_h;
};

} // namespace Hex8

} // namespace Mesh

// ------------------------------------------------------------------------------------- Vector

namespace detail {

struct Csr {
    array<int32_t> ptr, idx, last;
};

inline Csr elemvec_csr(const host::array<int32_t>& conn, const host::array<int32_t>& dofs,
                       int64_t ndof)
{
    host::array<int32_t> p({ndof + 1}), i({conn.size() * dofs.shape(1)});
    check(gfgpu_host_dof_csr(conn.data(), dofs.data(), conn.shape(0), int32_t(conn.shape(1)),
                             dofs.shape(0), int32_t(dofs.shape(1)), ndof, p.data(), i.data()),
          "gfgpu_host_dof_csr");
    Csr c{array<int32_t>::from_host(p), array<int32_t>::from_host(i), array<int32_t>({ndof})};
    check(gfgpu_csr_last(c.ptr.data(), c.idx.data(), ndof, c.last.data(), nullptr), "csr_last");
    return c;
}

inline Csr nodevec_csr(const host::array<int32_t>& dofs, int64_t ndof)
{
    host::array<int32_t> p({ndof + 1}), i({dofs.size()});
    check(gfgpu_host_dof_csr_nodevec(dofs.data(), dofs.shape(0), int32_t(dofs.shape(1)), ndof,
                                     p.data(), i.data()),
          "gfgpu_host_dof_csr_nodevec");
    Csr c{array<int32_t>::from_host(p), array<int32_t>::from_host(i), array<int32_t>({ndof})};
    check(gfgpu_csr_last(c.ptr.data(), c.idx.data(), ndof, c.last.data(), nullptr), "csr_last");
    return c;
}

inline int64_t max_plus_one(const host::array<int32_t>& a)
{
    int64_t m = -1;
    for (int64_t i = 0; i < a.size(); ++i) m = std::max<int64_t>(m, a[i]);
    return m + 1;
}

} // namespace detail

/* Vector(conn, dofs) (Vector.h:23-767). */
class Vector {
public:
    Vector(const host::array<int32_t>& conn, const host::array<int32_t>& dofs)
        : m_conn_h(conn), m_dofs_h(dofs)
    {
        if (conn.dimension() != 2 || dofs.dimension() != 2)
            throw std::runtime_error("Vector: conn and dofs must be 2-d");
        m_nelem = conn.shape(0);
        m_nne = int32_t(conn.shape(1));
        m_nnode = dofs.shape(0);
        m_ndim = int32_t(dofs.shape(1));
        m_ndof = detail::max_plus_one(dofs);
        if (detail::max_plus_one(conn) > m_nnode) throw std::runtime_error("Vector: conn > nnode");
        m_conn = array<int32_t>::from_host(conn);
        m_dofs = array<int32_t>::from_host(dofs);
        m_csr = detail::elemvec_csr(conn, dofs, m_ndof);
        m_csrn = detail::nodevec_csr(dofs, m_ndof);
    }
    int64_t nelem() const { return m_nelem; }
    int32_t nne() const { return m_nne; }
    int64_t nnode() const { return m_nnode; }
    int32_t ndim() const { return m_ndim; }
    int64_t ndof() const { return m_ndof; }
    const host::array<int32_t>& conn() const { return m_conn_h; }
    const host::array<int32_t>& dofs() const { return m_dofs_h; }
    shape_t shape_dofval() const { return {m_ndof}; }
    shape_t shape_nodevec() const { return {m_nnode, m_ndim}; }
    shape_t shape_elemvec() const { return {m_nelem, m_nne, m_ndim}; }
    array<double> allocate_dofval() const { return array<double>(shape_dofval()); }
    array<double> allocate_nodevec() const { return array<double>(shape_nodevec()); }
    array<double> allocate_elemvec() const { return array<double>(shape_elemvec()); }

    /* nodevec or dofval -> elemvec (Vector.h:659-697) */
    void asElement(const array<double>& arg, array<double>& ret) const
    {
        require_shape(ret.shape(), shape_elemvec(), "Vector::asElement");
        if (arg.shape() == shape_nodevec())
            check(gfgpu_as_element(m_conn.data(), m_nelem, m_nne, m_ndim, arg.data(), ret.data(),
                                   nullptr),
                  "Vector::asElement");
        else if (arg.shape() == shape_dofval())
            check(gfgpu_as_element_dofval(m_conn.data(), m_dofs.data(), m_nelem, m_nne, m_ndim,
                                          arg.data(), ret.data(), nullptr),
                  "Vector::asElement");
        else
            throw std::runtime_error("Vector::asElement unknown dimension for conversion");
    }
    array<double> AsElement(const array<double>& arg) const
    {
        auto r = allocate_elemvec();
        asElement(arg, r);
        return r;
    }
    /* dofval -> nodevec (Vector.h:615-629) */
    void asNode(const array<double>& arg, array<double>& ret) const
    {
        require_shape(arg.shape(), shape_dofval(), "Vector::asNode");
        require_shape(ret.shape(), shape_nodevec(), "Vector::asNode");
        check(gfgpu_as_node(m_dofs.data(), m_nnode, m_ndim, arg.data(), ret.data(), nullptr),
              "Vector::asNode");
    }
    array<double> AsNode(const array<double>& arg) const
    {
        auto r = allocate_nodevec();
        asNode(arg, r);
        return r;
    }
    /* nodevec or elemvec -> dofval, last writer wins (Vector.h:569-608) */
    void asDofs(const array<double>& arg, array<double>& ret) const
    {
        require_shape(ret.shape(), shape_dofval(), "Vector::asDofs");
        const auto& last = arg.shape() == shape_nodevec() ? m_csrn.last : m_csr.last;
        check(gfgpu_as_dofs(last.data(), m_ndof, arg.data(), ret.data(), nullptr), "Vector::asDofs");
    }
    array<double> AsDofs(const array<double>& arg) const
    {
        auto r = allocate_dofval();
        asDofs(arg, r);
        return r;
    }
    /* nodevec or elemvec -> dofval, summed in the reference's order (Vector.h:703-741) */
    void assembleDofs(const array<double>& arg, array<double>& ret) const
    {
        require_shape(ret.shape(), shape_dofval(), "Vector::assembleDofs");
        const auto& c = arg.shape() == shape_nodevec() ? m_csrn : m_csr;
        check(gfgpu_assemble_dofs(c.ptr.data(), c.idx.data(), m_ndof, arg.data(), ret.data(), nullptr),
              "Vector::assembleDofs");
    }
    array<double> AssembleDofs(const array<double>& arg) const
    {
        auto r = allocate_dofval();
        assembleDofs(arg, r);
        return r;
    }
    /* elemvec -> nodevec (Vector.h:747-757) */
    void assembleNode(const array<double>& arg, array<double>& ret) const
    {
        require_shape(arg.shape(), shape_elemvec(), "Vector::assembleNode");
        require_shape(ret.shape(), shape_nodevec(), "Vector::assembleNode");
        check(gfgpu_assemble_node(m_csr.ptr.data(), m_csr.idx.data(), m_dofs.data(), m_nnode, m_ndim,
                                  arg.data(), ret.data(), nullptr),
              "Vector::assembleNode");
    }
    array<double> AssembleNode(const array<double>& arg) const
    {
        auto r = allocate_nodevec();
        assembleNode(arg, r);
        return r;
    }
    const array<int32_t>& conn_device() const { return m_conn; }
    const array<int32_t>& dofs_device() const { return m_dofs; }
    const detail::Csr& csr() const { return m_csr; }

protected:
    host::array<int32_t> m_conn_h, m_dofs_h;
    int64_t m_nelem, m_nnode, m_ndof;
    int32_t m_nne, m_ndim;
    array<int32_t> m_conn, m_dofs;
    detail::Csr m_csr, m_csrn;
};

/* VectorPartitioned(conn, dofs, iip) (VectorPartitioned.h:45-661): the dofs split into unknown
 * (iiu) and prescribed (iip) parts; part(m, i) is the position of dofs(m, i) in [iiu, iip]. */
class VectorPartitioned : public Vector {
public:
    VectorPartitioned(const host::array<int32_t>& conn, const host::array<int32_t>& dofs,
                      const host::array<int32_t>& iip)
        : Vector(conn, dofs), m_iip_h(iip), m_iiu_h({dofs.size()}), m_part_h(dofs.shape())
    {
        int64_t nnu = 0;
        check(gfgpu_host_partition(dofs.data(), dofs.size(), iip.data(), iip.size(), m_iiu_h.data(),
                                   m_part_h.data(), &nnu),
              "VectorPartitioned");
        m_nnu = nnu;
        m_nnp = iip.size();
        host::array<int32_t> iiu({m_nnu}), dof2part({m_ndof});
        for (int64_t i = 0; i < m_nnu; ++i) {
            iiu[i] = m_iiu_h[i];
            dof2part[m_iiu_h[i]] = int32_t(i);
        }
        for (int64_t i = 0; i < m_nnp; ++i) dof2part[iip[i]] = int32_t(m_nnu + i);
        m_iiu_h = std::move(iiu);
        m_iiu = array<int32_t>::from_host(m_iiu_h);
        m_iip = array<int32_t>::from_host(m_iip_h);
        m_part = array<int32_t>::from_host(m_part_h);
        m_dof2part = array<int32_t>::from_host(dof2part);
    }
    int64_t nnu() const { return m_nnu; }
    int64_t nnp() const { return m_nnp; }
    const host::array<int32_t>& iiu() const { return m_iiu_h; }
    const host::array<int32_t>& iip() const { return m_iip_h; }
    const host::array<int32_t>& part() const { return m_part_h; }
    /* dofs_is_u / dofs_is_p (VectorPartitioned.h:126-161), 1 = true */
    host::array<uint8_t> dofs_is_u() const { return is_part(true); }
    host::array<uint8_t> dofs_is_p() const { return is_part(false); }

    /* copy_u / copy_p (VectorPartitioned.h:176-270): overwrite the unknown (prescribed) dofs of
     * dest from src, in place */
    void copy_u(const array<double>& src, array<double>& dest) const { copy_part(src, dest, 0, m_nnu); }
    void copy_p(const array<double>& src, array<double>& dest) const
    {
        copy_part(src, dest, m_nnu, m_ndof);
    }
    array<double> Copy_u(const array<double>& src, const array<double>& dest) const
    {
        auto r = dest.copy();
        copy_u(src, r);
        return r;
    }
    array<double> Copy_p(const array<double>& src, const array<double>& dest) const
    {
        auto r = dest.copy();
        copy_p(src, r);
        return r;
    }

    /* dofsFromParitioned / nodeFromPartitioned / elementFromPartitioned
     * (VectorPartitioned.h:276-418; the reference's spelling is kept) */
    void dofsFromParitioned(const array<double>& u, const array<double>& p, array<double>& dofval) const
    {
        require_up(u, p, "VectorPartitioned::dofsFromParitioned");
        require_shape(dofval.shape(), shape_dofval(), "VectorPartitioned::dofsFromParitioned");
        check(gfgpu_from_partitioned(m_dof2part.data(), m_ndof, m_nnu, m_nnp, u.data(), p.data(),
                                     dofval.data(), nullptr),
              "VectorPartitioned::dofsFromParitioned");
    }
    array<double> DofsFromParitioned(const array<double>& u, const array<double>& p) const
    {
        auto r = allocate_dofval();
        dofsFromParitioned(u, p, r);
        return r;
    }
    void nodeFromPartitioned(const array<double>& u, const array<double>& p, array<double>& nodevec) const
    {
        require_up(u, p, "VectorPartitioned::nodeFromPartitioned");
        require_shape(nodevec.shape(), shape_nodevec(), "VectorPartitioned::nodeFromPartitioned");
        check(gfgpu_from_partitioned(m_part.data(), m_nnode * m_ndim, m_nnu, m_nnp, u.data(), p.data(),
                                     nodevec.data(), nullptr),
              "VectorPartitioned::nodeFromPartitioned");
    }
    array<double> NodeFromPartitioned(const array<double>& u, const array<double>& p) const
    {
        auto r = allocate_nodevec();
        nodeFromPartitioned(u, p, r);
        return r;
    }
    void elementFromPartitioned(const array<double>& u, const array<double>& p,
                                array<double>& elemvec) const
    {
        require_up(u, p, "VectorPartitioned::elementFromPartitioned");
        require_shape(elemvec.shape(), shape_elemvec(), "VectorPartitioned::elementFromPartitioned");
        check(gfgpu_from_partitioned_elemvec(m_conn.data(), m_part.data(), m_nelem, m_nne, m_ndim, m_nnu,
                                             m_nnp, u.data(), p.data(), elemvec.data(), nullptr),
              "VectorPartitioned::elementFromPartitioned");
    }
    array<double> ElementFromPartitioned(const array<double>& u, const array<double>& p) const
    {
        auto r = allocate_elemvec();
        elementFromPartitioned(u, p, r);
        return r;
    }

    /* asDofs_u / asDofs_p of a dofval, nodevec or elemvec (VectorPartitioned.h:428-660); for a
     * nodevec or elemvec the last writer wins, as in the reference's serial loops */
    void asDofs_u(const array<double>& arg, array<double>& ret) const { as_sub(arg, ret, m_iiu, m_nnu); }
    void asDofs_p(const array<double>& arg, array<double>& ret) const { as_sub(arg, ret, m_iip, m_nnp); }
    array<double> AsDofs_u(const array<double>& arg) const
    {
        array<double> r({m_nnu});
        asDofs_u(arg, r);
        return r;
    }
    array<double> AsDofs_p(const array<double>& arg) const
    {
        array<double> r({m_nnp});
        asDofs_p(arg, r);
        return r;
    }
    const array<int32_t>& part_device() const { return m_part; }

private:
    host::array<uint8_t> is_part(bool u) const
    {
        host::array<uint8_t> r(m_part_h.shape());
        for (int64_t i = 0; i < r.size(); ++i) r[i] = uint8_t((m_part_h[i] < m_nnu) == u);
        return r;
    }
    void copy_part(const array<double>& src, array<double>& dest, int64_t lo, int64_t hi) const
    {
        require_shape(src.shape(), shape_nodevec(), "VectorPartitioned::copy");
        require_shape(dest.shape(), shape_nodevec(), "VectorPartitioned::copy");
        check(gfgpu_copy_partitioned_nodevec(m_part.data(), m_nnode, m_ndim, lo, hi, src.data(),
                                             dest.data(), nullptr),
              "VectorPartitioned::copy");
    }
    void require_up(const array<double>& u, const array<double>& p, const char* what) const
    {
        require_shape(u.shape(), {m_nnu}, what);
        require_shape(p.shape(), {m_nnp}, what);
    }
    void as_sub(const array<double>& arg, array<double>& ret, const array<int32_t>& sel, int64_t n) const
    {
        require_shape(ret.shape(), {n}, "VectorPartitioned::asDofs_u/p");
        if (arg.shape() == shape_dofval()) {
            check(gfgpu_from_partitioned(sel.data(), n, m_ndof, 0, arg.data(), nullptr, ret.data(),
                                         nullptr),
                  "VectorPartitioned::asDofs_u/p");
            return;
        }
        array<double> d = AsDofs(arg);
        check(gfgpu_from_partitioned(sel.data(), n, m_ndof, 0, d.data(), nullptr, ret.data(), nullptr),
              "VectorPartitioned::asDofs_u/p");
    }
    int64_t m_nnu = 0, m_nnp = 0;
    host::array<int32_t> m_iip_h, m_iiu_h, m_part_h;
    array<int32_t> m_iiu, m_iip, m_part, m_dof2part;
};

// ------------------------------------------------------------------------------------- Element

namespace Element {

namespace detail {

template <int NNE, int ND>
class Quadrature {
public:
    Quadrature(const array<double>& x, const host::array<double>& xi, const host::array<double>& w,
               bool planar = false, double thick = 1.0)
        : m_x(x.copy()), m_xi(array<double>::from_host(xi)), m_w(array<double>::from_host(w)),
          m_planar(planar), m_thick(thick)
    {
        if (x.dimension() != 3 || x.shape(1) != NNE || x.shape(2) != ND)
            throw std::runtime_error("Quadrature: x must be [nelem, nne, ndim]");
        m_nelem = x.shape(0);
        m_nip = int32_t(w.size());
        m_N = array<double>({m_nip, NNE});
        m_dNxi = array<double>({m_nip, NNE, ND});
        m_dNx = array<double>({m_nelem, m_nip, NNE, ND});
        m_vol = array<double>({m_nelem, m_nip});
        compute_dN();
    }
    void update_x(const array<double>& x)
    {
        require_shape(x.shape(), m_x.shape(), "Quadrature::update_x");
        m_x = x.copy();
        compute_dN();
    }
    int64_t nelem() const { return m_nelem; }
    int32_t nne() const { return NNE; }
    int32_t ndim() const { return ND; }
    int32_t tdim() const { return m_planar ? 3 : ND; }
    int32_t nip() const { return m_nip; }
    const array<double>& GradN() const { return m_dNx; }
    const array<double>& dV() const { return m_vol; }
    shape_t shape_elemvec() const { return {m_nelem, NNE, ND}; }
    shape_t shape_elemmat() const { return {m_nelem, NNE * ND, NNE * ND}; }
    shape_t shape_qscalar() const { return {m_nelem, m_nip}; }
    shape_t shape_qtensor2() const { return {m_nelem, m_nip, tdim(), tdim()}; }

    void gradN_vector(const array<double>& ev, array<double>& q) const { grad(0, ev, q); }
    array<double> GradN_vector(const array<double>& ev) const { return alloc2(0, ev); }
    void gradN_vector_T(const array<double>& ev, array<double>& q) const { grad(1, ev, q); }
    array<double> GradN_vector_T(const array<double>& ev) const { return alloc2(1, ev); }
    void symGradN_vector(const array<double>& ev, array<double>& q) const { grad(2, ev, q); }
    array<double> SymGradN_vector(const array<double>& ev) const { return alloc2(2, ev); }

    void interpQuad_vector(const array<double>& ev, array<double>& qv) const
    {
        int32_t n = int32_t(ev.shape(2));
        check(gfgpu_interp_quad_vector(m_N.data(), ev.data(), m_nelem, NNE, m_nip, n, qv.data(), nullptr),
              "interpQuad_vector");
    }
    array<double> InterpQuad_vector(const array<double>& ev) const
    {
        array<double> qv({m_nelem, m_nip, ev.shape(2)});
        interpQuad_vector(ev, qv);
        return qv;
    }
    void int_N_vector_dV(const array<double>& qv, array<double>& ev) const
    {
        int32_t n = int32_t(qv.shape(2));
        check(gfgpu_int_n_vector_dv(m_N.data(), m_vol.data(), qv.data(), m_nelem, NNE, m_nip, n,
                                    ev.data(), nullptr),
              "int_N_vector_dV");
    }
    array<double> Int_N_vector_dV(const array<double>& qv) const
    {
        array<double> ev({m_nelem, NNE, qv.shape(2)});
        int_N_vector_dV(qv, ev);
        return ev;
    }
    void int_N_scalar_NT_dV(const array<double>& qs, array<double>& em) const
    {
        require_shape(qs.shape(), shape_qscalar(), "int_N_scalar_NT_dV");
        require_shape(em.shape(), shape_elemmat(), "int_N_scalar_NT_dV");
        check(gfgpu_int_n_scalar_nt_dv(m_N.data(), m_vol.data(), qs.data(), m_nelem, NNE, m_nip, ND,
                                       em.data(), nullptr),
              "int_N_scalar_NT_dV");
    }
    array<double> Int_N_scalar_NT_dV(const array<double>& qs) const
    {
        array<double> em(shape_elemmat());
        int_N_scalar_NT_dV(qs, em);
        return em;
    }
    void int_gradN_dot_tensor2_dV(const array<double>& qt, array<double>& ev) const
    {
        require_shape(qt.shape(), shape_qtensor2(), "int_gradN_dot_tensor2_dV");
        require_shape(ev.shape(), shape_elemvec(), "int_gradN_dot_tensor2_dV");
        if (m_planar)
            check(gfgpu_int_grad_n_dot_tensor2_dv_planar(m_dNx.data(), m_vol.data(), qt.data(),
                                                         m_nelem, m_nip, ev.data(), nullptr),
                  "int_gradN_dot_tensor2_dV");
        else
            check(gfgpu_int_grad_n_dot_tensor2_dv(m_dNx.data(), m_vol.data(), qt.data(), m_nelem,
                                                  NNE, m_nip, ND, ev.data(), nullptr),
                  "int_gradN_dot_tensor2_dV");
    }
    array<double> Int_gradN_dot_tensor2_dV(const array<double>& qt) const
    {
        array<double> ev(shape_elemvec());
        int_gradN_dot_tensor2_dV(qt, ev);
        return ev;
    }
    void int_gradN_dot_tensor4_dot_gradNT_dV(const array<double>& qt, array<double>& em) const
    {
        require_shape(em.shape(), shape_elemmat(), "int_gradN_dot_tensor4_dot_gradNT_dV");
        int32_t t = tdim();
        require_shape(qt.shape(), {m_nelem, m_nip, t, t, t, t}, "int_gradN_dot_tensor4_dot_gradNT_dV");
        if (m_planar)
            check(gfgpu_int_grad_n_dot_tensor4_dot_grad_nt_dv_planar(
                      m_dNx.data(), m_vol.data(), qt.data(), m_nelem, m_nip, em.data(), nullptr),
                  "int_gradN_dot_tensor4_dot_gradNT_dV");
        else
            check(gfgpu_int_grad_n_dot_tensor4_dot_grad_nt_dv(m_dNx.data(), m_vol.data(), qt.data(),
                                                              m_nelem, NNE, m_nip, ND, em.data(),
                                                              nullptr),
                  "int_gradN_dot_tensor4_dot_gradNT_dV");
    }
    array<double> Int_gradN_dot_tensor4_dot_gradNT_dV(const array<double>& qt) const
    {
        array<double> em(shape_elemmat());
        int_gradN_dot_tensor4_dot_gradNT_dV(qt, em);
        return em;
    }

protected:
    // mode 0: GradN_vector, 1: GradN_vector_T, 2: SymGradN_vector
    void grad(int mode, const array<double>& ev, array<double>& q) const
    {
        require_shape(ev.shape(), shape_elemvec(), "GradN_vector");
        require_shape(q.shape(), shape_qtensor2(), "GradN_vector");
        int rc;
        if (m_planar) {
            auto f = mode == 0 ? gfgpu_grad_n_vector_planar
                               : (mode == 1 ? gfgpu_grad_n_vector_T_planar : gfgpu_sym_grad_n_vector_planar);
            rc = f(m_dNx.data(), ev.data(), m_nelem, m_nip, q.data(), nullptr);
        }
        else {
            auto f = mode == 0 ? gfgpu_grad_n_vector
                               : (mode == 1 ? gfgpu_grad_n_vector_T : gfgpu_sym_grad_n_vector);
            rc = f(m_dNx.data(), ev.data(), m_nelem, NNE, m_nip, ND, q.data(), nullptr);
        }
        check(rc, "GradN_vector");
    }
    array<double> alloc2(int mode, const array<double>& ev) const
    {
        array<double> q(shape_qtensor2());
        grad(mode, ev, q);
        return q;
    }
    void compute_dN()
    {
        int rc;
        if (m_planar)
            rc = gfgpu_quad4_planar_compute_dN(m_x.data(), m_nelem, m_xi.data(), m_w.data(), m_nip,
                                               m_thick, m_N.data(), m_dNxi.data(), m_dNx.data(),
                                               m_vol.data(), nullptr);
        else
            rc = (NNE == 4 ? gfgpu_quad4_compute_dN : gfgpu_hex8_compute_dN)(
                m_x.data(), m_nelem, m_xi.data(), m_w.data(), m_nip, m_N.data(), m_dNxi.data(),
                m_dNx.data(), m_vol.data(), nullptr);
        check(rc, "compute_dN");
    }
    array<double> m_x, m_xi, m_w, m_N, m_dNxi, m_dNx, m_vol;
    int64_t m_nelem;
    int32_t m_nip;
    bool m_planar;
    double m_thick;
};

inline host::array<double> rule(int nip, int nd, double a)
{
    static const int s[8][3] = {{-1, -1, -1}, {+1, -1, -1}, {+1, +1, -1}, {-1, +1, -1},
                                {-1, -1, +1}, {+1, -1, +1}, {+1, +1, +1}, {-1, +1, +1}};
    host::array<double> xi({nip, nd});
    for (int q = 0; q < nip; ++q)
        for (int d = 0; d < nd; ++d) xi(q, d) = s[q][d] * a;
    return xi;
}

} // namespace detail

namespace Quad4 {
namespace Gauss {
inline int64_t nip() { return 4; }
inline host::array<double> xi() { return detail::rule(4, 2, 1.0 / std::sqrt(3.0)); }
inline host::array<double> w() { return host::array<double>({4}, 1.0); }
} // namespace Gauss
namespace Nodal {
inline int64_t nip() { return 4; }
inline host::array<double> xi() { return detail::rule(4, 2, 1.0); }
inline host::array<double> w() { return host::array<double>({4}, 1.0); }
} // namespace Nodal

/* Element::Quad4::Quadrature (ElementQuad4.h:234-549). */
class Quadrature : public detail::Quadrature<4, 2> {
public:
    explicit Quadrature(const array<double>& x) : detail::Quadrature<4, 2>(x, Gauss::xi(), Gauss::w()) {}
    Quadrature(const array<double>& x, const host::array<double>& xi, const host::array<double>& w)
        : detail::Quadrature<4, 2>(x, xi, w)
    {
    }
};

/* Element::Quad4::QuadraturePlanar (ElementQuad4Planar.h:38-335): 3x3 quadrature-point tensors
 * (plane strain), out-of-plane thickness in dV. */
class QuadraturePlanar : public detail::Quadrature<4, 2> {
public:
    explicit QuadraturePlanar(const array<double>& x, double thick = 1.0)
        : detail::Quadrature<4, 2>(x, Gauss::xi(), Gauss::w(), true, thick)
    {
    }
    QuadraturePlanar(const array<double>& x, const host::array<double>& xi,
                     const host::array<double>& w, double thick = 1.0)
        : detail::Quadrature<4, 2>(x, xi, w, true, thick)
    {
    }
};
} // namespace Quad4

namespace Hex8 {
namespace Gauss {
inline int64_t nip() { return 8; }
inline host::array<double> xi() { return detail::rule(8, 3, 1.0 / std::sqrt(3.0)); }
inline host::array<double> w() { return host::array<double>({8}, 1.0); }
} // namespace Gauss
namespace Nodal {
inline int64_t nip() { return 8; }
inline host::array<double> xi() { return detail::rule(8, 3, 1.0); }
inline host::array<double> w() { return host::array<double>({8}, 1.0); }
} // namespace Nodal

/* Element::Hex8::Quadrature (ElementHex8.h:212-400). */
class Quadrature : public detail::Quadrature<8, 3> {
public:
    explicit Quadrature(const array<double>& x) : detail::Quadrature<8, 3>(x, Gauss::xi(), Gauss::w()) {}
    Quadrature(const array<double>& x, const host::array<double>& xi, const host::array<double>& w)
        : detail::Quadrature<8, 3>(x, xi, w)
    {
    }
};
} // namespace Hex8

/* Element::isDiagonal (Element.h:122-145). */
inline bool isDiagonal(const array<double>& elemmat)
{
    int flag = 0;
    check(gfgpu_is_diagonal(elemmat.data(), elemmat.shape(0), int32_t(elemmat.shape(1)), &flag,
                            nullptr),
          "isDiagonal");
    return flag != 0;
}

} // namespace Element

// ------------------------------------------------------------------------------ MatrixDiagonal

/* MatrixDiagonal(conn, dofs) (MatrixDiagonal.h:114-281). */
class MatrixDiagonal {
public:
    MatrixDiagonal(const host::array<int32_t>& conn, const host::array<int32_t>& dofs)
        : m_vec(conn, dofs), m_A({m_vec.ndof()}), m_inv({m_vec.ndof()})
    {
    }
    int64_t ndof() const { return m_vec.ndof(); }
    /* MatrixDiagonal::assemble (MatrixDiagonal.h:151-167) */
    void assemble(const array<double>& elemmat)
    {
        if (!Element::isDiagonal(elemmat)) throw std::runtime_error("MatrixDiagonal: not diagonal");
        check(gfgpu_diag_assemble(m_vec.csr().ptr.data(), m_vec.csr().idx.data(), ndof(), m_vec.nne(),
                                  m_vec.ndim(), elemmat.data(), m_A.data(), nullptr),
              "MatrixDiagonal::assemble");
        m_changed = true;
    }
    void set(const array<double>& A)
    {
        require_shape(A.shape(), {ndof()}, "MatrixDiagonal::set");
        check(gfgpu_memcpy_d2d(m_A.data(), A.data(), ndof() * 8), "MatrixDiagonal::set");
        m_changed = true;
    }
    const array<double>& data() const { return m_A; }
    /* nodevec solve (MatrixDiagonal.h:237-250) */
    void solve(const array<double>& b, array<double>& x)
    {
        factorize();
        check(gfgpu_diag_solve_nodevec(m_vec.dofs_device().data(), m_vec.nnode(), m_vec.ndim(), ndof(),
                                       m_inv.data(), b.data(), x.data(), nullptr),
              "MatrixDiagonal::solve");
    }
    array<double> Solve(const array<double>& b)
    {
        array<double> x(b.shape());
        solve(b, x);
        return x;
    }
    void dot(const array<double>& x, array<double>& b) const
    {
        check(gfgpu_diag_dot_nodevec(m_vec.dofs_device().data(), m_vec.nnode(), m_vec.ndim(),
                                     m_A.data(), x.data(), b.data(), nullptr),
              "MatrixDiagonal::dot");
    }
    array<double> Dot(const array<double>& x) const
    {
        array<double> b(x.shape());
        dot(x, b);
        return b;
    }

private:
    void factorize()
    {
        if (!m_changed) return;
        check(gfgpu_diag_factorize(m_A.data(), ndof(), m_inv.data(), nullptr), "factorize");
        m_changed = false;
    }
    Vector m_vec;
    array<double> m_A, m_inv;
    bool m_changed = true;
};

/* MatrixDiagonalPartitioned(conn, dofs, iip) (MatrixDiagonalPartitioned.h:42-392): the diagonal
 * stored as [A_uu, A_pp] back to back in the partitioned numbering. */
class MatrixDiagonalPartitioned {
public:
    MatrixDiagonalPartitioned(const host::array<int32_t>& conn, const host::array<int32_t>& dofs,
                              const host::array<int32_t>& iip)
        : m_vec(conn, dofs, iip),
          m_csr(detail::elemvec_csr(conn, m_vec.part(), m_vec.ndof())),
          m_A({m_vec.ndof()}),
          m_inv({std::max<int64_t>(m_vec.nnu(), 1)})
    {
    }
    int64_t ndof() const { return m_vec.ndof(); }
    int64_t nnu() const { return m_vec.nnu(); }
    int64_t nnp() const { return m_vec.nnp(); }
    const VectorPartitioned& vector() const { return m_vec; }
    /* MatrixDiagonalPartitioned::assemble (MatrixDiagonalPartitioned.h:73-98) */
    void assemble(const array<double>& elemmat)
    {
        if (!Element::isDiagonal(elemmat))
            throw std::runtime_error("MatrixDiagonalPartitioned: not diagonal");
        check(gfgpu_diag_assemble(m_csr.ptr.data(), m_csr.idx.data(), ndof(), m_vec.nne(), m_vec.ndim(),
                                  elemmat.data(), m_A.data(), nullptr),
              "MatrixDiagonalPartitioned::assemble");
        m_changed = true;
    }
    /* [A_uu, A_pp] back to back */
    const array<double>& data_partitioned() const { return m_A; }
    /* solve nodevec (MatrixDiagonalPartitioned.h:306-322): writes the unknown dofs of x only */
    void solve(const array<double>& b, array<double>& x)
    {
        require_shape(b.shape(), m_vec.shape_nodevec(), "MatrixDiagonalPartitioned::solve");
        require_shape(x.shape(), m_vec.shape_nodevec(), "MatrixDiagonalPartitioned::solve");
        if (m_changed) {
            check(gfgpu_diag_factorize(m_A.data(), nnu(), m_inv.data(), nullptr), "factorize");
            m_changed = false;
        }
        check(gfgpu_diag_solve_nodevec(m_vec.part_device().data(), m_vec.nnode(), m_vec.ndim(), nnu(),
                                       m_inv.data(), b.data(), x.data(), nullptr),
              "MatrixDiagonalPartitioned::solve");
    }
    array<double> Solve(const array<double>& b, const array<double>& x)
    {
        auto r = x.copy();
        solve(b, r);
        return r;
    }
    /* dot nodevec (MatrixDiagonalPartitioned.h:189-205) */
    void dot(const array<double>& x, array<double>& b) const
    {
        require_shape(x.shape(), m_vec.shape_nodevec(), "MatrixDiagonalPartitioned::dot");
        require_shape(b.shape(), m_vec.shape_nodevec(), "MatrixDiagonalPartitioned::dot");
        check(gfgpu_diag_dot_nodevec(m_vec.part_device().data(), m_vec.nnode(), m_vec.ndim(), m_A.data(),
                                     x.data(), b.data(), nullptr),
              "MatrixDiagonalPartitioned::dot");
    }
    array<double> Dot(const array<double>& x) const
    {
        array<double> b(x.shape());
        dot(x, b);
        return b;
    }
    /* reaction nodevec (MatrixDiagonalPartitioned.h:378-392): b_p = A_pp x_p, b_u untouched */
    void reaction(const array<double>& x, array<double>& b) const
    {
        require_shape(x.shape(), m_vec.shape_nodevec(), "MatrixDiagonalPartitioned::reaction");
        require_shape(b.shape(), m_vec.shape_nodevec(), "MatrixDiagonalPartitioned::reaction");
        check(gfgpu_diagp_reaction_nodevec(m_vec.part_device().data(), m_vec.nnode(), m_vec.ndim(), nnu(),
                                           m_A.data() + nnu(), x.data(), b.data(), nullptr),
              "MatrixDiagonalPartitioned::reaction");
    }
    array<double> Reaction(const array<double>& x, const array<double>& b) const
    {
        auto r = b.copy();
        reaction(x, r);
        return r;
    }

private:
    VectorPartitioned m_vec;
    detail::Csr m_csr;
    array<double> m_A, m_inv;
    bool m_changed = true;
};

/* MatrixPartitioned(conn, dofs, iip) (MatrixPartitioned.h:34-460): the assembled sparse matrix
 * as one CSR in the partitioned numbering (unknown dofs first); assemble() sums the element
 * matrices in the reference's triplet order (bit-exact). */
class MatrixPartitioned {
public:
    MatrixPartitioned(const host::array<int32_t>& conn, const host::array<int32_t>& dofs,
                      const host::array<int32_t>& iip)
        : m_vec(conn, dofs)
    {
        int64_t n = dofs.size();
        host::array<int32_t> iiu({n}), part(dofs.shape());
        int64_t nnu = 0;
        check(gfgpu_host_partition(dofs.data(), n, iip.data(), iip.size(), iiu.data(), part.data(), &nnu),
              "MatrixPartitioned");
        m_nnu = nnu;
        m_ndof = m_vec.ndof();
        host::array<int32_t> iperm({m_ndof});
        for (int64_t i = 0; i < nnu; ++i) iperm[i] = iiu[i];
        for (int64_t i = 0; i < iip.size(); ++i) iperm[nnu + i] = iip[i];
        int64_t nelem = conn.shape(0);
        int32_t nne = int32_t(conn.shape(1)), nd = int32_t(dofs.shape(1));
        int64_t K = int64_t(nne) * nd, total = nelem * K * K;
        host::array<int32_t> rowptr({m_ndof + 1}), col({std::max<int64_t>(total, 1)}),
            cptr({total + 1}), cidx({std::max<int64_t>(total, 1)});
        int64_t nnz = 0;
        check(gfgpu_host_matrix_pattern(conn.data(), part.data(), nelem, nne, dofs.shape(0), nd, m_ndof,
                                        rowptr.data(), col.data(), cptr.data(), cidx.data(), &nnz),
              "MatrixPartitioned: pattern");
        m_nnz = nnz;
        m_rowptr = array<int32_t>::from_host(rowptr);
        m_col = array<int32_t>::from_host(col.data(), {std::max<int64_t>(nnz, 1)});
        m_cptr = array<int32_t>::from_host(cptr.data(), {nnz + 1});
        m_cidx = array<int32_t>::from_host(cidx);
        m_val = array<double>({std::max<int64_t>(nnz, 1)});
        m_iperm = array<int32_t>::from_host(iperm);
    }
    int64_t ndof() const { return m_ndof; }
    int64_t nnu() const { return m_nnu; }
    int64_t nnp() const { return m_ndof - m_nnu; }
    int64_t nnz() const { return m_nnz; }
    const Vector& vector() const { return m_vec; }
    /* MatrixPartitioned::assemble (MatrixPartitioned.h:156-200) */
    void assemble(const array<double>& elemmat)
    {
        check(gfgpu_matrix_assemble(m_cptr.data(), m_cidx.data(), m_nnz, elemmat.data(), m_val.data(),
                                    nullptr),
              "MatrixPartitioned::assemble");
    }
    /* dot / Dot on dofval (MatrixPartitioned.h:378-398) or nodevec (:354-376) */
    void dot(const array<double>& x, array<double>& b) const
    {
        if (x.dimension() == 1) {
            check(gfgpu_matrixp_dot_dofval(m_rowptr.data(), m_col.data(), m_val.data(), m_ndof, m_nnu,
                                           m_iperm.data(), x.data(), b.data(), nullptr),
                  "MatrixPartitioned::dot");
            return;
        }
        array<double> xd = m_vec.AsDofs(x), bd({m_ndof});
        dot(xd, bd);
        m_vec.asNode(bd, b);
    }
    array<double> Dot(const array<double>& x) const
    {
        array<double> b(x.shape());
        dot(x, b);
        return b;
    }
    /* Reaction (MatrixPartitioned.h:401-433): copy of b with b_p = A_pu x_u + A_pp x_p */
    array<double> Reaction(const array<double>& x, const array<double>& b) const
    {
        if (x.dimension() == 1) {
            array<double> r = b.copy();
            check(gfgpu_matrixp_reaction_dofval(m_rowptr.data(), m_col.data(), m_val.data(), m_ndof,
                                                m_nnu, m_iperm.data(), x.data(), r.data(), nullptr),
                  "MatrixPartitioned::Reaction");
            return r;
        }
        array<double> xd = m_vec.AsDofs(x), bd = m_vec.AsDofs(b);
        array<double> rd = Reaction(xd, bd);
        return m_vec.AsNode(rd);
    }

private:
    friend class MatrixPartitionedSolver;
    Vector m_vec;
    int64_t m_ndof = 0, m_nnu = 0, m_nnz = 0;
    array<int32_t> m_rowptr, m_col, m_cptr, m_cidx, m_iperm;
    array<double> m_val;
};

/* MatrixPartitionedSolver (MatrixPartitioned.h:471-642): x_u = A_uu^-1 (b_u - A_up x_p). The
 * reference factorises A_uu (Eigen SimplicialLDLT); here a Krylov solve of the assembled A_uu in
 * FP64 to the relative residual tol: MINRES (default, symmetric indefinite allowed;
 * gfgpu_matrixp_solve_minres) or Jacobi-PCG (pcg = true, SPD; gfgpu_matrixp_solve). */
class MatrixPartitionedSolver {
public:
    explicit MatrixPartitionedSolver(double tol = 1e-12, int64_t maxiter = 1000000, bool pcg = false)
        : m_tol(tol), m_maxiter(maxiter), m_pcg(pcg)
    {
    }
    /* solve on dofval or nodevec: x holds x_p (and the initial guess of x_u) */
    void solve(MatrixPartitioned& A, const array<double>& b, array<double>& x)
    {
        if (x.dimension() != 1) {
            array<double> bd = A.m_vec.AsDofs(b), xd = A.m_vec.AsDofs(x);
            solve(A, bd, xd);
            A.m_vec.asNode(xd, x);
            return;
        }
        int64_t nb = m_pcg ? gfgpu_matrixp_solve_workspace_bytes(A.m_nnu)
                           : gfgpu_matrixp_solve_minres_workspace_bytes(A.m_nnu);
        array<double> ws({nb / 8 + 1});
        auto fn = m_pcg ? gfgpu_matrixp_solve : gfgpu_matrixp_solve_minres;
        check(fn(A.m_rowptr.data(), A.m_col.data(), A.m_val.data(), A.m_ndof, A.m_nnu, A.m_iperm.data(),
                 b.data(), x.data(), m_tol, m_maxiter, 16, ws.data(), nullptr, &m_iters, &m_relres),
              "MatrixPartitionedSolver::solve");
    }
    array<double> Solve(MatrixPartitioned& A, const array<double>& b, const array<double>& x)
    {
        array<double> r = x.copy();
        solve(A, b, r);
        return r;
    }
    int64_t iterations() const { return m_iters; }
    double relres() const { return m_relres; }

private:
    double m_tol;
    int64_t m_maxiter;
    bool m_pcg;
    int64_t m_iters = 0;
    double m_relres = 0.0;
};

} // namespace gfgpu

#endif
