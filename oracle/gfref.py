"""ctypes front-end of the CPU oracle (test infrastructure, not product code).

Thin numpy wrappers around ``oracle/gfref.cpp`` (a restatement of GooseFEM's
element hot path, see that file's header). Only the tests, ``__graft_entry__.smoke``
and ``bench.py``'s CPU-baseline leg use this module, and only as the checker.
"""

import ctypes as C
import os

import numpy as np

from . import build as _build

_LIBS = {}


def lib(parallel=False):
    name = "libgfref_omp.so" if parallel else "libgfref.so"
    if name not in _LIBS:
        path = os.path.join(_build.OUT, name)
        if not os.path.exists(path):
            _build.build()
        L = C.CDLL(path)
        _LIBS[name] = L
    return _LIBS[name]


_i64 = C.c_int64
_dbl = C.c_double


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ix(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def _call(name, *args, parallel=False, restype=None):
    f = getattr(lib(parallel), name)
    f.restype = restype
    conv = []
    for a in args:
        if isinstance(a, np.ndarray) or a is None:
            conv.append(_p(a))
        elif isinstance(a, float):
            conv.append(_dbl(a))
        else:
            conv.append(_i64(int(a)))
    return f(*conv)


# ---------------------------------------------------------------- mesh


def quad4_regular(nx, ny, h=1.0):
    coor = np.empty(((nx + 1) * (ny + 1), 2))
    conn = np.empty((nx * ny, 4), dtype=np.int64)
    _call("ref_quad4_regular", nx, ny, float(h), coor, conn)
    return coor, conn


def hex8_regular(nx, ny, nz, h=1.0):
    coor = np.empty(((nx + 1) * (ny + 1) * (nz + 1), 3))
    conn = np.empty((nx * ny * nz, 8), dtype=np.int64)
    _call("ref_hex8_regular", nx, ny, nz, float(h), coor, conn)
    return coor, conn


def dofs(nnode, ndim):
    return np.arange(nnode * ndim, dtype=np.int64).reshape(nnode, ndim)


def quad4_nodes_periodic(nx, ny):
    out = np.empty(((nx - 1) + (ny - 1) + 3, 2), dtype=np.int64)
    n = _call("ref_quad4_nodes_periodic", nx, ny, out, restype=C.c_int64)
    return out[:n]


def hex8_nodes_periodic(nx, ny, nz):
    n = 7 + 3 * (nx - 1 + ny - 1 + nz - 1) + (nx - 1) * (ny - 1) + (ny - 1) * (nz - 1) \
        + (nx - 1) * (nz - 1)
    out = np.empty((n, 2), dtype=np.int64)
    k = _call("ref_hex8_nodes_periodic", nx, ny, nz, out, restype=C.c_int64)
    assert k == n
    return out


def dofs_periodic(nnode, ndim, nodes_periodic):
    out = np.empty((nnode, ndim), dtype=np.int64)
    npr = _ix(nodes_periodic)
    _call("ref_dofs_periodic", nnode, ndim, npr, npr.shape[0], out)
    return out


def renumber(a):
    a = _ix(a)
    out = np.empty_like(a)
    _call("ref_renumber", a, a.size, out)
    return out


def partition(dofs_, iip):
    d = _ix(dofs_)
    iip = _ix(iip)
    iiu = np.empty(d.size, dtype=np.int64)
    part = np.empty_like(d)
    nnu = _call("ref_partition", d, d.size, iip, iip.size, iiu, part, restype=C.c_int64)
    return iiu[:nnu].copy(), part


def coordination(conn, nnode=None):
    conn = _ix(conn)
    nnode = int(conn.max()) + 1 if nnode is None else nnode
    N = np.empty(nnode, dtype=np.int64)
    _call("ref_coordination", conn, conn.shape[0], conn.shape[1], nnode, N)
    return N


def elem2node(conn, nnode=None):
    conn = _ix(conn)
    nnode = int(conn.max()) + 1 if nnode is None else nnode
    ptr = np.empty(nnode + 1, dtype=np.int64)
    out = np.empty(conn.size, dtype=np.int64)
    _call("ref_elem2node", conn, conn.shape[0], conn.shape[1], nnode, ptr, out)
    return ptr, out


# ---------------------------------------------------------------- quadrature


def quad4_gauss():
    xi, w = np.empty((4, 2)), np.empty(4)
    _call("ref_quad4_gauss", xi, w)
    return xi, w


def quad4_nodal():
    xi, w = np.empty((4, 2)), np.empty(4)
    _call("ref_quad4_nodal", xi, w)
    return xi, w


def hex8_gauss():
    xi, w = np.empty((8, 3)), np.empty(8)
    _call("ref_hex8_gauss", xi, w)
    return xi, w


def hex8_nodal():
    xi, w = np.empty((8, 3)), np.empty(8)
    _call("ref_hex8_nodal", xi, w)
    return xi, w


def shape(xi):
    xi = _f64(xi)
    nip, nd = xi.shape
    nne = 4 if nd == 2 else 8
    N = np.empty((nip, nne))
    dNxi = np.empty((nip, nne, nd))
    _call("ref_quad4_shape" if nd == 2 else "ref_hex8_shape", xi, nip, N, dNxi)
    return N, dNxi


def compute_dN(x, xi, w, parallel=False):
    x, xi, w = _f64(x), _f64(xi), _f64(w)
    nelem, nne, nd = x.shape
    nip = w.size
    dNx = np.empty((nelem, nip, nne, nd))
    vol = np.empty((nelem, nip))
    name = "ref_quad4_compute_dN" if nd == 2 else "ref_hex8_compute_dN"
    _call(name, x, nelem, xi, w, nip, dNx, vol, parallel=parallel)
    return dNx, vol


def interp_quad_vector(N, elemvec):
    N, ev = _f64(N), _f64(elemvec)
    nelem, nne, n = ev.shape
    nip = N.shape[0]
    out = np.empty((nelem, nip, n))
    _call("ref_interp_quad_vector", N, ev, nelem, nne, nip, n, out)
    return out


def _grad(dNx, elemvec, mode, parallel=False):
    dNx, ev = _f64(dNx), _f64(elemvec)
    nelem, nip, nne, nd = dNx.shape
    out = np.empty((nelem, nip, nd, nd))
    _call("ref_grad_n_vector", dNx, ev, nelem, nne, nip, nd, mode, out, parallel=parallel)
    return out


def grad_n_vector(dNx, elemvec):
    return _grad(dNx, elemvec, 0)


def grad_n_vector_T(dNx, elemvec):
    return _grad(dNx, elemvec, 1)


def sym_grad_n_vector(dNx, elemvec, parallel=False):
    return _grad(dNx, elemvec, 2, parallel)


def int_n_vector_dv(N, vol, qvector):
    N, vol, qv = _f64(N), _f64(vol), _f64(qvector)
    nelem, nip, n = qv.shape
    nne = N.shape[1]
    out = np.empty((nelem, nne, n))
    _call("ref_int_n_vector_dv", N, vol, qv, nelem, nne, nip, n, out)
    return out


def int_n_scalar_nt_dv(N, vol, qscalar, nd):
    N, vol, qs = _f64(N), _f64(vol), _f64(qscalar)
    nelem, nip = qs.shape
    nne = N.shape[1]
    out = np.empty((nelem, nne * nd, nne * nd))
    _call("ref_int_n_scalar_nt_dv", N, vol, qs, nelem, nne, nip, nd, out)
    return out


def int_grad_n_dot_tensor2_dv(dNx, vol, qtensor, parallel=False):
    dNx, vol, qt = _f64(dNx), _f64(vol), _f64(qtensor)
    nelem, nip, nne, nd = dNx.shape
    out = np.empty((nelem, nne, nd))
    _call("ref_int_grad_n_dot_tensor2_dv", dNx, vol, qt, nelem, nne, nip, nd, out,
          parallel=parallel)
    return out


def int_grad_n_dot_tensor4_dot_grad_nt_dv(dNx, vol, qtensor):
    dNx, vol, qt = _f64(dNx), _f64(vol), _f64(qtensor)
    nelem, nip, nne, nd = dNx.shape
    out = np.empty((nelem, nne * nd, nne * nd))
    _call("ref_int_grad_n_dot_tensor4_dot_grad_nt_dv", dNx, vol, qt, nelem, nne, nip, nd, out)
    return out


def quad4_planar_compute_dN(x, xi, w, thick=1.0):
    """QuadraturePlanar set-up: dNx [nelem,nip,4,2], vol including the thickness."""
    x, xi, w = _f64(x), _f64(xi), _f64(w)
    nelem, nip = x.shape[0], w.size
    dNx = np.empty((nelem, nip, 4, 2))
    vol = np.empty((nelem, nip))
    _call("ref_quad4_planar_compute_dN", x, nelem, xi, w, nip, float(thick), dNx, vol)
    return dNx, vol


def grad_n_vector_planar(dNx, elemvec, mode):
    """QuadraturePlanar GradN_vector (mode 0), _T (1), SymGradN_vector (2): [nelem,nip,3,3]."""
    dNx, ev = _f64(dNx), _f64(elemvec)
    nelem, nip = dNx.shape[:2]
    out = np.empty((nelem, nip, 3, 3))
    _call("ref_grad_n_vector_planar", dNx, ev, nelem, nip, mode, out)
    return out


def int_grad_n_dot_tensor2_dv_planar(dNx, vol, qtensor):
    dNx, vol, qt = _f64(dNx), _f64(vol), _f64(qtensor)
    nelem, nip = dNx.shape[:2]
    out = np.empty((nelem, 4, 2))
    _call("ref_int_grad_n_dot_tensor2_dv_planar", dNx, vol, qt, nelem, nip, out)
    return out


def int_grad_n_dot_tensor4_dot_grad_nt_dv_planar(dNx, vol, qtensor):
    dNx, vol, qt = _f64(dNx), _f64(vol), _f64(qtensor)
    nelem, nip = dNx.shape[:2]
    out = np.empty((nelem, 8, 8))
    _call("ref_int_grad_n_dot_tensor4_dot_grad_nt_dv_planar", dNx, vol, qt, nelem, nip, out)
    return out


def matrix_assemble(conn, dmap, elemmat, n):
    """Assembled sparse matrix (Eigen setFromTriplets semantics) as CSR (rowptr, col, val);
    dmap: dofs (Matrix) or part (MatrixPartitioned), n: number of rows."""
    conn, dm, em = _ix(conn), _ix(dmap), _f64(elemmat)
    nelem, nne = conn.shape
    nd = dm.shape[1]
    nnz = _call("ref_matrix_assemble", conn, dm, nelem, nne, nd, n, em, None, None, None,
                restype=_i64)
    rowptr = np.empty(n + 1, dtype=np.int64)
    col = np.empty(nnz, dtype=np.int64)
    val = np.empty(nnz)
    _call("ref_matrix_assemble", conn, dm, nelem, nne, nd, n, em, rowptr, col, val, restype=_i64)
    return rowptr, col, val


def matrix_dot(rowptr, col, val, x):
    n = rowptr.size - 1
    b = np.empty(n)
    _call("ref_matrix_dot", _ix(rowptr), _ix(col), _f64(val), n, _f64(x), b)
    return b


def matrixp_dot(rowptr, col, val, nnu, part1d, x):
    ndof = rowptr.size - 1
    b = np.empty(ndof)
    _call("ref_matrixp_dot", _ix(rowptr), _ix(col), _f64(val), ndof, nnu, _ix(part1d), _f64(x), b)
    return b


def tyings_periodic(coor, dofs_, control, tyings, iip):
    """Tyings::Periodic: (renumbered dofs, renumbered control, (nnu, nnp, nni, nnd), Cdi dense)."""
    coor, d, c, t = _f64(coor), _ix(dofs_), _ix(control), _ix(tyings).reshape(-1, 2)
    iip = _ix(iip).ravel()
    nnode, nd = d.shape
    dofs_out = np.empty_like(d)
    ctrl_out = np.empty_like(c)
    counts = np.zeros(4, dtype=np.int64)
    _call("ref_tyings_periodic", d, nnode, nd, c, t, t.shape[0], iip, iip.size, dofs_out, ctrl_out,
          counts)
    nnu, nnp, nni, nnd = (int(v) for v in counts)
    Cdi = np.empty((nnd, nni))
    _call("ref_tyings_cdi_dense", coor, dofs_out, ctrl_out, t, t.shape[0], nd, nni, Cdi)
    return dofs_out, ctrl_out, (nnu, nnp, nni, nnd), Cdi


def tyings_as_dofs_i(tdofs, nni, Cdi, nodevec, apply=True):
    td, nv, Cdi = _ix(tdofs), _f64(nodevec), _f64(Cdi)
    nnode, nd = td.shape
    out = np.empty(nni)
    _call("ref_tyings_as_dofs_i", td, nnode, nd, nni, Cdi.shape[0], Cdi, nv, int(apply), out)
    return out


# ---------------------------------------------------------------- vector


def as_element(conn, nodevec):
    conn, nv = _ix(conn), _f64(nodevec)
    nelem, nne = conn.shape
    nd = nv.shape[1]
    out = np.empty((nelem, nne, nd))
    _call("ref_as_element_nodevec", conn, nelem, nne, nd, nv, out)
    return out


def as_element_dofval(conn, dofs_, dofval):
    conn, d, dv = _ix(conn), _ix(dofs_), _f64(dofval)
    nelem, nne = conn.shape
    nd = d.shape[1]
    out = np.empty((nelem, nne, nd))
    _call("ref_as_element_dofval", conn, d, nelem, nne, nd, dv, out)
    return out


def as_dofs(dofs_, nodevec):
    d, nv = _ix(dofs_), _f64(nodevec)
    ndof = int(d.max()) + 1
    out = np.empty(ndof)
    _call("ref_as_dofs_nodevec", d, d.shape[0], d.shape[1], ndof, nv, out)
    return out


def as_dofs_elemvec(conn, dofs_, elemvec):
    conn, d, ev = _ix(conn), _ix(dofs_), _f64(elemvec)
    ndof = int(d.max()) + 1
    out = np.empty(ndof)
    _call("ref_as_dofs_elemvec", conn, d, conn.shape[0], conn.shape[1], d.shape[1], ndof, ev, out)
    return out


def as_node(dofs_, dofval):
    d, dv = _ix(dofs_), _f64(dofval)
    out = np.empty(d.shape)
    _call("ref_as_node_dofval", d, d.shape[0], d.shape[1], dv, out)
    return out


def assemble_dofs(dofs_, nodevec):
    d, nv = _ix(dofs_), _f64(nodevec)
    ndof = int(d.max()) + 1
    out = np.empty(ndof)
    _call("ref_assemble_dofs_nodevec", d, d.shape[0], d.shape[1], ndof, nv, out)
    return out


def assemble_dofs_elemvec(conn, dofs_, elemvec):
    conn, d, ev = _ix(conn), _ix(dofs_), _f64(elemvec)
    ndof = int(d.max()) + 1
    out = np.empty(ndof)
    _call("ref_assemble_dofs_elemvec", conn, d, conn.shape[0], conn.shape[1], d.shape[1], ndof,
          ev, out)
    return out


def assemble_node(conn, dofs_, elemvec):
    conn, d, ev = _ix(conn), _ix(dofs_), _f64(elemvec)
    ndof = int(d.max()) + 1
    out = np.empty(d.shape)
    _call("ref_assemble_node", conn, d, conn.shape[0], conn.shape[1], d.shape[0], d.shape[1],
          ndof, ev, out)
    return out


# ---------------------------------------------------------------- matrices


def is_diagonal(elemmat):
    em = _f64(elemmat)
    return bool(_call("ref_is_diagonal", em, em.shape[0], em.shape[1], restype=C.c_int))


def diag_assemble(conn, dofs_, elemmat):
    conn, d, em = _ix(conn), _ix(dofs_), _f64(elemmat)
    ndof = int(d.max()) + 1
    A = np.empty(ndof)
    _call("ref_diag_assemble", conn, d, conn.shape[0], conn.shape[1], d.shape[1], ndof, em, A)
    return A


def diag_solve(dofs_, A, b):
    d, A, b = _ix(dofs_), _f64(A), _f64(b)
    x = np.empty_like(b)
    _call("ref_diag_solve_nodevec", d, d.shape[0], d.shape[1], A.size, A, b, x)
    return x


def diag_dot(dofs_, A, x):
    d, A, x = _ix(dofs_), _f64(A), _f64(x)
    b = np.empty_like(x)
    _call("ref_diag_dot_nodevec", d, d.shape[0], d.shape[1], A, x, b)
    return b


def diagp_assemble(conn, part, nnu, nnp, elemmat):
    conn, part, em = _ix(conn), _ix(part), _f64(elemmat)
    Auu, App = np.empty(nnu), np.empty(nnp)
    _call("ref_diagp_assemble", conn, part, conn.shape[0], conn.shape[1], part.shape[1], nnu, nnp,
          em, Auu, App)
    return Auu, App


def diagp_solve(part, nnu, Auu, b, x):
    part, Auu, b = _ix(part), _f64(Auu), _f64(b)
    x = np.array(x, dtype=np.float64, copy=True)
    _call("ref_diagp_solve_nodevec", part, part.shape[0], part.shape[1], nnu, Auu, b, x)
    return x


def diagp_reaction(part, nnu, App, x, b):
    part, App, x = _ix(part), _f64(App), _f64(x)
    b = np.array(b, dtype=np.float64, copy=True)
    _call("ref_diagp_reaction_nodevec", part, part.shape[0], part.shape[1], nnu, App, x, b)
    return b


# ---------------------------------------------------------------- material and dynamics


def elastic_stress(eps, K, G, parallel=False):
    eps, K, G = _f64(eps), _f64(K), _f64(G)
    nelem, nip, nd, _ = eps.shape
    out = np.empty_like(eps)
    _call("ref_elastic_stress", eps, K, G, nelem, nip, nd, out, parallel=parallel)
    return out


def verlet_run(conn, dofs_, dNx, vol, K, G, Adiag, free_mask, fext, dt, eta, nsteps, u, v, a,
               parallel=False):
    """Explicit velocity-Verlet loop; u, v, a are updated in place (numpy float64)."""
    conn, d = _ix(conn), _ix(dofs_)
    dNx, vol, K, G, Adiag = _f64(dNx), _f64(vol), _f64(K), _f64(G), _f64(Adiag)
    fm = np.ascontiguousarray(free_mask, dtype=np.uint8)
    fx = None if fext is None else _f64(fext)
    for arr in (u, v, a):
        assert arr.dtype == np.float64 and arr.flags.c_contiguous
    nelem, nne = conn.shape
    nnode, nd = d.shape
    nip = vol.shape[1]
    _call("ref_verlet_run", conn, d, nelem, nne, nnode, nd, Adiag.size, dNx, vol, nip, K, G, Adiag,
          fm, fx, float(dt), float(eta), nsteps, u, v, a, parallel=parallel)


def num_threads(parallel=True):
    f = lib(parallel).ref_num_threads
    f.restype = C.c_int
    return f()
