"""Direct-solve oracle of the static linear elastic problem (test infrastructure only).

Restates the assembled partitioned solve of the reference:
 - element stiffness Int_gradN_dot_tensor4_dot_gradNT_dV (Element.h:1132-1176) with the
   isotropic elasticity tensor C4 = K II + 2G I4d (docs/theory/examples/
   cartesian_linear-elasticity.py:146-158), through the C restatement in gfref.cpp;
 - assembly into a sparse matrix (MatrixPartitioned.h:156-200 assembles triplets; duplicates are
   summed) and the partition into unknown (u) and prescribed (p) dofs;
 - MatrixPartitionedSolver::solve (MatrixPartitioned.h:583-613): A_uu x_u = b_u - A_up x_p,
   here with scipy's sparse LU (SuperLU) in place of Eigen's SimplicialLDLT (agreement to
   solver accuracy, not bitwise).
"""

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import gfref as R


def elasticity_tensor(K, G, nip, nd):
    """C4 [nelem, nip, nd, nd, nd, nd] = K II + 2G (I4s - II/3) (3-d identity tensors; for
    nd = 2 the in-plane block, i.e. plane strain)."""
    i = np.eye(3)
    II = np.einsum("ij,kl->ijkl", i, i)
    I4s = 0.5 * (np.einsum("il,jk->ijkl", i, i) + np.einsum("ik,jl->ijkl", i, i))
    I4d = I4s - II / 3.0
    C = K[:, None, None, None, None] * II + 2.0 * G[:, None, None, None, None] * I4d
    C = C[:, :nd, :nd, :nd, :nd]
    return np.ascontiguousarray(np.broadcast_to(C[:, None], (K.size, nip) + (nd,) * 4))


def stiffness(coor, conn, K, G):
    """Assembled stiffness (scipy CSR, full dof numbering = arange(nnode*ndim))."""
    nd = coor.shape[1]
    xi, w = R.quad4_gauss() if nd == 2 else R.hex8_gauss()
    dNx, vol = R.compute_dN(R.as_element(conn, coor), xi, w)
    Ke = R.int_grad_n_dot_tensor4_dot_grad_nt_dv(dNx, vol, elasticity_tensor(K, G, w.size, nd))
    nne = conn.shape[1]
    edofs = (conn[:, :, None] * nd + np.arange(nd)[None, None, :]).reshape(conn.shape[0], nne * nd)
    rows = np.repeat(edofs, nne * nd, axis=1).ravel()
    cols = np.tile(edofs, (1, nne * nd)).ravel()
    n = coor.shape[0] * nd
    return sp.coo_matrix((Ke.ravel(), (rows, cols)), shape=(n, n)).tocsr()


def solve_partitioned(A, iip, x_p):
    """x (full dofval) with x[iip] = x_p and A_uu x_u = -A_up x_p."""
    n = A.shape[0]
    mask = np.zeros(n, dtype=bool)
    mask[iip] = True
    iiu = np.flatnonzero(~mask)
    x = np.zeros(n)
    x[iip] = x_p
    Auu = A[iiu][:, iiu].tocsc()
    Aup = A[iiu][:, iip]
    b = -(Aup @ x_p)
    x[iiu] = spla.spsolve(Auu, b)
    return x


def residual(A, iip, x):
    """||b_u - A_uu x_u|| / ||b_u|| for a full dofval x (prescribed entries included)."""
    n = A.shape[0]
    mask = np.zeros(n, dtype=bool)
    mask[iip] = True
    iiu = np.flatnonzero(~mask)
    xp = np.zeros(n)
    xp[iip] = x[iip]
    b = -(A @ xp)[iiu]
    r = b - (A[iiu][:, iiu] @ x[iiu])
    return float(np.linalg.norm(r) / np.linalg.norm(b))


def solve_tyings(A, tdofs, nnu, nnp, Cdi, b, x):
    """MatrixPartitionedTyingsSolver::solve nodevec (MatrixPartitionedTyings.h, solve_nodevec_impl
    and factorize): the condensed system AC_uu x_u = B_u + C_ud B_d - AC_up x_p with
    AC = A_uu + A_ud C_du + C_ud A_du + C_ud A_dd C_du, solved directly (scipy SuperLU in place of
    Eigen's SimplicialLDLT); x_d = C_du x_u + C_dp x_p. A: assembled [ndof, ndof] matrix in the
    tyings numbering; b, x nodevec; returns the new x."""
    A = sp.csr_matrix(A)
    nni = nnu + nnp
    ndof = A.shape[0]
    Cdu = sp.csr_matrix(Cdi[:, :nnu])
    Cdp = sp.csr_matrix(Cdi[:, nnu:])
    u, p, d = slice(0, nnu), slice(nnu, nni), slice(nni, ndof)
    ACuu = A[u, u] + A[u, d] @ Cdu + Cdu.T @ A[d, u] + Cdu.T @ A[d, d] @ Cdu
    ACup = A[u, p] + A[u, d] @ Cdp + Cdu.T @ A[d, p] + Cdu.T @ A[d, d] @ Cdp
    td = np.asarray(tdofs).ravel()
    bv, xv = np.asarray(b).ravel(), np.asarray(x, dtype=float).ravel().copy()
    B = np.zeros(ndof)
    X = np.zeros(ndof)
    B[td] = bv
    X[td] = xv
    Bu = B[u] + Cdu.T @ B[d]
    Xu = spla.spsolve(ACuu.tocsc(), Bu - ACup @ X[p])
    Xd = Cdu @ Xu + Cdp @ X[p]
    X[u] = Xu
    X[d] = Xd
    return X[td].reshape(np.asarray(x).shape)
