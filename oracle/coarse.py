"""Two-level coarse space of a Regular Quad4 grid, restated with scipy (test infrastructure only:
the checker of csrc/coarse.cu, never on the product path).

No counterpart in the reference: GooseFEM solves the static system with a direct factorisation
(MatrixPartitionedSolver, MatrixPartitioned.h:471-642). The coarse space is the standard
bilinear one: a hat function per coarse node and component on every hc-th node along each axis
(the last interval may be shorter), restricted to the free dofs; the coarse operator is the
Galerkin product P^T A_uu P.
"""

import numpy as np
import scipy.sparse as sp


def coarse_coords(nel, hc):
    nc = (nel + hc - 1) // hc + 1
    return np.minimum(np.arange(nc) * hc, nel)


def hat_matrix(nel, hc):
    """[nel + 1, nc] 1-d linear interpolation from the coarse coordinates."""
    X = coarse_coords(nel, hc)
    rows, cols, vals = [], [], []
    for i in range(nel + 1):
        j = min(int(np.searchsorted(X, i, side="right")) - 1, X.size - 2)
        t = (i - X[j]) / (X[j + 1] - X[j])
        rows += [i, i]
        cols += [j, j + 1]
        vals += [1.0 - t, t]
    M = sp.csr_matrix((vals, (rows, cols)), shape=(nel + 1, X.size))
    M.eliminate_zeros()
    return M


def prolongation(nx, ny, hc, free):
    """P [(nx+1)(ny+1)*2, ncx*ncy*2] (node-major fine dofs, coarse dof (jy ncx + jx) 2 + c),
    rows of prescribed dofs zero."""
    P = sp.kron(sp.kron(hat_matrix(ny, hc), hat_matrix(nx, hc)), sp.eye(2)).tocsr()
    return sp.diags(np.asarray(free, dtype=float)) @ P


def galerkin(A, P):
    """P^T A P (dense) with A the full stiffness and P masked to the free dofs."""
    return (P.T @ (A @ P)).toarray()
