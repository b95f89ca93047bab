"""Direct-solve fixture of the 3-d static case at 32^3 Hex8 elements.

    python tests/golden/make_static_golden.py   # writes tests/golden/hex8_32_static.npz

Hex8 Regular 32x32x32 (h = 1), K ~ U[0.5,1.5], G ~ U[0.25,0.75] per element (seed below),
z = 0 face fixed in all dofs, z = top face uz = -1e-2 (ux, uy free). Solved with the oracle's
restated partitioned direct solve (oracle/statics.py, scipy SuperLU); the solution is stored as
float64 nodevec so the GPU Jacobi-PCG can be compared without a minutes-long direct solve.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

N = 32
SEED = 3


def case(n=N, seed=SEED):
    from oracle import gfref as R

    coor, conn = R.hex8_regular(n, n, n)
    rng = np.random.default_rng(seed)
    K = rng.uniform(0.5, 1.5, n ** 3)
    G = rng.uniform(0.25, 0.75, n ** 3)
    nxy = (n + 1) ** 2
    front = np.arange(nxy)
    back = front + n * nxy
    iip = np.unique(np.concatenate([(front[:, None] * 3 + np.arange(3)).ravel(), back * 3 + 2]))
    xp = np.where(np.isin(iip, back * 3 + 2), -1e-2, 0.0)
    return coor, conn, K, G, iip, xp


if __name__ == "__main__":
    from oracle import statics as S

    coor, conn, K, G, iip, xp = case()
    A = S.stiffness(coor, conn, K, G)
    x = S.solve_partitioned(A, iip, xp)
    np.savez_compressed(os.path.join(HERE, "hex8_32_static.npz"), x=x.reshape(-1, 3),
                        residual=S.residual(A, iip, x))
