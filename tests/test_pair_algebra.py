"""The algebra behind the float-float element kernels, checked in FP64 on the CPU (no GPU): the
restated element stiffness of the general pair path against the oracle's operator chain, its
translation invariance and the node-difference form the kernel evaluates, and the difference form
of the square closed form (A1 = P + Q, A2 = P - Q, A3 = D + E) that the mixed kernel feeds with
FP64 differences."""

import numpy as np


def _element_stiffness(dNx, vol, K, G):
    """K_e[(m,j),(n,l)] = sum_q vol_q (lam dNx(m,j) dNx(n,l) + G (delta_jl dNx(m,.).dNx(n,.) +
    dNx(m,l) dNx(n,j))), the formula of k_pair_stiffness (verlet_pair.cu)."""
    ne = dNx.shape[0]
    Ke = np.zeros((ne, 8, 8))
    lam = K - 2.0 * G / 3.0
    for q in range(dNx.shape[1]):
        g = dNx[:, q]  # [ne, 4, 2]
        v = vol[:, q]
        for m in range(4):
            for n in range(4):
                dd = np.einsum("ek,ek->e", g[:, m], g[:, n])
                for j in range(2):
                    for l in range(2):
                        val = lam * g[:, m, j] * g[:, n, l] + G * ((dd if j == l else 0.0) + g[:, m, l] * g[:, n, j])
                        Ke[:, 2 * m + j, 2 * n + l] += v * val
    return Ke


def test_general_pair_path_algebra(oracle):
    R = oracle
    rng = np.random.default_rng(21)
    coor, conn = R.quad4_regular(9, 7)
    coor = coor + rng.uniform(-0.2, 0.2, coor.shape)  # distorted elements
    ne = conn.shape[0]
    K = rng.uniform(0.5, 1.5, ne)
    G = rng.uniform(0.25, 0.75, ne)
    u = rng.uniform(-1e-3, 1e-3, coor.shape)
    dNx, vol = R.compute_dN(R.as_element(conn, coor), *R.quad4_gauss())
    ue = R.as_element(conn, u)  # [ne, 4, 2]
    # the oracle's chain: symGradN -> stress -> int_gradN_dot_tensor2_dV
    fe_ref = R.int_grad_n_dot_tensor2_dv(dNx, vol, R.elastic_stress(R.sym_grad_n_vector(dNx, ue), K, G))
    Ke = _element_stiffness(dNx, vol, K, G)
    fe_K = np.einsum("eab,eb->ea", Ke, ue.reshape(ne, 8)).reshape(ne, 4, 2)
    scale = np.max(np.abs(fe_ref))
    assert np.max(np.abs(fe_K - fe_ref)) <= 1e-13 * scale
    # symmetric, and no force from a rigid translation: every row sums to zero per direction
    assert np.max(np.abs(Ke - Ke.transpose(0, 2, 1))) <= 1e-15 * np.max(np.abs(Ke))
    rows = Ke.reshape(ne, 8, 4, 2).sum(axis=2)  # sum over n for each (m, j), l
    assert np.max(np.abs(rows)) <= 1e-14 * np.max(np.abs(Ke))
    # the kernel's form: only the off-diagonal node blocks, f_m = sum_{n != m} K_mn (u_n - u_m)
    fe_d = np.zeros_like(fe_K)
    B = Ke.reshape(ne, 4, 2, 4, 2)
    for m in range(4):
        for n in range(4):
            if n != m:
                fe_d[:, m] += np.einsum("ejl,el->ej", B[:, m, :, n, :], ue[:, n] - ue[:, m])
    assert np.max(np.abs(fe_d - fe_ref)) <= 1e-13 * scale


def test_square_closed_form_difference_form():
    """A1 = (u2 - u0) + (u1 - u3), A2 = (u2 - u0) - (u1 - u3), A3 = (u0 - u1) + (u2 - u3) equal the
    node sums of the square closed form; an affine field u = gamma (y, 0) cancels from A1 and A3
    exactly in the difference form."""
    rng = np.random.default_rng(3)
    u = rng.uniform(-1, 1, (1000, 4, 2))
    P, Q = u[:, 2] - u[:, 0], u[:, 1] - u[:, 3]
    D, E = u[:, 0] - u[:, 1], u[:, 2] - u[:, 3]
    A1, A2, A3 = P + Q, P - Q, D + E
    assert np.allclose(A1, (u[:, 1] + u[:, 2]) - (u[:, 0] + u[:, 3]), rtol=0, atol=1e-14)
    assert np.allclose(A2, (u[:, 2] + u[:, 3]) - (u[:, 0] + u[:, 1]), rtol=0, atol=1e-14)
    assert np.allclose(A3, (u[:, 0] + u[:, 2]) - (u[:, 1] + u[:, 3]), rtol=0, atol=1e-14)
    # unit square nodes (0,0), (1,0), (1,1), (0,1) at height y0: u_x = gamma y
    y0, gamma = 311.0, 2e-3
    ux = gamma * (y0 + np.array([0.0, 0.0, 1.0, 1.0]))
    Px, Qx, Dx, Ex = ux[2] - ux[0], ux[1] - ux[3], ux[0] - ux[1], ux[2] - ux[3]
    assert Px + Qx == 0.0 and Dx + Ex == 0.0
