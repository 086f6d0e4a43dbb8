"""The algebra of the blocked Hessenberg reduction and of Q formed in panels (the FP32 form's
gehrd_panel_kernel and unghr_panel_kernel, wavebit_gb300/csrc/wb_eig.cu), restated in NumPy and
held to the column-at-a-time reflectors the other forms use: the same reflectors, taus and
storage below the subdiagonal, the same Q, and A = Q H Q^H.

Per panel of b columns starting at k, with Q_j = I - V_j T_j V_j^H and Y_j = A V_j T_j (A as at
the panel's start), column c = k + j of Q_j^H A Q_j is b = a_c - Y_j V_j(c, :)^H followed by
b <- b - V_j T_j^H (V_j^H b) below row k; its reflector extends T and Y; after the panel the
columns to its right get A <- Q^H (A - Y V^H). Q is formed last panel first as
Z <- (I - V T V^H) Z on the trailing block.
"""
import numpy as np
import pytest


def _reflector(alpha, xnorm):
    if xnorm == 0 and alpha.imag == 0:
        return 0.0, 0.0, alpha.real
    beta = -np.copysign(np.hypot(abs(alpha), xnorm), alpha.real)
    return (beta - alpha) / beta, 1.0 / (alpha - beta), beta


def _gehrd_columns(A):
    A = A.copy()
    n = A.shape[0]
    taus = np.zeros(n, complex)
    for k in range(n - 2):
        x = A[k + 1:, k]
        tau, scale, beta = _reflector(x[0], np.linalg.norm(x[1:]))
        taus[k] = tau
        if tau == 0:
            continue
        v = np.concatenate([[1.0], x[1:] * scale])
        A[k + 1:, k:] -= np.conj(tau) * np.outer(v, v.conj() @ A[k + 1:, k:])
        A[:, k + 1:] -= tau * np.outer(A[:, k + 1:] @ v, v.conj())
        A[k + 2:, k] = v[1:]
    return A, taus


def _gehrd_panels(A, nb):
    A = A.copy()
    n = A.shape[0]
    taus = np.zeros(n, complex)
    for k in range(0, n - 2, nb):
        b = min(nb, n - 2 - k)
        V = np.zeros((n, b), complex)
        Y = np.zeros((n, b), complex)
        T = np.zeros((b, b), complex)
        for j in range(b):
            c = k + j
            col = A[:, c] - Y[:, :j] @ V[c, :j].conj()
            col[k + 1:] -= V[k + 1:, :j] @ (T[:j, :j].conj().T @ (V[k + 1:, :j].conj().T @ col[k + 1:]))
            x = col[c + 1:]
            tau, scale, beta = _reflector(x[0], np.linalg.norm(x[1:]))
            taus[c] = tau
            v = np.zeros(n, complex)
            if tau != 0:
                v[c + 1] = 1.0
                v[c + 2:] = x[1:] * scale
            A[:c + 1, c] = col[:c + 1]
            A[c + 1:, c] = np.concatenate([[beta], v[c + 2:]]) if tau != 0 else x
            V[:, j] = v
            w = V[:, :j].conj().T @ v
            T[:j, j] = -tau * (T[:j, :j] @ w)
            T[j, j] = tau
            Y[:, j] = tau * (A[:, c + 1:] @ v[c + 1:] - Y[:, :j] @ w)
        cs = slice(k + b, n)
        A[:, cs] -= Y @ V[cs, :].conj().T
        A[k + 1:, cs] -= V[k + 1:, :] @ (T.conj().T @ (V[k + 1:, :].conj().T @ A[k + 1:, cs]))
    return A, taus


def _q_columns(H, taus):
    n = H.shape[0]
    Z = np.eye(n, dtype=complex)
    for k in range(n - 3, -1, -1):
        if taus[k] == 0:
            continue
        v = np.concatenate([[1.0], H[k + 2:, k]])
        Z[k + 1:, k + 1:] -= taus[k] * np.outer(v, v.conj() @ Z[k + 1:, k + 1:])
    return Z


def _q_panels(H, taus, nb):
    n = H.shape[0]
    Z = np.eye(n, dtype=complex)
    nk = n - 2
    for k0 in reversed(range(0, nk, nb)):
        b = min(nb, nk - k0)
        V = np.zeros((n, b), complex)
        T = np.zeros((b, b), complex)
        for j in range(b):
            c = k0 + j
            if taus[c] != 0:
                V[c + 1, j] = 1.0
                V[c + 2:, j] = H[c + 2:, c]
        for j in range(b):
            T[:j, j] = -taus[k0 + j] * (T[:j, :j] @ (V[:, :j].conj().T @ V[:, j]))
            T[j, j] = taus[k0 + j]
        blk = slice(k0 + 1, n)
        Z[blk, blk] -= V[blk, :] @ (T @ (V[blk, :].conj().T @ Z[blk, blk]))
    return Z


@pytest.mark.parametrize('n,nb', [(7, 2), (33, 8), (70, 32), (97, 32), (64, 5)])
def test_panels_give_the_column_at_a_time_reflectors_and_q(n, nb):
    rng = np.random.default_rng(n * 100 + nb)
    M = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    H1, t1 = _gehrd_columns(M)
    H2, t2 = _gehrd_panels(M, nb)
    scale = np.abs(H1).max()
    assert np.abs(H1 - H2).max() <= 1e-13 * scale
    assert np.abs(t1 - t2).max() <= 1e-12
    Z1 = _q_columns(H1, t1)
    Z2 = _q_panels(H2, t2, nb)
    assert np.abs(Z1 - Z2).max() <= 1e-13
    Hh = np.triu(H2, -1)
    assert np.abs(Z2 @ Hh @ Z2.conj().T - M).max() <= 1e-12 * np.abs(M).max()
    assert np.abs(Z2.conj().T @ Z2 - np.eye(n)).max() <= 1e-13


def test_a_column_already_reduced_gives_the_identity_reflector():
    """A column with nothing below its subdiagonal keeps tau = 0 and its storage, in panels too."""
    rng = np.random.default_rng(3)
    n = 12
    M = rng.standard_normal((n, n)) + 0j
    M[2:, 0] = 0.0
    M[1, 0] = 2.0
    H1, t1 = _gehrd_columns(M)
    H2, t2 = _gehrd_panels(M, 4)
    assert t1[0] == 0 and t2[0] == 0
    assert np.abs(H1 - H2).max() <= 1e-13 * np.abs(H1).max()
    assert np.abs(_q_columns(H1, t1) - _q_panels(H2, t2, 4)).max() <= 1e-13
