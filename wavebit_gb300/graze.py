"""The grazing-cluster rebuild of a 2D layer's modes, the reference's correct-or-loud contract at
an order sitting on a layer's light line (rcwa/_engine/solve_2d.py:118-222 and :2463-2488).

At such a condition some eigenvalues of the layer operator ``Omega^2 = Omega_L Omega_R`` are
zero to round-off (``min|w| < 1e-9 max|w|``, the kernels' ``WB_ST_GRAZING``). Their eigenvectors
are then set by round-off, and no ``V`` makes ``(W_j, V_j, q_j)`` satisfy both first-order
relations ``Omega_R W = V q`` and ``Omega_L V = W q``. The invariant subspace pair is well
determined, though: ``S_E`` (the cluster of ``Omega_L Omega_R``) and ``S_H`` (the cluster of
``Omega_R Omega_L``). The rebuild restricts both factors to those subspaces, takes the
eigenpairs of the small first-order matrix ``[[0, L_r], [R_r, 0]]``, and picks ``k`` of them so
that the E and H parts stay jointly independent (greedy, by residual norm). Each picked pair has
its root chosen by the layer's ``mode_q``, and the H part's sign goes with it.

When the coupled rates split by less than ``1e-10`` of the layer's modal scale, the cluster is
numerically defective: the exponential mode basis does not exist there at working precision,
and the rebuild refuses (``FloatingPointError``), as the reference does. The lifecycle turns the
refusal into ``NumericalError(code='rcwa.singular')`` with the reference's remedy (detune).

This runs on the host over the FP64 modes the kernels computed, only for the solves they flag,
as the reference's own rebuild runs in NumPy whatever the backend (solve_2d.py:156-161). The
solves are then finished on the device by ``wb_smm_solve``.
"""
import numpy as np

_COUPLED_REL = 1e-9          # solve_2d.py:61, the grazing gate
_DEFECTIVE_REL = 1e-10       # solve_2d.py:73, the defective-cluster refusal
_FLAT = 1e-12                # conventions.py:70, the mode_q tie

DEFECTIVE_MESSAGE = (
    'a 2D layer eigenmode pair is numerically defective at a grazing condition (an order sitting on the layer '
    'light line, so its q**2 is 0): the coupled mode rates split by less than 1e-10 of the layer modal scale, and '
    'the exponential mode basis this formulation uses does not exist there at working precision -- the true '
    'limit basis is {1, z}, and any exponential spelling returns quietly wrong efficiencies (measured 1e-4 up to '
    '1e0). Move off the condition: one ULP of wavelength, period or angle is enough, and '
    'rcwa.Numerics(detuning=...) makes that retry for a single plane wave; it is off by default (detuning=None).')


def mode_q(w):
    """``q = sqrt(w)`` with ``Re q >= 0``, ties ``Im q <= 0`` (conventions.py:186-249)."""
    v = np.sqrt(np.asarray(w, dtype=np.complex128))
    flip = np.where(np.abs(v.real) > _FLAT, v.real < 0, v.imag > 0)
    return np.where(flip, -v, v)


def layer_factors(kx, ky, epx, epy, epz_i):
    """``(Omega_L, Omega_R)`` of a Li layer with ``epxy = epyx = 0`` (solve_2d.py:2377-2418):
    ``Omega_L = [[-Cc, B], [-D, E]]``, ``Omega_R = [[-Kx Ky, Kx^2 - epy], [epx - Ky^2, Ky Kx]]``
    with ``B = Kx epz_i Kx - I``, ``D = Ky epz_i Ky - I``, ``Cc = Kx epz_i Ky``, ``E = Ky epz_i Kx``."""
    kx = np.asarray(kx, dtype=np.complex128)
    ky = np.asarray(ky, dtype=np.complex128)
    N = kx.shape[0]
    eye = np.eye(N, dtype=np.complex128)
    B = (kx[:, None] * epz_i) * kx[None, :] - eye
    D = (ky[:, None] * epz_i) * ky[None, :] - eye
    Cc = (kx[:, None] * epz_i) * ky[None, :]
    Em = (ky[:, None] * epz_i) * kx[None, :]
    omega_l = np.block([[-Cc, B], [-D, Em]])
    omega_r = np.block([[-np.diag(kx * ky), np.diag(kx * kx) - epy], [epx - np.diag(ky * ky), np.diag(ky * kx)]])
    return omega_l, omega_r


def grazing(w):
    """True when ``min|w| < 1e-9 max|w|`` (the gate of solve_2d.py:2463-2464)."""
    aw = np.abs(np.asarray(w))
    return bool(aw.min() < _COUPLED_REL * aw.max())


def rebuild_grazing_cluster(w, W, V, q, omega_l, omega_r):
    """``(W, V, q)`` with the grazing cluster's columns re-derived from the coupled first-order
    problem; ``None`` when the two products' clusters do not have the same size (the structure
    is not understood, and the caller keeps the flag); ``FloatingPointError`` when the cluster
    is numerically defective."""
    w, W, V, q = (np.asarray(a, dtype=np.complex128) for a in (w, W, V, q))
    aw = np.abs(w)
    J = np.where(aw < _COUPLED_REL * aw.max())[0]
    wh, Vh = np.linalg.eig(omega_r @ omega_l)
    Jh = np.where(np.abs(wh) < _COUPLED_REL * np.abs(wh).max())[0]
    if len(Jh) != len(J):
        return None
    k = len(J)
    Q_E = np.linalg.qr(W[:, J])[0]
    Q_H = np.linalg.qr(Vh[:, Jh])[0]
    R_r = Q_H.conj().T @ (omega_r @ Q_E)
    L_r = Q_E.conj().T @ (omega_l @ Q_H)
    Z = np.zeros((k, k), dtype=np.complex128)
    mu_e, g = np.linalg.eig(np.block([[Z, L_r], [R_r, Z]]))
    g = g / np.linalg.norm(g, axis=0, keepdims=True)
    # k of the 2k first-order pairs, keeping the E parts and the H parts jointly independent
    sel = []
    resid_e, resid_h = g[:k, :].copy(), g[k:, :].copy()
    for _ in range(k):
        score = np.linalg.norm(resid_e, axis=0) ** 2 + np.linalg.norm(resid_h, axis=0) ** 2
        score[sel] = -1.0
        pick = int(np.argmax(score))
        sel.append(pick)
        for resid in (resid_e, resid_h):
            col = resid[:, pick]
            nrm = np.linalg.norm(col)
            if nrm > 1e-150:
                d = col / nrm
                resid -= d[:, None] * (d.conj() @ resid)[None, :]
    if np.abs(mu_e[sel]).min() < _DEFECTIVE_REL * np.sqrt(aw.max()):
        raise FloatingPointError(DEFECTIVE_MESSAGE)
    Wc = np.empty((W.shape[0], k), dtype=np.complex128)
    Vc = np.empty_like(Wc)
    qc = np.empty(k, dtype=np.complex128)
    for i, col in enumerate(sel):
        mu_i = mu_e[col]
        q_i = mode_q(np.asarray([mu_i ** 2]))[0]
        g_e, g_h = g[:k, col], g[k:, col]
        if abs(q_i - mu_i) > abs(q_i + mu_i):
            g_h = -g_h                             # the -q member: its H part flips
        Wc[:, i] = Q_E @ g_e
        Vc[:, i] = Q_H @ g_h
        qc[i] = q_i
    W, V, q = W.copy(), V.copy(), q.copy()
    W[:, J], V[:, J], q[J] = Wc, Vc, qc
    return W, V, q
