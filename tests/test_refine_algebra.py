"""The algebra the mixed form's kernels implement, restated in NumPy and checked on the CPU.

* The closed-form eigen-decomposition of 2-member groups (group2_apply_kernel, wb_solve.cu).
* The elimination with source terms that solves the stack's interface equations
  (cascade_sources, wb_solve.cu): bottom-up h_l = R_l g_l + s_l, top-down g, c+, c-; the
  residuals of every equation vanish, and one defect correction from a perturbed state lands on
  the solution.
"""
import numpy as np


def _eig2(a, b, c, d):
    """B = [[a, b], [c, d]]: eigenvalues m +- r and eigenvectors (s, c), (b, -s), s = dl + r with
    the sign of r making |s| the larger root difference (as group2_apply_kernel)."""
    m, dl = 0.5 * (a + d), 0.5 * (a - d)
    r = np.sqrt(dl * dl + b * c + 0j)
    if abs(dl + r) < abs(dl - r):
        r = -r
    s = dl + r
    v1 = np.array([s, c]) / np.sqrt(abs(s) ** 2 + abs(c) ** 2)
    v2 = np.array([b, -s]) / np.sqrt(abs(b) ** 2 + abs(s) ** 2)
    return (m + r, m - r), np.stack([v1, v2], axis=1)


def test_closed_form_2x2_groups_are_eigenpairs():
    rng = np.random.default_rng(0)
    for scale in (1.0, 1e-4, 1e-9):                      # generic, near-degenerate, tightly coupled
        for _ in range(200):
            d0 = rng.standard_normal() + 1j * rng.standard_normal()
            B = d0 * np.eye(2) + scale * (rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2)))
            lam, V = _eig2(B[0, 0], B[0, 1], B[1, 0], B[1, 1])
            res = np.abs(B @ V - V * np.array(lam)[None, :]).max()
            assert res <= 1e-13 * max(1.0, np.abs(B).max()), (scale, res)
            assert abs(np.vdot(V[:, 0], V[:, 1])) < 1.0


def _layer(rng, n):
    """A random layer: well-conditioned modes W, V and decaying X."""
    W = np.eye(n) + 0.3 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    V = np.eye(n) * (1.3 - 0.2j) + 0.3 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    X = np.exp(-(0.2 + rng.random(n)) - 1j * rng.random(n))
    return W, V, X


def _solve_sources(layers, wg, vg, r21, r22, t11, f):
    """cascade_sources: the FP32 kernels' elimination, in complex128."""
    L, n = len(layers), len(wg)
    Wg, Vg = np.diag(wg), np.diag(vg)
    R = [None] * (L + 1)
    s = [None] * (L + 1)
    Mi, rhob, sig, asum = [None] * L, [None] * L, [None] * L, [None] * L
    R[L], s[L] = np.diag(t11), f['bot']
    for l in range(L - 1, -1, -1):
        W, V, X = layers[l]
        Wi, Vi = np.linalg.inv(W), np.linalg.inv(V)
        P1 = Wi @ Wg @ (np.eye(n) + R[l + 1])
        P2 = Vi @ Vg @ (np.eye(n) - R[l + 1])
        M, N = P1 + P2, P1 - P2
        rb = N @ np.linalg.inv(M)
        rt = np.diag(X) @ rb @ np.diag(X)
        X1, X2 = (np.eye(n) - rt) @ Wi, (np.eye(n) + rt) @ Vi
        A, Bm = X1 @ Wg + X2 @ Vg, -X1 @ Wg + X2 @ Vg
        R[l] = np.linalg.solve(A, Bm)
        a3 = Wi @ (wg[:, None] * s[l + 1] + f['e3'][l])
        a4 = Vi @ (-vg[:, None] * s[l + 1] + f['e4'][l])
        sig[l] = 0.5 * ((a3 - a4) - rb @ (a3 + a4))
        asum[l] = a3 + a4
        D = Wi @ f['e1'][l] - Vi @ f['e2'][l]
        Y2 = X[:, None] * (Wi @ f['e1'][l] + Vi @ f['e2'][l])
        s[l] = np.linalg.solve(A, 2 * X[:, None] * sig[l] - D + X[:, None] * (rb @ Y2))
        Mi[l], rhob[l] = np.linalg.inv(M), rb
    G0 = np.eye(n) - np.diag(r22) @ R[0]
    g = [None] * (L + 1)
    h = [None] * (L + 1)
    cp, cm = [None] * L, [None] * L
    g[0] = np.linalg.solve(G0, r22[:, None] * s[0] + f['top'])
    for l in range(L):
        W, V, X = layers[l]
        h[l] = R[l] @ g[l] + s[l]
        r1 = np.linalg.solve(W, wg[:, None] * (g[l] + h[l]) + f['e1'][l])
        r2 = np.linalg.solve(V, vg[:, None] * (g[l] - h[l]) + f['e2'][l])
        cp[l] = 0.5 * (r1 + r2)
        g[l + 1] = Mi[l] @ (2 * X[:, None] * cp[l] - asum[l])
        cm[l] = rhob[l] @ (X[:, None] * cp[l]) + sig[l]
    h[L] = t11[:, None] * g[L] + s[L]
    return g, h, cp, cm


def _residual(layers, wg, vg, r21, r22, t11, C, g, h, cp, cm):
    """The interface equations' residuals (res_u/res_f/res_tb kernels)."""
    out = {'top': g[0] - r21[:, None] * C - r22[:, None] * h[0], 'e1': [], 'e2': [], 'e3': [], 'e4': []}
    for l, (W, V, X) in enumerate(layers):
        out['e1'].append(W @ (cp[l] + X[:, None] * cm[l]) - wg[:, None] * (g[l] + h[l]))
        out['e2'].append(V @ (cp[l] - X[:, None] * cm[l]) - vg[:, None] * (g[l] - h[l]))
        out['e3'].append(W @ (X[:, None] * cp[l] + cm[l]) - wg[:, None] * (g[l + 1] + h[l + 1]))
        out['e4'].append(V @ (X[:, None] * cp[l] - cm[l]) - vg[:, None] * (g[l + 1] - h[l + 1]))
    out['bot'] = h[-1] - t11[:, None] * g[-1]
    return out


def test_source_carrying_elimination_solves_the_interface_equations():
    rng = np.random.default_rng(3)
    n, L, k = 6, 3, 3
    layers = [_layer(rng, n) for _ in range(L)]
    wg = 1.0 + 0.1 * rng.random(n) + 0j
    vg = -1j * (1.0 + rng.random(n))
    r21 = 0.8 + 0.1j * rng.random(n)
    r22 = 0.2 * (rng.random(n) - 0.5) + 0j
    t11 = 0.3 * (rng.random(n) - 0.5) + 0j
    C = rng.standard_normal((n, k)) + 1j * rng.standard_normal((n, k))
    # 1) from a zero state with only the incidence as a source: the plain cascade's solution
    zero = {'top': r21[:, None] * C, 'bot': np.zeros((n, k), complex),
            'e1': [np.zeros((n, k), complex)] * L, 'e2': [np.zeros((n, k), complex)] * L,
            'e3': [np.zeros((n, k), complex)] * L, 'e4': [np.zeros((n, k), complex)] * L}
    g, h, cp, cm = _solve_sources(layers, wg, vg, r21, r22, t11, zero)
    res = _residual(layers, wg, vg, r21, r22, t11, C, g, h, cp, cm)
    worst = max(np.abs(v).max() if not isinstance(v, list) else max(np.abs(x).max() for x in v) for v in res.values())
    assert worst <= 1e-12, worst
    # 2) a defect correction: perturb the state, solve for the correction from the residuals
    g2 = [x + 1e-3 * rng.standard_normal(x.shape) for x in g]
    h2 = [x + 1e-3 * rng.standard_normal(x.shape) for x in h]
    cp2 = [x + 1e-3 * rng.standard_normal(x.shape) for x in cp]
    cm2 = [x + 1e-3 * rng.standard_normal(x.shape) for x in cm]
    r = _residual(layers, wg, vg, r21, r22, t11, C, g2, h2, cp2, cm2)
    f = {key: ([-x for x in v] if isinstance(v, list) else -v) for key, v in r.items()}
    dg, dh, dcp, dcm = _solve_sources(layers, wg, vg, r21, r22, t11, f)
    for a, b, c in ((g2, dg, g), (h2, dh, h), (cp2, dcp, cp), (cm2, dcm, cm)):
        for x, dx, y in zip(a, b, c):
            assert np.abs(x + dx - y).max() <= 1e-11
