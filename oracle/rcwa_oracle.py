"""NumPy complex128 restatement of Wavebit's RCWA raster layer path (the CPU oracle).

Test infrastructure only: the product path never imports this module. It restates, in plain
NumPy, the route the reference takes for a stack of permittivity rasters under
``Numerics(orders=..., algorithm='smm')`` with the defaults ``fourier_coefficients='sampled'``,
``factorization='li'`` and ``li_nesting='fixed'``:

* stage A — harmonic tables, the exact staircase Fourier series of each raster line, the
  Toeplitz gather and Li's nested inverse rules (``rcwa/_engine/factorization.py``);
* stage B — the 2D layer operator, its eigen-decomposition, the ``q`` branch and the H-field
  modes (``rcwa/_engine/solve_2d.py``, ``_common/conventions.py``);
* stage C — gap bases, layer S-matrices, the Redheffer cascade and the per-order s/p
  efficiencies (``rcwa/_engine/scattering.py``, ``observations/power.py``).

Each function cites the reference lines it follows (paths inside ``src/wavebit``). Scope: real
incidence angles from a lossless superstrate with ``Re(eps) > 0``, non-magnetic isotropic
media, top-side plane-wave incidence on the specular order. Of the reference's exceptional-point
handling (``solve_2d.py:2463-2575``) the grazing-cluster rebuild is restated
(``rebuild_grazing_cluster``, on request); the defective-pair and cluster rebuilds are not, and
``layer_modes_2d`` reports a grazing layer through ``status``.

Parity of this module is pinned by ``tests/test_oracle_golden.py`` against fixtures generated
from the reference itself (``tests/golden/make_fixtures.py``) and against the reference's own
golden vectors.
"""
import math

import numpy as np

_PI = 3.141592653589793
_HALF_PI = 1.5707963267948966
_FLAT = 1e-12            # conventions.py:70
_COUPLED_REL = 1e-9      # solve_2d.py (grazing gate of layer_modes_2d, :2463-2464)

# ----------------------------------------------------------------------------- stage A1: tables


def order_labels(h, centre=0):
    """Order labels ``centre-h .. centre+h`` of one axis (engine.py:984-985)."""
    return np.arange(centre - h, centre + h + 1, dtype=np.int64)


def circulant_index(h):
    """``[[r - c]]`` for ``r, c`` in ``0..2h`` (factorization.py:276-286)."""
    size = 2 * h + 1
    r = np.arange(size)
    return (r[:, None] - r[None, :]).astype(np.int32)


def toeplitz_positions(h):
    """Row-major gather index ``r - c + 2h`` into a ``4h+1`` coefficient vector
    (factorization.py:358-366)."""
    return (circulant_index(h) + 2 * h).reshape(-1).astype(np.int32)


def separable_kxy(wavelength, period, k_inc, hu, hv):
    """Normalised in-plane wavevectors of the retained orders (engine.py:953-993).

    ``kx = k_inc_x + m * (wavelength / period_x)``, ``ky`` likewise, as complex128; ``m`` runs
    over :func:`order_labels`.
    """
    mu_, mv_ = order_labels(hu), order_labels(hv)
    kx = (k_inc[0] + mu_ * (wavelength / period[0])).astype(np.complex128)
    ky = (k_inc[1] + mv_ * (wavelength / period[1])).astype(np.complex128)
    return kx, ky


def incident_kxy(theta, phi, eps_top):
    """``n * sin(theta) * (cos(phi), sin(phi))`` for a lossless superstrate
    (engine.py:2706-2790, the real-angle branch with ``N = sqrt(eps)``)."""
    index = math.sqrt(float(np.real(eps_top)))
    theta = complex(theta)
    phi = complex(phi)
    st = np.sin(np.complex128(theta))
    return (np.complex128(index * st * np.cos(np.complex128(phi))),
            np.complex128(index * st * np.sin(np.complex128(phi))))


def order_grid(kx, ky):
    """Flattened order grid, ``i = n * n_u + m`` (solve_2d.py:76-98, :2720-2724)."""
    n_u, n_v = kx.shape[0], ky.shape[0]
    kxg = np.broadcast_to(kx[None, :], (n_v, n_u)).reshape(-1)
    kyg = np.broadcast_to(ky[:, None], (n_v, n_u)).reshape(-1)
    return kxg, kyg

# -------------------------------------------------------------------- stage A2: raster series


def pixel_correction(orders, n):
    """``sinc(k/n) * exp(-i*pi*k/n)`` — the exact box transform of a pixel
    (factorization.py:289-333)."""
    k = np.asarray(orders, dtype=np.complex128)
    t = k / n
    num = np.sin(_PI * t)
    den = np.where(t == 0, np.ones_like(t), _PI * t)
    sinc = np.where(t == 0, np.ones_like(t), num / den)
    return sinc * np.exp(-1j * _PI * k / n)


def raster_series(a, h):
    """Orders ``-2h..2h`` of the staircase along the last axis (factorization.py:369-440).

    ``DFT((a - a0)/n)`` picked at ``k mod n``, times :func:`pixel_correction`, plus ``a0`` at
    order 0.
    """
    a = np.asarray(a, dtype=np.complex128)
    n = a.shape[-1]
    orders = list(range(-2 * h, 2 * h + 1))
    base = a[..., :1]
    d = a - base
    if n == 1:
        spectrum = d
    else:
        spectrum = np.fft.fft(d / n, axis=-1)
    picked = np.take(spectrum, [k % n for k in orders], axis=-1)
    out = picked * pixel_correction(orders, n)
    at_zero = np.asarray([k == 0 for k in orders])
    return out + np.where(at_zero, base, np.zeros_like(base))

# ------------------------------------------------------------------ stage A3: Li's nested rules


def conv_matrix(grid, hu, hv, su=None, sv=None):
    """Direct rule both ways, BTTB layout rows ``i = n*n_u + m`` (factorization.py:504-520).
    ``su`` / ``sv`` are the series along u / v (default: the raster staircase series)."""
    su = su or (lambda a: raster_series(a, hu))
    sv = sv or (lambda a: raster_series(a, hv))
    n_u, n_v = 2 * hu + 1, 2 * hv + 1
    by_column = sv(grid.T)                                # [j_u, k_v]
    coeffs = su(by_column.T)                              # [k_v, k_u]
    blocks = np.take(np.take(coeffs, toeplitz_positions(hv), axis=0),
                     toeplitz_positions(hu), axis=1)
    out = blocks.reshape(n_v, n_v, n_u, n_u).transpose(0, 2, 1, 3)
    return out.reshape(n_v * n_u, n_v * n_u)


def nested_rule_v_inner(grid, hu, hv, invert_outer, su=None, sv=None):
    """``T_u([T_v(g)]^-1)``, optionally inverted (factorization.py:523-567, ``inner='v'``)."""
    su = su or (lambda a: raster_series(a, hu))
    sv = sv or (lambda a: raster_series(a, hv))
    n_u, n_v = 2 * hu + 1, 2 * hv + 1
    lines = sv(grid.T)                                    # [j_u, k_v]
    inner = np.linalg.inv(np.take(lines, toeplitz_positions(hv), axis=1)
                          .reshape(lines.shape[0], n_v, n_v))
    entries = inner.reshape(lines.shape[0], n_v * n_v).T  # [(n, n'), j_u]
    outer = np.take(su(entries), toeplitz_positions(hu), axis=1)
    out = outer.reshape(n_v, n_v, n_u, n_u).transpose(0, 2, 1, 3).reshape(n_v * n_u, n_v * n_u)
    return np.linalg.inv(out) if invert_outer else out


def li_conv(eps, hu, hv, su=None, sv=None):
    """One layer's ``(epx, epy, epz_i)`` under fixed nesting (factorization.py:600-671)."""
    eps = np.asarray(eps, dtype=np.complex128)
    epx = nested_rule_v_inner(eps, hu, hv, invert_outer=True, su=su, sv=sv)
    epy = nested_rule_v_inner(1.0 / eps, hu, hv, invert_outer=False, su=su, sv=sv)
    epz_i = np.linalg.inv(conv_matrix(eps, hu, hv, su=su, sv=sv))
    return epx, epy, epz_i


# ------------------------------------------------------ stage A: integrated coefficients


def compression_indices(cell):
    """Last row / column of each run of identical neighbours, and the right-hand edges they
    place on the unit cell (factorization.py:3005-3045). Columns are compared first; rows are
    compared on the column-reduced raster."""
    cell = np.asarray(cell)
    n_row, n_col = cell.shape
    col_idx = np.flatnonzero(np.any(cell[:, :-1] != cell[:, 1:], axis=0)).tolist() + [n_col - 1]
    reduced = cell[:, col_idx]
    row_idx = np.flatnonzero(np.any(reduced[:-1, :] != reduced[1:, :], axis=1)).tolist() + [n_row - 1]
    x = (np.asarray(col_idx, dtype=np.float64) + 1.0) / n_col
    y = (np.asarray(row_idx, dtype=np.float64) + 1.0) / n_row
    return row_idx, col_idx, x, y


def segment_bounds(edges):
    """``(left, width)`` of the segments ending at ``edges`` on the unit cell
    (factorization.py:443-454)."""
    right = np.asarray(edges, dtype=np.float64).reshape(-1)
    right = right / right[-1]
    left = np.concatenate([[0.0], right[:-1]])
    return left, right - left


def segment_series(left, width, h):
    """Orders ``-2h..2h`` of a profile constant on segments ``[left_j, left_j + width_j)``, in the
    jump form ``c_k = sum_j (a_j - a_{j-1}) exp(-2 pi i k left_j) / (2 pi i k)``,
    ``c_0 = sum_j a_j width_j`` (factorization.py:457-501)."""
    orders = np.arange(-2 * h, 2 * h + 1)
    scale = np.array([0j if o == 0 else 1.0 / (2j * math.pi * o) for o in orders])
    weights = np.exp(-2j * math.pi * (left[:, None] * orders[None, :]))

    def series(a):
        a = np.asarray(a, dtype=np.complex128)
        jumps = a - np.roll(a, 1, axis=-1)
        ac = jumps @ (weights * scale[None, :])
        dc = (a @ width.astype(np.complex128))[..., None]
        return np.where(orders == 0, dc, ac)
    return series


def li_conv_integrated(eps, hu, hv):
    """One layer's ``(epx, epy, epz_i)`` with integrated (closed-form segment) coefficients on
    the compressed raster (factorization.py:674-686, :3135-3206)."""
    eps = np.asarray(eps, dtype=np.complex128)
    row_idx, col_idx, x, y = compression_indices(eps)
    comp = eps[np.ix_(row_idx, col_idx)]
    su = segment_series(*segment_bounds(x), hu)
    sv = segment_series(*segment_bounds(y), hv)
    return li_conv(comp, hu, hv, su=su, sv=sv)


def to_conv_mat_raster_integrated(structure, hu, hv):
    """Per-layer integrated slots stacked ``(L, N, N)`` (factorization.py:3181-3206)."""
    out = [li_conv_integrated(e, hu, hv) for e in structure]
    return tuple(np.stack([o[i] for o in out]) for i in range(3))


def to_conv_mat_raster_sampled(structure, hu, hv):
    """Per-layer slots stacked ``(L, N, N)`` (factorization.py:915-941)."""
    out = [li_conv(e, hu, hv) for e in structure]
    return tuple(np.stack([o[i] for o in out]) for i in range(3))


def swap_fourier_origin(conv, hu, hv):
    """Corner frame <-> centre frame: ``D C D``, ``D = diag((-1)^(m+n))``
    (conventions.py:1263-1292)."""
    m = order_labels(hu)[None, :] + order_labels(hv)[:, None]
    d = np.where(m.reshape(-1) % 2 == 0, 1.0, -1.0)
    return d[:, None] * conv * d[None, :]

# ----------------------------------------------------------------- stage B: layer eigenmodes


def mode_q(w):
    """``q = sqrt(w)`` with ``Re q >= 0``, tie ``Im q <= 0`` (conventions.py:186-249)."""
    v = np.sqrt(w)
    flip = np.where(np.abs(np.real(v)) > _FLAT, np.real(v) < 0, np.imag(v) > 0)
    return np.where(flip, -v, v)


def layer_operator(kxg, kyg, epx, epy, epz_i):
    """``Omega2_LR`` and ``Omega_R`` of a Li layer, ``epxy = epyx = 0``
    (solve_2d.py:2377-2418)."""
    N = kxg.shape[0]
    Bm = (kxg[:, None] * epz_i) * kxg[None, :] - np.eye(N)
    Dm = (kyg[:, None] * epz_i) * kyg[None, :] - np.eye(N)
    Cc = (kxg[:, None] * epz_i) * kyg[None, :]
    Em = (kyg[:, None] * epz_i) * kxg[None, :]
    Kx, Ky = np.diag(kxg), np.diag(kyg)
    O = np.zeros((N, N), np.complex128)
    omega2 = np.block([
        [Ky @ Ky + Bm @ epx - Cc @ O, Cc @ epy - Kx @ Ky - Bm @ O],
        [Em @ epx - Ky @ Kx - Dm @ O, Kx @ Kx + Dm @ epy - Em @ O]])
    omega_r = np.block([[-(Kx @ Ky) + O, Kx @ Kx - epy],
                        [epx - Ky @ Ky, Ky @ Kx - O]])
    return omega2, omega_r


def layer_modes_2d(kxg, kyg, epx, epy, epz_i, rebuild=False):
    """``(W, V, q, status)`` of one 2D layer (solve_2d.py:2303-2460).

    ``status`` is 0, or 1 where ``min|w| < 1e-9 max|w|`` (the grazing gate at
    solve_2d.py:2463-2464). With ``rebuild`` such a layer's cluster is re-derived from the
    first-order problem (:func:`rebuild_grazing_cluster`) and status goes back to 0, or
    ``FloatingPointError`` is raised where the cluster is numerically defective.
    """
    omega2, omega_r = layer_operator(kxg, kyg, epx, epy, epz_i)
    w, W = np.linalg.eig(omega2)
    q = mode_q(w)
    V = (omega_r @ W) / q
    aw = np.abs(w)
    status = int(np.min(aw) < _COUPLED_REL * np.max(aw))
    if status and rebuild:
        out = rebuild_grazing_cluster(w, W, V, q, left_factor(kxg, kyg, epz_i), omega_r)
        if out is not None:
            W, V, q = out
            status = 0
    return W, V, q, w, status


_DEFECTIVE_REL = 1e-10   # solve_2d.py:73


def left_factor(kxg, kyg, epz_i):
    """``Omega_L = [[-Cc, B], [-D, E]]`` (solve_2d.py:2380-2390, 2470-2471), with
    ``Omega2 = Omega_L Omega_R`` for a non-magnetic layer."""
    N = kxg.shape[0]
    I = np.eye(N, dtype=np.complex128)
    Bm = (kxg[:, None] * epz_i) * kxg[None, :] - I
    Dm = (kyg[:, None] * epz_i) * kyg[None, :] - I
    Cc = (kxg[:, None] * epz_i) * kyg[None, :]
    Em = (kyg[:, None] * epz_i) * kxg[None, :]
    return np.block([[-Cc, Bm], [-Dm, Em]])


def rebuild_grazing_cluster(w, W, V, q, omega_l, omega_r):
    """The grazing cluster re-derived from the coupled first-order problem
    (solve_2d.py:118-222): the clusters of ``Omega_L Omega_R`` and ``Omega_R Omega_L`` as
    orthonormal bases, the factors restricted to them, the small first-order eigenproblem,
    ``k`` of its pairs chosen jointly independent, each rooted by ``mode_q``. ``None`` where the
    two clusters differ in size; ``FloatingPointError`` where the coupled rates split by less
    than 1e-10 of the modal scale."""
    aw = np.abs(w)
    J = np.where(aw < _COUPLED_REL * aw.max())[0]
    wh, Vh = np.linalg.eig(omega_r @ omega_l)
    Jh = np.where(np.abs(wh) < _COUPLED_REL * np.abs(wh).max())[0]
    if len(Jh) != len(J):
        return None
    k = len(J)
    QE = np.linalg.qr(W[:, J])[0]
    QH = np.linalg.qr(Vh[:, Jh])[0]
    Rr = QH.conj().T @ (omega_r @ QE)
    Lr = QE.conj().T @ (omega_l @ QH)
    Zk = np.zeros((k, k), np.complex128)
    mu, g = np.linalg.eig(np.block([[Zk, Lr], [Rr, Zk]]))
    g = g / np.linalg.norm(g, axis=0, keepdims=True)
    chosen, re_, rh_ = [], g[:k].copy(), g[k:].copy()
    for _ in range(k):
        score = np.linalg.norm(re_, axis=0) ** 2 + np.linalg.norm(rh_, axis=0) ** 2
        score[chosen] = -1.0
        c = int(np.argmax(score))
        chosen.append(c)
        for m in (re_, rh_):
            v = m[:, c]
            nv = np.linalg.norm(v)
            if nv > 1e-150:
                u = v / nv
                m -= u[:, None] * (u.conj() @ m)[None, :]
    if np.abs(mu[chosen]).min() < _DEFECTIVE_REL * np.sqrt(aw.max()):
        raise FloatingPointError('a 2D layer eigenmode pair is numerically defective at a grazing condition')
    W, V, q = W.copy(), V.copy(), q.copy()
    for i, c in enumerate(chosen):
        qi = mode_q(np.asarray([mu[c] ** 2]))[0]
        gh = g[k:, c] if abs(qi - mu[c]) <= abs(qi + mu[c]) else -g[k:, c]
        W[:, J[i]] = QE @ g[:k, c]
        V[:, J[i]] = QH @ gh
        q[J[i]] = qi
    return W, V, q


def order_azimuth(ky, kx, phi):
    """Per-order azimuth of ``(kx, ky)`` (conventions.py:1316-1431)."""
    zero_kx = kx == 0
    safe_kx = np.where(zero_kx, np.ones_like(kx * ky), kx)
    varphi = np.arctan(ky / safe_kx)
    varphi = varphi + _PI * (np.real(kx + np.zeros_like(varphi)) < 0).astype(varphi.dtype)
    ky_b = ky + np.zeros_like(varphi)
    right = np.where(np.real(ky_b) < 0, np.full_like(varphi, -_HALF_PI),
                     np.full_like(varphi, _HALF_PI))
    safe_ky = np.where(ky_b == 0, np.ones_like(ky_b), ky_b)
    right = right - (kx + np.zeros_like(varphi)) / safe_ky
    varphi = np.where(zero_kx, right, varphi)
    p = np.complex128(phi)
    inc = (np.arctan(np.sin(p) / np.cos(p)) + _PI * float(np.real(np.cos(p)) < 0)
           + np.zeros_like(varphi))
    return np.where(zero_kx & (ky == 0), inc, varphi).reshape(-1)


def sp_modes_2d(W, V, c, s, N):
    """Rotate ``W, V`` into the per-order s/p basis (solve_2d.py:2584-2616)."""
    c = c[:, None]
    s = s[:, None]
    W11, W12, W21, W22 = W[:N, :N], W[:N, N:], W[N:, :N], W[N:, N:]
    V11, V12, V21, V22 = V[:N, :N], V[:N, N:], V[N:, :N], V[N:, N:]
    big_W = np.block([[c * W21 - s * W11, c * W22 - s * W12],
                      [c * W11 + s * W21, c * W12 + s * W22]])
    big_V = np.block([[c * V11 + s * V21, c * V12 + s * V22],
                      [c * V21 - s * V11, c * V22 - s * V12]])
    return big_W, big_V

# ---------------------------------------------------------------------- stage C: S-matrices


def boundary_kz(eps, k_par_sq):
    """Downward ``kz`` on Maystre's cut (conventions.py:655-760, non-magnetic branch)."""
    v = np.sqrt(eps - k_par_sq)
    return np.where(np.real(v) + np.imag(v) < 0, -v, v)


def gap_waves(kxg, kyg):
    """``sqrt(1 + |kx|^2 + |ky|^2)`` per order (scattering.py:128-160)."""
    abs_sq = np.real(kxg * np.conj(kxg)) + np.real(kyg * np.conj(kyg))
    return np.sqrt(1 + abs_sq).astype(np.complex128)


def ab_matrices(W_to, V_to, W_from, V_from):
    """``A = W_to^-1 W_from + V_to^-1 V_from``, ``B`` the difference (scattering.py:116-125)."""
    P = np.linalg.inv(W_to) @ W_from
    Q = np.linalg.inv(V_to) @ V_from
    return P + Q, P - Q


def s_layer(A, B, X):
    """Symmetric layer S-matrix between gaps (scattering.py:163-174)."""
    A_i = np.linalg.inv(A)
    XB = X @ B
    common = np.linalg.inv(A - XB @ A_i @ X @ B)
    S11 = common @ (XB @ A_i @ X @ A - B)
    S12 = common @ X @ (A - B @ A_i @ B)
    return S11, S12, S12, S11


def s_reflection(W_top, V_top, W_gap, V_gap):
    """Superstrate -> gap interface (scattering.py:177-181)."""
    A, B = ab_matrices(W_gap, V_gap, W_top, V_top)
    A_i = np.linalg.inv(A)
    return -A_i @ B, 2 * A_i, 0.5 * (A - B @ A_i @ B), B @ A_i


def s_transmission(W_bot, V_bot, W_gap, V_gap):
    """Gap -> substrate interface (scattering.py:184-188)."""
    A, B = ab_matrices(W_gap, V_gap, W_bot, V_bot)
    A_i = np.linalg.inv(A)
    return B @ A_i, 0.5 * (A - B @ A_i @ B), 2 * A_i, -A_i @ B


def redheffer_star(S_a, S_b):
    """``S_a * S_b`` (scattering.py:191-200)."""
    a11, a12, a21, a22 = S_a
    b11, b12, b21, b22 = S_b
    I = np.eye(a11.shape[0], dtype=a11.dtype)
    D_i = np.linalg.inv(I - b11 @ a22)
    F_i = np.linalg.inv(I - a22 @ b11)
    return (a11 + a12 @ D_i @ b11 @ a21, a12 @ D_i @ b12,
            b21 @ F_i @ a21, b22 + b21 @ F_i @ a22 @ b12)


def polarization_pair(polarization):
    """``(a_s, a_p)``: ``'s'`` is ``psi = pi/2``, ``'p'`` is ``psi = 0``, a pair is normalised
    (conventions.py:1022-1066)."""
    if isinstance(polarization, str):
        psi = _HALF_PI if polarization == 's' else 0.0
        return np.sin(np.complex128(psi)), np.cos(np.complex128(psi))
    a_s, a_p = (np.complex128(v) for v in polarization)
    norm = np.sqrt(abs(a_s) ** 2 + abs(a_p) ** 2)
    return a_s / norm, a_p / norm


def sp_result(S, kx, ky, kz_top, kz_bot, n_top, n_bot, eps_top, eps_bot, incidence):
    """Per-order efficiencies for the given, pure-s and pure-p columns
    (scattering.py:907-994; solve_1d.py:1588-1610; observations/power.py:13-159)."""
    N = kz_top.shape[0]
    n_v, n_u = ky.shape[0], kx.shape[0]
    delta = np.zeros((N, 1), np.complex128)
    delta[N // 2] = 1.0

    def incident(a_s, a_p):
        return np.concatenate([a_s * delta, -1j * (n_top / 1.0) * a_p * delta], axis=0)

    cols = [incident(*incidence),
            incident(np.sin(np.complex128(_HALF_PI)), np.cos(np.complex128(_HALF_PI))),
            incident(np.sin(np.complex128(0.0)), np.cos(np.complex128(0.0)))]
    c_inc = np.concatenate(cols, axis=1)
    c_ref = S[0] @ c_inc
    c_trn = S[2] @ c_inc

    def as_orders(M):
        return M.T.reshape(3, n_v, n_u)

    R_s, R_p = as_orders(c_ref[:N]), as_orders(-c_ref[N:])
    T_s, T_p = as_orders(c_trn[:N]), as_orders(c_trn[N:])
    kzt, kzb = kz_top.reshape(n_v, n_u), kz_bot.reshape(n_v, n_u)
    spec_t = kz_top[N // 2]
    s_power = np.real(spec_t / 1.0)
    p_power = abs(n_top / 1.0) ** 2 * np.real(spec_t / eps_top)
    a_s, a_p = incidence
    powers = np.array([abs(a_s) ** 2 * s_power + abs(a_p) ** 2 * p_power, s_power, p_power])
    denom = powers.reshape(3, 1, 1)

    def wave_power(a, adm):
        return np.real(a * np.conj(a)) * np.real(adm)

    eff = (wave_power(R_s, kzt / 1.0) / denom, wave_power(R_p, kzt / eps_top) / denom,
           wave_power(T_s, kzb / 1.0) / denom, wave_power(T_p, kzb / eps_bot) / denom)
    R = eff[0] + eff[1]
    T = eff[2] + eff[3]
    amps = (R_s, R_p / (-1j * n_top), T_s, T_p / (-1j * n_bot))
    return R, T, eff, amps


def exported_scattering(S, hu, hv):
    """The stack's ``S`` as the reference publishes it (``Outputs(scattering=True)``,
    scattering.py:482-605): the four blocks at the half-space ports with s amplitudes first and
    the p port variables after, each order referenced at the cell centre -- ``C S C`` of the
    corner-frame cascade, ``C = diag((-1)^(m+n))`` on both polarization halves."""
    m = order_labels(hu)[None, :] + order_labels(hv)[:, None]
    d = np.where(m.reshape(-1) % 2 == 0, 1.0, -1.0)
    c = np.concatenate([d, d])
    return tuple(c[:, None] * blk * c[None, :] for blk in S)


def amplitude_ratios(amps, hu, hv):
    """The published amplitude ratios (results.py:357-390): the Fresnel amplitudes of
    :func:`sp_result` (r_s, r_p, t_s, t_p, each ``(3, n_v, n_u)``) referenced at the cell centre,
    order (m, n) times ``(-1)^(m+n)``."""
    m = order_labels(hu)[None, :] + order_labels(hv)[:, None]
    d = np.where(m % 2 == 0, 1.0, -1.0)
    return tuple(d[None] * a for a in amps)


def solve_stack(structure, thickness, wavelength, period, hu, hv, theta=0.0, phi=0.0,
                eps_top=1.0, eps_bot=1.0, polarization='s', conv=None, keep=False, rebuild_grazing=False):
    """One SMM solve of a raster stack (scattering.py:1185-1456; engine.py:7836-7880).

    ``structure`` is ``(L, ny, nx)`` relative permittivity, ``thickness`` ``(L,)`` in the
    units of ``wavelength`` and ``period``. Returns a dict with ``R``, ``T`` of shape
    ``(3, n_v, n_u)`` (given polarization, pure s, pure p), the s/p efficiencies, the
    amplitudes, the final S-matrix and per-layer statuses.
    """
    structure = np.asarray(structure, dtype=np.complex128)
    L = structure.shape[0]
    if conv is None:
        conv = to_conv_mat_raster_sampled(structure, hu, hv)
    epx_all, epy_all, epz_i_all = conv
    k_inc = incident_kxy(theta, phi, eps_top)
    kx, ky = separable_kxy(wavelength, period, k_inc, hu, hv)
    kxg, kyg = order_grid(kx, ky)
    N = kxg.shape[0]
    k0 = 2 * _PI / wavelength
    eps_top = np.complex128(eps_top)
    eps_bot = np.complex128(eps_bot)
    n_top, n_bot = np.sqrt(eps_top), np.sqrt(eps_bot)
    k_par_sq = kxg ** 2 + kyg ** 2
    kz_top = boundary_kz(n_top ** 2, k_par_sq)
    kz_bot = boundary_kz(n_bot ** 2, k_par_sq)
    y = gap_waves(kxg, kyg)
    I, O = np.eye(N, dtype=np.complex128), np.zeros((N, N), np.complex128)
    W_top = np.block([[I, O], [O, -1j * np.diag(kz_top) / eps_top]])
    V_top = np.block([[-1j * np.diag(kz_top) / 1.0, O], [O, I]])
    W_bot = np.block([[I, O], [O, -1j * np.diag(kz_bot) / eps_bot]])
    V_bot = np.block([[-1j * np.diag(kz_bot) / 1.0, O], [O, I]])
    W_gap = np.block([[I, O], [O, -1j * np.diag(y)]])
    V_gap = np.block([[-1j * np.diag(y), O], [O, I]])
    varphi = order_azimuth(kyg.reshape(ky.shape[0], kx.shape[0]),
                           kxg.reshape(ky.shape[0], kx.shape[0]), phi)
    c, s = np.cos(varphi), np.sin(varphi)
    S = s_reflection(W_top, V_top, W_gap, V_gap)
    S_trn = s_transmission(W_bot, V_bot, W_gap, V_gap)
    status = []
    layers = []
    for i in range(L):
        W, V, q, w, st = layer_modes_2d(kxg, kyg, epx_all[i], epy_all[i], epz_i_all[i], rebuild=rebuild_grazing)
        status.append(st)
        big_W, big_V = sp_modes_2d(W, V, c, s, N)
        X = np.diag(np.exp(-k0 * thickness[i] * q))
        A, B = ab_matrices(big_W, big_V, W_gap, V_gap)
        S = redheffer_star(S, s_layer(A, B, X))
        if keep:
            layers.append(dict(W=W, V=V, q=q, w=w))
    S = redheffer_star(S, S_trn)
    inc = polarization_pair(polarization)
    R, T, eff, amps = sp_result(S, kx, ky, kz_top, kz_bot, n_top, n_bot, eps_top, eps_bot, inc)
    out = dict(R=R, T=T, eff=eff, amps=amps, S=S, status=status, kx=kx, ky=ky)
    if keep:
        out['layers'] = layers
    return out

# ------------------------------------------------------------ fields (Outputs(fields=True))

_Z0 = 1.0 / (8.8541878188e-12 * 299792458.0)     # free-space impedance, units.py:7-9
_TOP_FACE = 1.0                                  # scattering.py:225-232


def below_reflections(S_layers, S_trn):
    """``(gamma, F)``: the reflection below each split plane and each layer's gap-to-gap map,
    bottom-up (scattering.py:236-267)."""
    n = len(S_layers)
    I = np.eye(S_trn[0].shape[0], dtype=np.complex128)
    gamma, F = [None] * (n + 1), [None] * n
    gamma[n] = S_trn[0]
    for p in range(n - 1, -1, -1):
        s11, s12, s21, s22 = S_layers[p]
        below = gamma[p + 1]
        F[p] = np.linalg.solve(I - s22 @ below, s21)
        gamma[p] = s11 + s12 @ (below @ F[p])
    return gamma, F


def field_state(S_ref, S_trn, S_layers, AB, roots, c_inc):
    """Each layer's ``(+, -)`` mode amplitudes, ``+`` at its top face and ``-`` at its bottom,
    read off the gap amplitudes of the cascade (scattering.py:270-350); a mode with
    ``|k0 q d| < 1`` takes its ``-`` from the top face (modal_gradient.two_face, value only)."""
    I = np.eye(S_trn[0].shape[0], dtype=np.complex128)
    gamma, F = below_reflections(S_layers, S_trn)
    g = np.linalg.solve(I - S_ref[3] @ gamma[0], S_ref[2] @ c_inc)
    out = []
    for p, ((A, B), (q, k0_d)) in enumerate(zip(AB, roots)):
        g_next = F[p] @ g
        up_top = gamma[p] @ g
        plus = 0.5 * (A @ g + B @ up_top)
        minus_top = 0.5 * (B @ g + A @ up_top)
        minus_bottom = 0.5 * (B @ g_next + A @ (gamma[p + 1] @ g_next))
        keep = (np.abs(q * k0_d) < _TOP_FACE)[:, None]
        with np.errstate(over='ignore', invalid='ignore'):
            carried = np.exp(k0_d * q)[:, None] * minus_top
        out.append((plus, np.where(keep, carried, minus_bottom)))
        g = g_next
    return out


def layer_field_coefficients(W, V, q, d, k0, epz_i, kxg, kyg, plus, minus, z):
    """Per-order ``(Sx, Sy, -Sz, i Ux, i Uy, -i Uz)`` at depths ``z`` below a layer's top face,
    in the propagation frame (fields.py:630-790, 2D layout, ``U = i H``)."""
    N = kxg.shape[0]
    z = np.asarray(z, dtype=np.float64)[:, None]
    fwd = np.exp(-k0 * q[None, :] * z)                  # (nz, n)
    bwd = np.exp(k0 * q[None, :] * (z - d))
    ap = fwd * plus[None, :]
    am = bwd * minus[None, :]
    a1p, a2p, a1m, a2m = ap[:, :N], ap[:, N:], am[:, :N], am[:, N:]
    W11, W12, W21, W22 = W[:N, :N], W[:N, N:], W[N:, :N], W[N:, N:]
    V11, V12, V21, V22 = V[:N, :N], V[:N, N:], V[N:, :N], V[N:, N:]
    s1, s2, d1, d2 = a1p + a1m, a2p + a2m, -a1p + a1m, -a2p + a2m
    Sx = s1 @ W11.T + s2 @ W12.T
    Sy = s1 @ W21.T + s2 @ W22.T
    Ux = d1 @ V11.T + d2 @ V12.T
    Uy = d1 @ V21.T + d2 @ V22.T
    Sz = 1j * (kxg[None, :] * Uy - kyg[None, :] * Ux) @ epz_i.T
    Uz = 1j * (kxg[None, :] * Sy - kyg[None, :] * Sx)
    return np.stack([Sx, Sy, -Sz, 1j * Ux, 1j * Uy, -1j * Uz], axis=-1)   # (nz, N, 6)


def field_phasors(structure, thickness, wavelength, period, hu, hv, theta, phi, eps_top, eps_bot,
                  polarization, amplitude, x, y, z, conv=None):
    """Collocated ``(Ex, Ey, Ez, Hx, Hy, Hz)`` at the points ``x`` (from the cell centre),
    ``y`` and ``z`` (upward from the stack's bottom face; a face belongs to the layer above it),
    shape ``(nz, ny, nx, 6)``, E in V/m per V/m of ``amplitude`` and H in A/m
    (results.py:148-229, field_result.py:332-700, fields.py:630-790). Layers are listed entry
    (top) face first, as :func:`solve_stack` takes them."""
    structure = np.asarray(structure, dtype=np.complex128)
    thickness = np.asarray(thickness, dtype=np.float64)
    L = structure.shape[0]
    if conv is None:
        conv = to_conv_mat_raster_sampled(structure, hu, hv)
    epx_all, epy_all, epz_i_all = conv
    k_inc = incident_kxy(theta, phi, eps_top)
    kx, ky = separable_kxy(wavelength, period, k_inc, hu, hv)
    kxg, kyg = order_grid(kx, ky)
    N = kxg.shape[0]
    k0 = 2 * _PI / wavelength
    eps_top, eps_bot = np.complex128(eps_top), np.complex128(eps_bot)
    n_top = np.sqrt(eps_top)
    k_par_sq = kxg ** 2 + kyg ** 2
    kz_top, kz_bot = boundary_kz(eps_top, k_par_sq), boundary_kz(eps_bot, k_par_sq)
    yg = gap_waves(kxg, kyg)
    I, O = np.eye(N, dtype=np.complex128), np.zeros((N, N), np.complex128)
    W_top = np.block([[I, O], [O, -1j * np.diag(kz_top) / eps_top]])
    V_top = np.block([[-1j * np.diag(kz_top), O], [O, I]])
    W_bot = np.block([[I, O], [O, -1j * np.diag(kz_bot) / eps_bot]])
    V_bot = np.block([[-1j * np.diag(kz_bot), O], [O, I]])
    W_gap = np.block([[I, O], [O, -1j * np.diag(yg)]])
    V_gap = np.block([[-1j * np.diag(yg), O], [O, I]])
    varphi = order_azimuth(kyg.reshape(ky.shape[0], kx.shape[0]), kxg.reshape(ky.shape[0], kx.shape[0]), phi)
    c, s = np.cos(varphi), np.sin(varphi)
    S_ref = s_reflection(W_top, V_top, W_gap, V_gap)
    S_trn = s_transmission(W_bot, V_bot, W_gap, V_gap)
    modes, S_layers, AB, roots = [], [], [], []
    for i in range(L):
        W, V, q, w, _ = layer_modes_2d(kxg, kyg, epx_all[i], epy_all[i], epz_i_all[i])
        big_W, big_V = sp_modes_2d(W, V, c, s, N)
        X = np.diag(np.exp(-k0 * thickness[i] * q))
        A, B = ab_matrices(big_W, big_V, W_gap, V_gap)
        S_layers.append(s_layer(A, B, X))
        AB.append((A, B))
        roots.append((q, k0 * thickness[i]))
        modes.append((W, V, q))
    a_s, a_p = polarization_pair(polarization)
    delta = np.zeros((N, 1), np.complex128)
    delta[N // 2] = 1.0
    c_inc = np.concatenate([a_s * delta, -1j * n_top * a_p * delta], axis=0)
    amps = field_state(S_ref, S_trn, S_layers, AB, roots, c_inc)
    # public heights -> (layer in propagation order, depth below its top face)
    z = np.asarray(z, dtype=np.float64).reshape(-1)
    ds = thickness[::-1]                                  # bottom layer first
    edges = np.concatenate([[0.0], np.cumsum(ds)])
    owner = np.minimum((z[:, None] >= edges[None, 1:]).sum(axis=1), L - 1)
    coef = np.zeros((z.shape[0], N, 6), np.complex128)
    for j in range(L):
        sel = np.flatnonzero(owner == j)
        if not sel.size:
            continue
        p = L - 1 - j
        depth = ds[j] - (z[sel] - edges[j])
        W, V, q = modes[p]
        plus, minus = amps[p]
        coef[sel] = layer_field_coefficients(W, V, q, thickness[p], k0, epz_i_all[p], kxg, kyg,
                                             plus[:, 0], minus[:, 0], depth)
    coef = coef * np.array([1, 1, -1, -1, -1, 1])[None, None, :]          # mirror into the scene frame
    m = order_labels(hu)[None, :] + order_labels(hv)[:, None]
    coef = coef * np.where(m.reshape(-1) % 2 == 0, 1.0, -1.0)[None, :, None]   # corner -> centre
    xs = np.asarray(x, dtype=np.float64)
    ys = np.asarray(y, dtype=np.float64)
    phase = np.exp(1j * k0 * (xs[None, :, None] * kxg[None, None, :] + ys[:, None, None] * kyg[None, None, :]))
    out = np.einsum('yxo,zoc->zyxc', phase, coef)
    return amplitude * out * np.array([1, 1, 1, 1 / _Z0, 1 / _Z0, 1 / _Z0])

# --------------------------------------------------- the ETM connecting algorithm (cross-check)


def etm_stack(structure, thickness, wavelength, period, hu, hv, theta=0.0, phi=0.0, eps_top=1.0, eps_bot=1.0,
              polarization='s', conv=None):
    """One enhanced-transmittance-matrix solve (solve_2d.py:2619-2843, solve_1d.py:1389-1520):
    from the substrate up, ``a = (W^-1 F + V^-1 G)/2``, ``b = (W^-1 F - V^-1 G)/2``,
    ``Y = X b a^-1 X``, ``F = W (I + Y)``, ``G = V (I - Y)``, ``T = T a^-1 X``; then one block
    solve of the superstrate's boundary equations for ``R_s``, ``R_p`` and ``T_1``,
    ``(T_s, T_p) = T T_1``. Real in-plane wavevectors and passive layers, where the ETM's
    labels (conventions.py:252-300) are :func:`mode_q`'s and the max-volume relabelling is off;
    every layer in the plain (non-run) form of ``_run_ab``. Returns ``R``, ``T`` as
    :func:`solve_stack` does (given polarization, pure s, pure p)."""
    structure = np.asarray(structure, dtype=np.complex128)
    L = structure.shape[0]
    if conv is None:
        conv = to_conv_mat_raster_sampled(structure, hu, hv)
    epx_all, epy_all, epz_i_all = conv
    k_inc = incident_kxy(theta, phi, eps_top)
    kx, ky = separable_kxy(wavelength, period, k_inc, hu, hv)
    kxg, kyg = order_grid(kx, ky)
    N = kxg.shape[0]
    n_v, n_u = ky.shape[0], kx.shape[0]
    k0 = 2 * _PI / wavelength
    eps_top, eps_bot = np.complex128(eps_top), np.complex128(eps_bot)
    n_top = np.sqrt(eps_top)
    k_par_sq = kxg ** 2 + kyg ** 2
    kz_top, kz_bot = boundary_kz(eps_top, k_par_sq), boundary_kz(eps_bot, k_par_sq)
    varphi = order_azimuth(kyg.reshape(n_v, n_u), kxg.reshape(n_v, n_u), phi)
    c, s = np.cos(varphi), np.sin(varphi)
    I, O = np.eye(N, dtype=np.complex128), np.zeros((N, N), np.complex128)
    I2 = np.eye(2 * N, dtype=np.complex128)
    F = np.block([[I, O], [O, -1j * np.diag(kz_bot) / eps_bot]])
    G = np.block([[-1j * np.diag(kz_bot), O], [O, I]])
    T = I2.copy()
    for i in range(L - 1, -1, -1):
        W, V, q, w, _ = layer_modes_2d(kxg, kyg, epx_all[i], epy_all[i], epz_i_all[i])
        big_W, big_V = sp_modes_2d(W, V, c, s, N)
        Wi_F = np.linalg.solve(big_W, F)
        Vi_G = np.linalg.solve(big_V, G)
        a, b = 0.5 * (Wi_F + Vi_G), 0.5 * (Wi_F - Vi_G)
        a_i = np.linalg.inv(a)
        X = np.diag(np.exp(-k0 * thickness[i] * q))
        Y = X @ b @ a_i @ X
        F, G = big_W @ (I2 + Y), big_V @ (I2 - Y)
        T = T @ a_i @ X
    kz_inc = kz_top[N // 2]
    Kt = np.diag(kz_top)
    final_A = np.block([[I, O, -F[:N, :N], -F[:N, N:]],
                        [O, 1j * Kt / eps_top, -F[N:, :N], -F[N:, N:]],
                        [1j * Kt, O, -G[:N, :N], -G[:N, N:]],
                        [O, I, -G[N:, :N], -G[N:, N:]]])
    delta = np.zeros((N, 1), np.complex128)
    delta[N // 2] = 1.0
    h_p, e_p = n_top, n_top * kz_inc / eps_top

    def column(a_s, a_p):
        return np.concatenate([-a_s * delta, a_p * e_p * delta, 1j * a_s * kz_inc * delta, 1j * h_p * a_p * delta])

    inc = polarization_pair(polarization)
    cols = np.concatenate([column(*inc), column(np.sin(np.complex128(_HALF_PI)), np.cos(np.complex128(_HALF_PI))),
                           column(np.sin(np.complex128(0.0)), np.cos(np.complex128(0.0)))], axis=1)
    x = np.linalg.solve(final_A, cols)
    Rs, Rp = x[:N], x[N:2 * N]
    Tt = T @ x[2 * N:]
    Ts, Tp = Tt[:N], Tt[N:]

    def as_orders(M):
        return M.T.reshape(3, n_v, n_u)

    s_power = np.real(kz_inc)
    p_power = abs(n_top) ** 2 * np.real(kz_inc / eps_top)
    a_s, a_p = inc
    denom = np.array([abs(a_s) ** 2 * s_power + abs(a_p) ** 2 * p_power, s_power, p_power]).reshape(3, 1, 1)
    kzt, kzb = kz_top.reshape(n_v, n_u), kz_bot.reshape(n_v, n_u)

    def wave_power(amp, adm):
        return np.real(amp * np.conj(amp)) * np.real(adm)

    R = (wave_power(as_orders(Rs), kzt) + wave_power(as_orders(Rp), kzt / eps_top)) / denom
    Tr = (wave_power(as_orders(Ts), kzb) + wave_power(as_orders(Tp), kzb / eps_bot)) / denom
    return dict(R=R, T=Tr)
