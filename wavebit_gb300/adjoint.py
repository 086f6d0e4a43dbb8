"""Hand-written adjoint of the RCWA raster path: gradients of a loss on the per-order
efficiencies with respect to raster permittivities and layer thicknesses.

Reference behaviour: the reference differentiates through its array backends
(rcwa/_engine/modal_gradient.py:56-251 — the eigen-solve carries its derivative through a
square-root Sylvester generator; _common/backend.py:1724-1759 — the broadened reciprocal gap
``conj(D)/(|D|^2 + eps)`` for (near-)degenerate eigenvalues). Here every stage has an explicit
reverse pass:

* efficiencies    R = sum |a|^2 Re(kz / mu or kz / eps) / P_inc      (scattering.py:907-994)
* cascade         bottom-up reflections R_k and the top-down incidence pass (the star algebra
                  of scattering.py:163-200 evaluated for the blocks the answer reads)
* modal exponential X = exp(-k0 d q)                                 (modal_gradient.py:344-427)
* H-field modes   V = Omega_R W diag(1/q), the s/p rotation          (solve_2d.py:2445-2616)
* branch          q = mode_q(w), dq/dw = 1/(2q)                      (conventions.py:186-249)
* eigen-solve     dA = W^-H (diag(dw) + F o (W^H dW)) W^H with F_ij = (w_j - w_i)/(|w_j - w_i|^2 +
                  eps), eps = (n u max|w|)^2 — the Lorentzian-broadened reciprocal gap; the loss is
                  invariant to eigenvector scaling, so no normalisation term enters
* layer operator  Omega^2 from epx, epy, epz_i and the order wavevectors (solve_2d.py:2377-2418)
* Li's rules      outer inverse, block-Toeplitz gather, staircase series (an exact corrected DFT,
                  linear in the raster), inner Toeplitz inverses, 1/eps  (factorization.py:289-671)

With ``impl='gb300'`` every stage and every reverse pass runs on the library's kernels through
its C ABI: wb_assemble_li, wb_layer_modes and wb_smm_solve forward, then wb_smm_solve_vjp,
wb_layer_modes_vjp and wb_assemble_li_vjp (csrc/wb_vjp.h: the same formulas as the functions
below, batched over the wavelengths of a chunk). ``impl='torch'`` evaluates the formulas below
in torch, stage by stage and one wavelength at a time; it is the restatement the kernels are
held to and what the CPU tests check against finite differences. The wavelength gradient (a
forward tangent) runs the torch restatement over the kernels' stage-A slots and eigenpairs.
"""
import math

import numpy as np
import torch

PI = math.pi


# ----------------------------------------------------------------------------- utilities

def _eye(n, dtype, device):
    return torch.eye(n, dtype=dtype, device=device)


def _H(A):
    return A.conj().transpose(-1, -2)


def _toeplitz_index(h, device):
    r = torch.arange(2 * h + 1, device=device)
    return (r[:, None] - r[None, :] + 2 * h)


def series_matrix(npts, h, dtype=torch.complex128, device='cpu'):
    """W[k, j] with coefficient_k = sum_j W[k, j] a_j: the exact staircase series of
    factorization.py:289-440 (corrected DFT; the a0-subtracted spelling is the same map)."""
    k = torch.arange(-2 * h, 2 * h + 1, dtype=torch.float64, device=device)
    j = torch.arange(npts, dtype=torch.float64, device=device)
    t = k / npts
    sinc = torch.where(t == 0, torch.ones_like(t), torch.sin(PI * t) / torch.where(t == 0, torch.ones_like(t), PI * t))
    corr = sinc * torch.exp(-1j * PI * k.to(dtype) / npts)
    ph = torch.exp(-2j * PI * (k[:, None] * j[None, :] % npts).to(dtype) / npts)
    return (corr[:, None] * ph / npts).to(dtype)


def bttb(coef2, hu, hv):
    """conv[(r,m),(c,m')] = coef2[r-c+2hv, m-m'+2hu]; coef2 (..., 4hv+1, 4hu+1)."""
    iv = _toeplitz_index(hv, coef2.device)
    iu = _toeplitz_index(hu, coef2.device)
    nv, nu = 2 * hv + 1, 2 * hu + 1
    blocks = coef2[..., iv[:, :, None, None], iu[None, None, :, :]]      # (.., r, c, m, m')
    return blocks.permute(*range(blocks.dim() - 4), -4, -2, -3, -1).reshape(*coef2.shape[:-2], nv * nu, nv * nu)


def bttb_adjoint(G, hu, hv):
    """Adjoint of :func:`bttb`: scatter-add G[(r,m),(c,m')] into coef2[r-c+2hv, m-m'+2hu]."""
    nv, nu = 2 * hv + 1, 2 * hu + 1
    g = G.reshape(*G.shape[:-2], nv, nu, nv, nu).permute(*range(G.dim() - 2), -4, -2, -3, -1)   # r, c, m, m'
    iv = _toeplitz_index(hv, G.device)
    iu = _toeplitz_index(hu, G.device)
    flat = (iv[:, :, None, None] * (4 * hu + 1) + iu[None, None, :, :]).reshape(-1)
    out = torch.zeros(*G.shape[:-2], (4 * hv + 1) * (4 * hu + 1), dtype=G.dtype, device=G.device)
    out.index_add_(out.dim() - 1, flat, g.reshape(*G.shape[:-2], -1))
    return out.reshape(*G.shape[:-2], 4 * hv + 1, 4 * hu + 1)


# ------------------------------------------------------------------- stage A in torch

def nested_torch(grid, hu, hv, invert_outer):
    """``T_u([T_v(grid)]^-1)`` (optionally inverted) and what its reverse pass needs."""
    ny, nx = grid.shape
    nv, nu = 2 * hv + 1, 2 * hu + 1
    Sv = series_matrix(ny, hv, device=grid.device)                # (4hv+1, ny)
    Su = series_matrix(nx, hu, device=grid.device)                # (4hu+1, nx)
    cv = (Sv @ grid).T                                            # (nx, 4hv+1)
    iv = _toeplitz_index(hv, grid.device)
    Tv = cv[:, iv]                                                # (nx, nv, nv)
    inner = torch.linalg.inv(Tv)
    ent = inner.reshape(nx, nv * nv).T                            # ((r,c), x)
    cu = ent @ Su.T                                               # ((r,c), 4hu+1)
    iu = _toeplitz_index(hu, grid.device)
    outer = cu.reshape(nv, nv, 4 * hu + 1)[:, :, iu]              # (r, c, m, m')
    P = outer.permute(0, 2, 1, 3).reshape(nv * nu, nv * nu)
    out = torch.linalg.inv(P) if invert_outer else P
    return out, dict(Sv=Sv, Su=Su, inner=inner, out=out)


def nested_torch_adjoint(Gout, hu, hv, invert_outer, saved):
    """Reverse pass of :func:`nested_torch` -> cotangent of the grid (complex)."""
    nv, nu = 2 * hv + 1, 2 * hu + 1
    if invert_outer:
        Y = saved['out']
        GP = -_H(Y) @ Gout @ _H(Y)
    else:
        GP = Gout
    g = GP.reshape(nv, nu, nv, nu).permute(0, 2, 1, 3)          # (r, c, m, m')
    iu = _toeplitz_index(hu, GP.device)
    gcu = torch.zeros(nv, nv, 4 * hu + 1, dtype=GP.dtype, device=GP.device)
    gcu.index_add_(2, iu.reshape(-1), g.reshape(nv, nv, nu * nu))
    gcu = gcu.reshape(nv * nv, 4 * hu + 1)
    Su, Sv, inner = saved['Su'], saved['Sv'], saved['inner']
    gent = gcu @ Su.conj()                                        # ((r,c), x)
    ginner = gent.T.reshape(-1, nv, nv)
    gTv = -_H(inner) @ ginner @ _H(inner)                         # (nx, nv, nv)
    iv = _toeplitz_index(hv, GP.device)
    gcv = torch.zeros(gTv.shape[0], 4 * hv + 1, dtype=GP.dtype, device=GP.device)
    gcv.index_add_(1, iv.reshape(-1), gTv.reshape(gTv.shape[0], -1))
    return Sv.conj().T @ gcv.T                                    # (ny, nx)


def li_conv_torch(eps, hu, hv):
    """One layer's (epx, epy, epz_i) in torch, with the state its reverse pass needs."""
    eps = eps.to(torch.complex128)
    epx, sx = nested_torch(eps, hu, hv, True)
    epy, sy = nested_torch(1.0 / eps, hu, hv, False)
    ny, nx = eps.shape
    Sv = series_matrix(ny, hv, device=eps.device)
    Su = series_matrix(nx, hu, device=eps.device)
    c2 = Sv @ eps @ Su.T                                          # (4hv+1, 4hu+1)
    C = bttb(c2, hu, hv)
    epz_i = torch.linalg.inv(C)
    return (epx, epy, epz_i), dict(sx=sx, sy=sy, Sv=Sv, Su=Su, epz_i=epz_i, eps=eps)


def li_conv_adjoint(g, hu, hv, saved):
    """Cotangent of one raster from cotangents (gepx, gepy, gepz) of its slots."""
    gepx, gepy, gepz = g
    eps = saved['eps']
    ge = nested_torch_adjoint(gepx, hu, hv, True, saved['sx'])
    ginv = nested_torch_adjoint(gepy, hu, hv, False, saved['sy'])
    ge = ge + (-1.0 / eps ** 2).conj() * ginv
    Y = saved['epz_i']
    gC = -_H(Y) @ gepz @ _H(Y)
    gc2 = bttb_adjoint(gC, hu, hv)
    ge = ge + saved['Sv'].conj().T @ gc2 @ saved['Su'].conj()
    return ge


# ---------------------------------------------------------------- stage B pieces in torch

def layer_operator_torch(kx, ky, epx, epy, epz):
    """Omega^2 and Omega_R of solve_2d.py:2377-2418 (epxy = epyx = 0)."""
    N = kx.shape[0]
    I = _eye(N, epx.dtype, epx.device)
    kxc, kyc = kx.to(epx.dtype), ky.to(epx.dtype)
    Bm = kxc[:, None] * epz * kxc[None, :] - I
    Dm = kyc[:, None] * epz * kyc[None, :] - I
    Cc = kxc[:, None] * epz * kyc[None, :]
    Em = kyc[:, None] * epz * kxc[None, :]
    om2 = torch.cat([torch.cat([torch.diag(kyc * kyc) + Bm @ epx, Cc @ epy - torch.diag(kxc * kyc)], 1),
                     torch.cat([Em @ epx - torch.diag(kyc * kxc), torch.diag(kxc * kxc) + Dm @ epy], 1)], 0)
    omr = torch.cat([torch.cat([-torch.diag(kxc * kyc), torch.diag(kxc * kxc) - epy], 1),
                     torch.cat([epx - torch.diag(kyc * kyc), torch.diag(kyc * kxc)], 1)], 0)
    return om2, omr, dict(Bm=Bm, Dm=Dm, Cc=Cc, Em=Em, kx=kxc, ky=kyc, epx=epx, epy=epy)


def layer_operator_adjoint(G2, GR, saved):
    """Cotangents of (epx, epy, epz_i) from those of Omega^2 (G2) and Omega_R (GR)."""
    N = saved['kx'].shape[0]
    G11, G12, G21, G22 = G2[:N, :N], G2[:N, N:], G2[N:, :N], G2[N:, N:]
    epx, epy = saved['epx'], saved['epy']
    gepx = _H(saved['Bm']) @ G11 + _H(saved['Em']) @ G21 + GR[N:, :N]
    gepy = _H(saved['Cc']) @ G12 + _H(saved['Dm']) @ G22 - GR[:N, N:]
    gB, gC, gE, gD = G11 @ _H(epx), G12 @ _H(epy), G21 @ _H(epx), G22 @ _H(epy)
    kx, ky = saved['kx'], saved['ky']          # real
    gepz = (kx[:, None] * gB * kx[None, :] + kx[:, None] * gC * ky[None, :]
            + ky[:, None] * gE * kx[None, :] + ky[:, None] * gD * ky[None, :])
    return gepx, gepy, gepz


def mode_q_torch(w):
    v = torch.sqrt(w)
    flip = torch.where(v.real.abs() > 1e-12, v.real < 0, v.imag > 0)
    return torch.where(flip, -v, v)


def eig_adjoint(A_shape_n, w, W, gw, gW):
    """Cotangent of A from those of its eigenvalues w and (scale-free) eigenvectors W, with the
    broadened reciprocal gap F_ij = (w_j - w_i)/(|w_j - w_i|^2 + eps), eps = (n u max|w|)^2."""
    n = A_shape_n
    d = w[None, :] - w[:, None]                                  # d_ij = w_j - w_i
    scale = w.abs().max().clamp_min(1e-300)
    eps = (n * 2.220446049250313e-16 * scale) ** 2
    F = d / (d.abs() ** 2 + eps)
    F.fill_diagonal_(0)
    inner = torch.diag(gw) + F * (_H(W) @ gW)
    return torch.linalg.solve(_H(W), inner @ _H(W))


# ----------------------------------------------------------------- per-solve port data

def ports(wavelength, period, theta, phi, eps_top, eps_bot, hu, hv, device):
    """The per-solve vectors of the ports kernel (wb_solve.cu), in torch, FP64."""
    nu, nv = 2 * hu + 1, 2 * hv + 1
    N = nu * nv
    index = math.sqrt(float(np.real(eps_top)))
    kix = index * math.sin(theta) * math.cos(phi)
    kiy = index * math.sin(theta) * math.sin(phi)
    u = torch.arange(N, device=device) % nu - hu
    v = torch.arange(N, device=device) // nu - hv
    kx = kix + u.double() * (wavelength / period[0])
    ky = kiy + v.double() * (wavelength / period[1])
    vphi = torch.where(kx == 0,
                       torch.where(ky == 0, torch.full_like(kx, math.atan(math.sin(phi) / math.cos(phi)) + (PI if math.cos(phi) < 0 else 0.0)),
                                   torch.where(ky < 0, torch.full_like(kx, -PI / 2), torch.full_like(kx, PI / 2)) - kx / torch.where(ky == 0, torch.ones_like(ky), ky)),
                       torch.atan(ky / torch.where(kx == 0, torch.ones_like(kx), kx)) + PI * (kx < 0).double())
    c, s = torch.cos(vphi), torch.sin(vphi)
    et, eb = complex(eps_top), complex(eps_bot)
    nt, nb = np.sqrt(et), np.sqrt(eb)
    kpar = (kx * kx + ky * ky).to(torch.complex128)

    def kz(n2):
        z = torch.sqrt(n2 - kpar)
        return torch.where((z.real + z.imag) < 0, -z, z)
    kzt, kzb = kz(nt * nt), kz(nb * nb)
    y = torch.sqrt(1 + kx * kx + ky * ky).to(torch.complex128)
    one = torch.ones(N, dtype=torch.complex128, device=device)
    wg = torch.cat([one, -1j * y]); vg = torch.cat([-1j * y, one])
    wt = torch.cat([one, -1j * kzt / et]); vt = torch.cat([-1j * kzt, one])
    wb = torch.cat([one, -1j * kzb / eb]); vb = torch.cat([-1j * kzb, one])
    At, Bt = wt / wg + vt / vg, wt / wg - vt / vg
    Ab, Bb = wb / wg + vb / vg, wb / wg - vb / vg
    return dict(kx=kx, ky=ky, c=c, s=s, kzt=kzt, kzb=kzb, wg=wg, vg=vg, nt=nt, nb=nb, et=et, eb=eb,
                r11=-Bt / At, r12=2 / At, r21=0.5 * (At - Bt * Bt / At), r22=Bt / At, t11=Bb / Ab, t21=2 / Ab)


# ------------------------------------------------------------------ cascade forward/back

def cascade_forward(bW, bV, X, pv, C):
    """Bottom-up reflections and the top-down pass (wb_solve.cu stage C) for one solve.
    bW, bV: lists of (n, n); X: list of (n,); C: (n, 3) incidence columns."""
    L = len(bW)
    n = bW[0].shape[0]
    I = _eye(n, bW[0].dtype, bW[0].device)
    wg, vg = pv['wg'], pv['vg']
    Rk = [None] * (L + 1)
    Rk[L] = torch.diag(pv['t11'])
    st = [None] * L
    for l in range(L - 1, -1, -1):
        Rb = Rk[l + 1]
        U1 = wg[:, None] * (I + Rb)
        U2 = vg[:, None] * (I - Rb)
        P1 = torch.linalg.solve(bW[l], U1)
        P2 = torch.linalg.solve(bV[l], U2)
        M, Nm = P1 + P2, P1 - P2
        rb = torch.linalg.solve(M.T, Nm.T).T                       # Nm M^-1
        rt = X[l][:, None] * rb * X[l][None, :]
        X1 = torch.linalg.solve(bW[l].T, (I - rt).T).T              # (I - rt) bW^-1
        X2 = torch.linalg.solve(bV[l].T, (I + rt).T).T
        A = X1 * wg[None, :] + X2 * vg[None, :]
        Bt = -X1 * wg[None, :] + X2 * vg[None, :]
        Rk[l] = torch.linalg.solve(A, Bt)
        st[l] = dict(P1=P1, P2=P2, M=M, rb=rb, X1=X1, X2=X2, A=A, Rb=Rb)
    G0 = I - pv['r22'][:, None] * Rk[0]
    g = [None] * (L + 1)
    g[0] = torch.linalg.solve(G0, pv['r21'][:, None] * C)
    h0 = Rk[0] @ g[0]
    cref = pv['r11'][:, None] * C + pv['r12'][:, None] * h0
    td = []
    for l in range(L):
        h = h0 if l == 0 else Rk[l] @ g[l]
        b1 = torch.linalg.solve(bW[l], wg[:, None] * (g[l] + h))
        b2 = torch.linalg.solve(bV[l], vg[:, None] * (g[l] - h))
        e = X[l][:, None] * (b1 + b2)
        g[l + 1] = torch.linalg.solve(st[l]['M'], e)
        td.append(dict(h=h, b1=b1, b2=b2))
    ctrn = pv['t21'][:, None] * g[L]
    return cref, ctrn, dict(Rk=Rk, st=st, g=g, td=td, G0=G0, bW=bW, bV=bV, X=X)


def cascade_adjoint(gcref, gctrn, pv, sv):
    """Reverse pass of :func:`cascade_forward`: cotangents of bW, bV (lists) and X (list)."""
    Rk, st, g, td, bW, bV, X = sv['Rk'], sv['st'], sv['g'], sv['td'], sv['bW'], sv['bV'], sv['X']
    L = len(bW)
    wg, vg = pv['wg'], pv['vg']
    gbW = [torch.zeros_like(b) for b in bW]
    gbV = [torch.zeros_like(b) for b in bV]
    gX = [torch.zeros_like(x) for x in X]
    gM = [None] * L
    gR = [None] * (L + 1)
    gg = pv['t21'].conj()[:, None] * gctrn
    gh0 = None
    for l in range(L - 1, -1, -1):
        M = st[l]['M']
        ge = torch.linalg.solve(_H(M), gg)
        gM[l] = -ge @ _H(g[l + 1])
        bsum = td[l]['b1'] + td[l]['b2']
        gX[l] = gX[l] + (bsum.conj() * ge).sum(dim=1)
        gb = X[l].conj()[:, None] * ge
        ga1 = torch.linalg.solve(_H(bW[l]), gb)
        gbW[l] = gbW[l] - ga1 @ _H(td[l]['b1'])
        ga2 = torch.linalg.solve(_H(bV[l]), gb)
        gbV[l] = gbV[l] - ga2 @ _H(td[l]['b2'])
        gga = wg.conj()[:, None] * ga1
        ggb = vg.conj()[:, None] * ga2
        gl = gga + ggb
        gh = gga - ggb
        if l == 0:
            gh0 = gh
        else:
            h_g = g[l]
            gR[l] = gh @ _H(h_g)
            gl = gl + _H(Rk[l]) @ gh
        gg = gl
    # c_ref = r11 C + r12 h0, h0 = R0 g0
    gh0 = gh0 + pv['r12'].conj()[:, None] * gcref
    gR0 = gh0 @ _H(g[0])
    gg0 = gg + _H(Rk[0]) @ gh0
    # g0 = G0^-1 (r21 C), G0 = I - r22 R0
    gk = torch.linalg.solve(_H(sv['G0']), gg0)
    gG0 = -gk @ _H(g[0])
    gR0 = gR0 - pv['r22'].conj()[:, None] * gG0
    gR[0] = gR0
    # bottom-up reflections, top layer first
    for l in range(L):
        s_ = st[l]
        gRl = gR[l]
        A, Rl = s_['A'], Rk[l]
        gBt = torch.linalg.solve(_H(A), gRl)
        gA = -gBt @ _H(Rl)
        gX1 = (gA - gBt) * wg.conj()[None, :]
        gX2 = (gA + gBt) * vg.conj()[None, :]
        K1 = torch.linalg.solve(bW[l].conj(), gX1.T).T              # gX1 bW^-H
        K2 = torch.linalg.solve(bV[l].conj(), gX2.T).T
        gbW[l] = gbW[l] - _H(s_['X1']) @ K1
        gbV[l] = gbV[l] - _H(s_['X2']) @ K2
        grt = K2 - K1
        rb, Xl = s_['rb'], X[l]
        grb = Xl.conj()[:, None] * grt * Xl.conj()[None, :]
        gX[l] = gX[l] + (grt * (rb * Xl[None, :]).conj()).sum(dim=1) + (grt * (Xl[:, None] * rb).conj()).sum(dim=0)
        M = s_['M']
        gNm = torch.linalg.solve(M.conj(), grb.T).T                  # grb M^-H
        gMl = -_H(rb) @ gNm + gM[l]
        gP1, gP2 = gMl + gNm, gMl - gNm
        gU1 = torch.linalg.solve(_H(bW[l]), gP1)
        gbW[l] = gbW[l] - gU1 @ _H(s_['P1'])
        gU2 = torch.linalg.solve(_H(bV[l]), gP2)
        gbV[l] = gbV[l] - gU2 @ _H(s_['P2'])
        gRb = wg.conj()[:, None] * gU1 - vg.conj()[:, None] * gU2
        if l + 1 < L:
            gR[l + 1] = gR[l + 1] + gRb
    return gbW, gbV, gX


# ----------------------------------------------------------------------- full solve

def _efficiency_weights(pv, pol, N):
    kzs = pv['kzt'][N // 2]
    s_power = kzs.real
    p_power = abs(pv['nt']) ** 2 * (kzs / pv['et']).real
    den = abs(pol[0]) ** 2 * s_power + abs(pol[1]) ** 2 * p_power
    wr = torch.cat([pv['kzt'].real, (pv['kzt'] / pv['et']).real]) / den
    wt = torch.cat([pv['kzb'].real, (pv['kzb'] / pv['eb']).real]) / den
    return wr, wt


def _incidence(pv, pol, N, device):
    C = torch.zeros(2 * N, 1, dtype=torch.complex128, device=device)
    C[N // 2, 0] = complex(pol[0])
    C[N + N // 2, 0] = -1j * pv['nt'] * complex(pol[1])
    return C


def efficiencies(cref, ctrn, wr, wt, N):
    """Per-order R and T of the given column (efficiency_kernel, wb_solve.cu)."""
    a = (cref[:, 0].abs() ** 2) * wr
    b = (ctrn[:, 0].abs() ** 2) * wt
    return a[:N] + a[N:], b[:N] + b[N:]


# ------------------------------------------------------------ d loss / d wavelength

_PV_KEYS = ('kx', 'ky', 'c', 's', 'kzt', 'kzb', 'wg', 'vg', 'r11', 'r12', 'r21', 'r22', 't11', 't21')


def _rotate(W, V, c, s, N):
    """The s/p rotation of a layer's Cartesian modes (sp_rotate_kernel)."""
    W1, W2, V1, V2 = W[:N], W[N:], V[:N], V[N:]
    bw = torch.cat([c[:, None] * W2 - s[:, None] * W1, c[:, None] * W1 + s[:, None] * W2], 0)
    bv = torch.cat([c[:, None] * V1 + s[:, None] * V2, c[:, None] * V2 - s[:, None] * V1], 0)
    return bw, bv


def eig_tangent(w, W, dA):
    """Tangents of the eigenvalues and (scale-free) eigenvectors of A along dA: with
    E = W^-1 dA W, dw = diag(E) and dW = W C, C_ij = E_ij / (w_j - w_i) off the diagonal, the
    reciprocal gap broadened as in :func:`eig_adjoint` (whose F is this one's conjugate)."""
    n = w.shape[0]
    E = torch.linalg.solve(W, dA @ W)
    d = w[None, :] - w[:, None]
    scale = w.abs().max().clamp_min(1e-300)
    eps = (n * 2.220446049250313e-16 * scale) ** 2
    G = d.conj() / (d.abs() ** 2 + eps)
    G.fill_diagonal_(0)
    return torch.diagonal(E).clone(), W @ (G * E)


def wavelength_tangent(*args):
    """:func:`_wavelength_tangent`, quiet about torch's own deprecation notices from inside
    ``torch.func``."""
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter('ignore', DeprecationWarning)
        return _wavelength_tangent(*args)


def _wavelength_tangent(lam, period, theta, phi, eps_top, eps_bot, hu, hv, conv, thickness, per_layer, pol,
                        wR, wT, device):
    """``d loss / d wavelength`` of one solve by a forward tangent: the wavelength moves k0
    (``d k0 = -k0 / lam``) and every order's in-plane wavevector (``d kx = u / Lx``,
    ``d ky = v / Ly``), hence the ports, each layer's operator, its eigenpairs (:func:`eig_tangent`),
    ``q``, ``V``, the s/p rotation and ``X = exp(-k0 d q)``, and through the cascade the
    efficiencies. The pure-torch pieces are differentiated exactly by ``torch.func.jvp``."""
    from torch.func import jvp
    N = (2 * hu + 1) * (2 * hv + 1)
    n = 2 * N
    lam_t = torch.tensor(float(lam), dtype=torch.float64, device=device)
    one = torch.ones((), dtype=torch.float64, device=device)

    def port_vectors(l):
        pv = ports(l, period, theta, phi, eps_top, eps_bot, hu, hv, device)
        return tuple(pv[k] for k in _PV_KEYS)

    pv_vals, pv_tans = jvp(port_vectors, (lam_t,), (one,))
    pv0 = ports(float(lam), period, theta, phi, eps_top, eps_bot, hu, hv, device)
    k0 = 2 * PI / float(lam)
    dk0 = -k0 / float(lam)
    kx, ky = pv_vals[0], pv_vals[1]
    dkx, dky = pv_tans[0], pv_tans[1]
    c, s, dc, ds = pv_vals[2], pv_vals[3], pv_tans[2], pv_tans[3]
    bWs, bVs, Xs, dbWs, dbVs, dXs = [], [], [], [], [], []
    for l, p in enumerate(per_layer):
        epx, epy, epz = conv[l]
        (om2, omr, _), (dom2, domr, _) = jvp(lambda a, b: layer_operator_torch(a, b, epx, epy, epz), (kx, ky),
                                             (dkx, dky))
        w, W, q = p['w'], p['W'], p['q']
        dw, dW = eig_tangent(w, W, dom2)
        dq = dw / (2.0 * q)
        V = (omr @ W) / q[None, :]
        dV = (domr @ W + omr @ dW) / q[None, :] - (omr @ W) * (dq / q ** 2)[None, :]
        (bw, bv), (dbw, dbv) = jvp(lambda W_, V_, c_, s_: _rotate(W_, V_, c_, s_, N), (W, V, c, s), (dW, dV, dc, ds))
        d = float(thickness[l])
        X = torch.exp(-k0 * d * q)
        dX = X * (-d) * (dk0 * q + k0 * dq)
        bWs.append(bw); bVs.append(bv); Xs.append(X)
        dbWs.append(dbw); dbVs.append(dbv); dXs.append(dX)
    C = _incidence(pv0, pol, N, device)
    wR_t = torch.as_tensor(wR, dtype=torch.float64, device=device)
    wT_t = torch.as_tensor(wT, dtype=torch.float64, device=device)

    def loss_of(bWl, bVl, Xl, pvt):
        pv = dict(pv0)
        pv.update(zip(_PV_KEYS, pvt))
        cref, ctrn, _ = cascade_forward(list(bWl), list(bVl), list(Xl), pv, C)
        wr, wt = _efficiency_weights(pv, pol, N)
        a = (cref[:, 0] * cref[:, 0].conj()).real * wr
        b = (ctrn[:, 0] * ctrn[:, 0].conj()).real * wt
        return (wR_t * (a[:N] + a[N:])).sum() + (wT_t * (b[:N] + b[N:])).sum()

    _, dloss = jvp(loss_of, (tuple(bWs), tuple(bVs), tuple(Xs), tuple(pv_vals)),
                   (tuple(dbWs), tuple(dbVs), tuple(dXs), tuple(pv_tans)))
    return float(dloss)


def _stage_b_batch(impl, conv, pvs, L, hu, hv, cs=None):
    """Eigenpairs of every (wavelength, layer) pair: one wb_layer_modes launch on the CUDA
    kernels (gb300) or torch.linalg.eig (torch reference). Returns w (P, n), W (P, n, n)."""
    B = len(pvs)
    if impl == 'gb300':
        from . import engine
        kx = torch.stack([pv['kx'] for pv in pvs for _ in range(L)]).cpu().numpy()
        ky = torch.stack([pv['ky'] for pv in pvs for _ in range(L)]).cpu().numpy()
        pl = np.tile(np.arange(L), B)
        w, q, W, V, st = engine.layer_modes(cs, pl, kx, ky)
        if int((st.cpu().numpy() & 2).sum()):
            raise RuntimeError('the eigen-solve did not converge')
        return w, W.contiguous()
    ws, Ws = [], []
    for pv in pvs:
        for l in range(L):
            om2, _, _ = layer_operator_torch(pv['kx'], pv['ky'], *conv[l])
            w, W = torch.linalg.eig(om2)
            ws.append(w)
            Ws.append(W / torch.linalg.vector_norm(W, dim=0, keepdim=True))
    return torch.stack(ws), torch.stack(Ws)


def _chunk_size(L, n, budget, device):
    """Wavelengths per stage-B chunk: the eigenpairs and the reverse pass's per-layer temporaries
    (about 8 complex n x n matrices per layer) of one chunk fit `budget` bytes (default: a quarter
    of the free device memory; unbounded on the CPU)."""
    per = 8 * 16 * n * n * L
    if budget is None:
        if torch.device(device).type != 'cuda':
            return None
        budget = torch.cuda.mem_get_info(torch.device(device))[0] // 4
    return max(1, int(budget // per))


def solve_and_grad(eps, thickness, wavelengths, period, hu, hv, weights_R, weights_T, theta=0.0, phi=0.0,
                   eps_top=1.0, eps_bot=1.0, pol=(0.0, 1.0), impl='gb300', device=None, grad=True,
                   hbm_budget=None, grad_wavelength=False, fourier_coefficients=None, modes='double'):
    """Loss = sum_b sum_i (weights_R[b, i] R[b, i] + weights_T[b, i] T[b, i]) over the given
    polarization's per-order efficiencies, and its gradients with respect to the raster
    permittivities (real part; shape of ``eps``) and the thicknesses.

    eps: (L, ny, nx) entry face first; thickness (L,); wavelengths (B,). ``eps_top`` is the lit
    half-space: a scene lit from below is its z-mirror lit from above, so pass its layers
    bottom-first with the half-spaces swapped (the gradients come back in that order).
    Returns (loss, R (B, N), T (B, N), d_loss/d_eps (L, ny, nx) real, d_loss/d_thickness (L,)).

    The eigenpairs are computed for a chunk of wavelengths at a time, sized by ``hbm_budget``
    (bytes), and dropped after the chunk's forward and reverse passes: however many wavelengths,
    no more than one chunk's modes are resident.

    With ``grad_wavelength`` a sixth value is returned: ``d loss / d wavelength`` (B,), each
    wavelength's own term by a forward tangent (:func:`wavelength_tangent`).

    ``modes`` is the eigen-solve of the kernel path (``impl='gb300'``): ``'double'`` (FP64),
    ``'mixed'`` (FP32 refined by Newton steps on the FP64 operator) or ``'mixed_df64'`` (double-float
    on the FP32 pipes); the last two give FP64-class eigenpairs. The cascade and every reverse pass
    are FP64 in every case.

    ``fourier_coefficients`` may be ``'sampled'`` or ``'integrated'``: a differentiated raster
    keeps every pixel edge (factorization.py:3135-3150 of the reference), and over one segment
    per pixel the closed-form segment series is the exact staircase series the sampled rule
    computes, so both take the same pass.
    """
    if fourier_coefficients not in (None, 'sampled', 'integrated'):
        raise ValueError("fourier_coefficients must be 'sampled' or 'integrated'")
    device = device or ('cuda' if impl == 'gb300' else 'cpu')
    eps = torch.as_tensor(eps, dtype=torch.complex128, device=device)
    if impl == 'gb300' and not grad_wavelength:
        return _solve_and_grad_kernels(eps, thickness, wavelengths, period, hu, hv, weights_R, weights_T, theta, phi,
                                       eps_top, eps_bot, pol, device, grad, hbm_budget, modes)
    L = eps.shape[0]
    N = (2 * hu + 1) * (2 * hv + 1)
    n = 2 * N
    saved_a = [li_conv_torch(e, hu, hv) for e in eps]
    cs = None
    if impl == 'gb300':
        from . import engine
        cs = engine.assemble(eps, hu, hv)                        # stage A on the CUDA kernels
        conv = [tuple(cs.slot(k)[i].contiguous() for k in range(3)) for i in range(L)]
    else:
        conv = [sa[0] for sa in saved_a]
    wls = [float(v) for v in np.atleast_1d(wavelengths)]
    pvs = [ports(lam, period, theta, phi, eps_top, eps_bot, hu, hv, device) for lam in wls]
    chunk = _chunk_size(L, n, hbm_budget, device) or len(wls)
    w_all = W_all = None
    g_conv = [[torch.zeros(N, N, dtype=torch.complex128, device=device) for _ in range(3)] for _ in range(L)]
    g_th = torch.zeros(L, dtype=torch.float64, device=device)
    loss = 0.0
    Rs, Ts = [], []
    g_wl = []
    for b, lam in enumerate(wls):
        if b % chunk == 0:
            w_all = W_all = None
            w_all, W_all = _stage_b_batch(impl, conv, pvs[b:b + chunk], L, hu, hv, cs)
        pv = pvs[b]
        k0 = 2 * PI / lam
        bW, bV, Xs, per_layer = [], [], [], []
        for l in range(L):
            om2, omr, so = layer_operator_torch(pv['kx'], pv['ky'], *conv[l])
            w, W = w_all[(b % chunk) * L + l], W_all[(b % chunk) * L + l]
            q = mode_q_torch(w)
            V = (omr @ W) / q[None, :]
            c, s = pv['c'], pv['s']
            W1, W2, V1, V2 = W[:N], W[N:], V[:N], V[N:]
            bw = torch.cat([c[:, None] * W2 - s[:, None] * W1, c[:, None] * W1 + s[:, None] * W2], 0)
            bv = torch.cat([c[:, None] * V1 + s[:, None] * V2, c[:, None] * V2 - s[:, None] * V1], 0)
            X = torch.exp(-k0 * float(thickness[l]) * q)
            bW.append(bw); bV.append(bv); Xs.append(X)
            per_layer.append(dict(omr=omr, so=so, w=w, W=W, q=q, V=V))
        C = _incidence(pv, pol, N, device)
        cref, ctrn, sv = cascade_forward(bW, bV, Xs, pv, C)
        wr, wt = _efficiency_weights(pv, pol, N)
        Rb, Tb = efficiencies(cref, ctrn, wr, wt, N)
        wR = torch.as_tensor(weights_R[b], dtype=torch.float64, device=device)
        wT = torch.as_tensor(weights_T[b], dtype=torch.float64, device=device)
        loss += float((wR * Rb).sum() + (wT * Tb).sum())
        Rs.append(Rb); Ts.append(Tb)
        if grad_wavelength:
            g_wl.append(wavelength_tangent(lam, period, theta, phi, eps_top, eps_bot, hu, hv, conv, thickness,
                                           per_layer, pol, weights_R[b], weights_T[b], device))
        if not grad:
            continue
        # reverse: efficiencies -> amplitudes (d|a|^2 = 2 Re(conj(a) da))
        gcref = torch.zeros_like(cref)
        gctrn = torch.zeros_like(ctrn)
        gcref[:, 0] = 2 * torch.cat([wR, wR]) * wr * cref[:, 0]
        gctrn[:, 0] = 2 * torch.cat([wT, wT]) * wt * ctrn[:, 0]
        gbW, gbV, gX = cascade_adjoint(gcref, gctrn, pv, sv)
        c, s = pv['c'], pv['s']
        for l in range(L):
            p = per_layer[l]
            # X = exp(-k0 d q)
            gq = (-k0 * float(thickness[l]) * Xs[l]).conj() * gX[l]
            g_th[l] += torch.real(((-k0 * p['q'] * Xs[l]).conj() * gX[l]).sum())
            # s/p rotation
            gb, gv = gbW[l], gbV[l]
            gW = torch.cat([-s[:, None] * gb[:N] + c[:, None] * gb[N:], c[:, None] * gb[:N] + s[:, None] * gb[N:]], 0)
            gV = torch.cat([c[:, None] * gv[:N] - s[:, None] * gv[N:], s[:, None] * gv[:N] + c[:, None] * gv[N:]], 0)
            # V = Omega_R W diag(1/q)
            iq = 1.0 / p['q']
            gW = gW + _H(p['omr']) @ (gV * iq.conj()[None, :])
            gomr = (gV * iq.conj()[None, :]) @ _H(p['W'])
            giq = ((p['omr'] @ p['W']).conj() * gV).sum(dim=0)
            gq = gq + (-(iq ** 2)).conj() * giq
            # q = mode_q(w)
            gw = (1.0 / (2.0 * p['q'])).conj() * gq
            # eigen-decomposition
            gom2 = eig_adjoint(n, p['w'], p['W'], gw, gW)
            gx, gy, gz = layer_operator_adjoint(gom2, gomr, p['so'])
            g_conv[l][0] += gx; g_conv[l][1] += gy; g_conv[l][2] += gz
    extra = (torch.tensor(g_wl, dtype=torch.float64, device=device),) if grad_wavelength else ()
    if not grad:
        return (loss, torch.stack(Rs), torch.stack(Ts), None, None) + extra
    g_eps = torch.stack([li_conv_adjoint(g_conv[l], hu, hv, saved_a[l][1]) for l in range(L)])
    return (loss, torch.stack(Rs), torch.stack(Ts), g_eps.real, g_th) + extra


def _solve_and_grad_kernels(eps, thickness, wavelengths, period, hu, hv, weights_R, weights_T, theta, phi, eps_top,
                            eps_bot, pol, device, grad, hbm_budget, modes='double'):
    """:func:`solve_and_grad` with every stage and every reverse pass on the library's kernels:
    wb_assemble_li, then per chunk of wavelengths wb_layer_modes (FP64), wb_smm_solve (FP64),
    wb_smm_solve_vjp and wb_layer_modes_vjp, and finally wb_assemble_li_vjp. The chunk's modes
    are dropped after its reverse pass."""
    from . import engine
    L = eps.shape[0]
    N = (2 * hu + 1) * (2 * hv + 1)
    n = 2 * N
    cs = engine.assemble(eps, hu, hv)
    wls = [float(v) for v in np.atleast_1d(wavelengths)]
    B = len(wls)
    th = [float(t) for t in np.asarray(thickness, dtype=np.float64).reshape(L)]
    chunk = _chunk_size(L, n, hbm_budget, device) or B
    wR_all = np.asarray(weights_R, dtype=np.float64).reshape(B, N)
    wT_all = np.asarray(weights_T, dtype=np.float64).reshape(B, N)
    g_conv = torch.zeros_like(cs.buf)
    g_th = torch.zeros(L, dtype=torch.float64, device=device)
    loss = 0.0
    Rs, Ts = [], []
    for b0 in range(0, B, chunk):
        lam = wls[b0:b0 + chunk]
        Bc = len(lam)
        pvs = [ports(x, period, theta, phi, eps_top, eps_bot, hu, hv, device) for x in lam]
        kx = torch.stack([pv['kx'] for pv in pvs for _ in range(L)])
        ky = torch.stack([pv['ky'] for pv in pvs for _ in range(L)])
        pl = np.tile(np.arange(L), Bc)
        w, q, W, V, st = engine.layer_modes(cs, pl, kx, ky, precision=modes)
        if int((st.cpu().numpy() & 2).sum()):
            raise RuntimeError('the eigen-solve did not converge')
        inp = engine.BatchInputs([list(range(L))] * Bc, [th] * Bc, lam, [list(period)] * Bc, [theta] * Bc,
                                 [phi] * Bc, [complex(eps_top)] * Bc, [complex(eps_bot)] * Bc, [list(pol)] * Bc,
                                 device=device)
        R, T, st = engine.smm_solve(W, V, q, inp, hu, hv, precision='double')
        R0, T0 = R[:, 0].reshape(Bc, N), T[:, 0].reshape(Bc, N)
        wR = torch.as_tensor(wR_all[b0:b0 + Bc], device=device)
        wT = torch.as_tensor(wT_all[b0:b0 + Bc], device=device)
        loss += float((wR * R0).sum() + (wT * T0).sum())
        Rs.append(R0); Ts.append(T0)
        if not grad:
            continue
        gR = torch.zeros((Bc, 3, N), dtype=torch.float64, device=device)
        gT = torch.zeros_like(gR)
        gR[:, 0] = wR
        gT[:, 0] = wT
        gW, gV, gq, gth, st = engine.smm_solve_vjp(W, V, q, inp, hu, hv, gR, gT)
        if int((st.cpu().numpy() & 1).sum()):
            raise RuntimeError('a cascade factor is singular')
        g_th += gth.sum(dim=0)
        gc, _ = engine.layer_modes_vjp(cs, pl, kx, ky, w, q, W, V, g_q=gq, g_W=gW, g_V=gV)
        g_conv += gc.buf
        del w, q, W, V, gW, gV, gq
    Rt, Tt = torch.cat(Rs), torch.cat(Ts)
    if not grad:
        return loss, Rt, Tt, None, None
    g_eps = engine.assemble_vjp(eps, cs, engine.ConvStack(g_conv, hu, hv))
    return loss, Rt, Tt, g_eps.real, g_th


class EfficiencyLoss(torch.autograd.Function):
    """``loss = sum(weights_R * R + weights_T * T)`` of a raster stack as a differentiable
    function of the (real) raster permittivities, the layer thicknesses and the wavelengths.

    The forward runs stages A and B on the CUDA kernels and evaluates the hand-written reverse
    pass at once (one solve per wavelength; nothing but the gradients is kept for ``backward``,
    so no per-layer eigenpairs stay resident between the passes). The wavelength gradient (a
    forward tangent per wavelength) is computed only when ``wavelengths`` requires it.
    """

    @staticmethod
    def forward(ctx, eps, thickness, wavelengths, weights_R, weights_T, spec):
        want_wl = bool(ctx.needs_input_grad[2])
        out = solve_and_grad(
            eps.detach().to(torch.complex128), thickness.detach().cpu().numpy(),
            [float(v) for v in wavelengths.detach().cpu().reshape(-1)],
            spec['period'], spec['hu'], spec['hv'], weights_R.detach().cpu().numpy(),
            weights_T.detach().cpu().numpy(), theta=spec.get('theta', 0.0), phi=spec.get('phi', 0.0),
            eps_top=spec.get('eps_top', 1.0), eps_bot=spec.get('eps_bot', 1.0), pol=spec.get('pol', (0.0, 1.0)),
            impl=spec.get('impl', 'gb300'), device=eps.device, grad_wavelength=want_wl,
            fourier_coefficients=spec.get('fourier_coefficients'))
        loss, g_eps, g_th = out[0], out[3], out[4]
        g_wl = out[5].to(wavelengths.dtype).to(wavelengths.device).reshape(wavelengths.shape) if want_wl \
            else torch.zeros_like(wavelengths)
        ctx.save_for_backward(g_eps.to(eps.dtype), g_th.to(thickness.dtype).to(thickness.device), g_wl)
        ctx.want_wl = want_wl
        return torch.as_tensor(loss, dtype=torch.float64, device=eps.device)

    @staticmethod
    def backward(ctx, grad):
        g_eps, g_th, g_wl = ctx.saved_tensors
        return grad * g_eps, grad * g_th, (grad * g_wl if ctx.want_wl else None), None, None, None


def efficiency_loss(eps, thickness, weights_R, weights_T, **spec):
    """Functional form of :class:`EfficiencyLoss`; ``spec['wavelengths']`` may be a tensor that
    requires grad."""
    spec = dict(spec)
    wl = spec.pop('wavelengths')
    wl = wl if torch.is_tensor(wl) else torch.as_tensor(np.atleast_1d(wl), dtype=torch.float64)
    return EfficiencyLoss.apply(eps, thickness, wl, torch.as_tensor(weights_R), torch.as_tensor(weights_T), spec)
