"""Shared case for the reverse-pass tests: a small raster stack, its forward state in torch
(slots, eigenpairs, port vectors) laid out as the C ABI takes it, and the hand-written torch
adjoint's per-stage reverse passes (wavebit_gb300/adjoint.py) to compare against.

Layouts: the library's matrices are column-major, so a torch matrix M (row-major) is passed as
M.T; batches stack along the first axis.
"""
import math

import numpy as np
import torch

from wavebit_gb300 import adjoint as A

PI = math.pi


def colmajor(M):
    """(…, r, c) row-major torch matrices -> the same matrices as column-major buffers."""
    return M.transpose(-1, -2).contiguous()


def rowmajor(buf):
    return buf.transpose(-1, -2).contiguous()


class Case:
    """L layers of an ny x nx raster, B wavelengths, orders (hu, hv); everything FP64 torch on
    `device`. Pairs are p = b * L + l."""

    def __init__(self, seed=0, L=2, ny=6, nx=8, hu=2, hv=1, wavelengths=(620.0, 710.0), period=(700.0, 650.0),
                 theta=0.25, phi=0.3, eps_top=1.0, eps_bot=2.25, pol=(0.6, 0.8), device='cpu', eps=None,
                 thickness=None, kernels=False):
        rng = np.random.default_rng(seed)
        if eps is None:
            eps = 1.0 + 11.25 / (1 + np.exp(-3 * rng.standard_normal((L, ny, nx))))
            eps = eps + 0.05j * rng.random((L, ny, nx))
        self.eps_np = np.asarray(eps, complex)
        self.L, self.ny, self.nx = self.eps_np.shape
        L = self.L
        self.th = np.asarray(thickness if thickness is not None else rng.uniform(80, 200, size=L), float)
        self.hu, self.hv = hu, hv
        self.N = (2 * hu + 1) * (2 * hv + 1)
        self.n = 2 * self.N
        self.wls = [float(x) for x in wavelengths]
        self.B = len(self.wls)
        self.period, self.theta, self.phi = period, theta, phi
        self.eps_top, self.eps_bot, self.pol = eps_top, eps_bot, pol
        self.device = device
        self.eps = torch.as_tensor(self.eps_np, device=device)
        self.saved_a = [A.li_conv_torch(e, hu, hv) for e in self.eps]
        self.pvs = [A.ports(lam, period, theta, phi, eps_top, eps_bot, hu, hv, device) for lam in self.wls]
        self.modes = []                                                  # per pair: dict(w, W, q, V, omr, so)
        self.cs = None
        if kernels:
            # slots and eigenpairs from the library's kernels (wb_assemble_li, wb_layer_modes)
            from wavebit_gb300 import engine
            self.cs = engine.assemble(self.eps, hu, hv)
            self.conv = [tuple(self.cs.slot(k)[l].contiguous() for k in range(3)) for l in range(L)]
            kx, ky = self.kxy()
            w, q, W, V, st = engine.layer_modes(self.cs, np.tile(np.arange(L), self.B), kx, ky, precision='double')
            assert int(st.abs().sum()) == 0
            for p in range(self.B * L):
                pv = self.pvs[p // L]
                _, omr, so = A.layer_operator_torch(pv['kx'], pv['ky'], *self.conv[p % L])
                self.modes.append(dict(w=w[p], W=W[p], q=q[p], V=V[p], omr=omr, so=so))
            return
        self.conv = [sa[0] for sa in self.saved_a]                       # [(epx, epy, epz)] row-major
        for pv in self.pvs:
            for l in range(L):
                om2, omr, so = A.layer_operator_torch(pv['kx'], pv['ky'], *self.conv[l])
                w, W = torch.linalg.eig(om2)
                W = W / torch.linalg.vector_norm(W, dim=0, keepdim=True)
                q = A.mode_q_torch(w)
                V = (omr @ W) / q[None, :]
                self.modes.append(dict(w=w, W=W, q=q, V=V, omr=omr, so=so))

    # ------------------------------------------------------------------ C-ABI layouts
    def conv_buf(self):
        """(L, 3, N, N) column-major slots."""
        return torch.stack([torch.stack([colmajor(m) for m in c]) for c in self.conv])

    def slot_planes(self, k):
        """(L, N, N) column-major plane of slot k."""
        return torch.stack([colmajor(c[k]) for c in self.conv])

    def pairs(self, key):
        return torch.stack([m[key] for m in self.modes])

    def kxy(self):
        kx = torch.stack([pv['kx'] for pv in self.pvs for _ in range(self.L)])
        ky = torch.stack([pv['ky'] for pv in self.pvs for _ in range(self.L)])
        return kx.contiguous(), ky.contiguous()

    def solve_arrays(self):
        dev = self.device
        B = self.B
        return dict(
            thickness=torch.tensor(np.tile(self.th, (B, 1)), dtype=torch.float64, device=dev),
            wavelength=torch.tensor(self.wls, dtype=torch.float64, device=dev),
            period=torch.tensor([list(self.period)] * B, dtype=torch.float64, device=dev),
            theta=torch.full((B,), float(self.theta), dtype=torch.float64, device=dev),
            phi=torch.full((B,), float(self.phi), dtype=torch.float64, device=dev),
            eps_top=torch.full((B,), complex(self.eps_top), dtype=torch.complex128, device=dev),
            eps_bot=torch.full((B,), complex(self.eps_bot), dtype=torch.complex128, device=dev),
            pol=torch.tensor([list(self.pol)] * B, dtype=torch.complex128, device=dev))

    def port_arrays(self):
        keys_r = ('kx', 'ky', 'c', 's')
        keys_c = ('kzt', 'kzb', 'wg', 'vg', 'r11', 'r12', 'r21', 'r22', 't11', 't21')
        out = {k: torch.stack([pv[k] for pv in self.pvs]).to(torch.float64).contiguous() for k in keys_r}
        out.update({k: torch.stack([pv[k] for pv in self.pvs]).to(torch.complex128).contiguous() for k in keys_c})
        out['nt'] = torch.tensor([complex(pv['nt']) for pv in self.pvs], dtype=torch.complex128, device=self.device)
        out['nb'] = torch.tensor([complex(pv['nb']) for pv in self.pvs], dtype=torch.complex128, device=self.device)
        return out

    # ------------------------------------------------------------------ torch reverse passes
    def stage_c_torch(self, wR, wT):
        """Cotangents of W, V (Cartesian), q per pair and of the thicknesses (B, L) for the loss
        sum_b wR[b] . R_b + wT[b] . T_b of the given polarization (adjoint.solve_and_grad's stage C)."""
        N, L = self.N, self.L
        gW, gV, gq, gth = [], [], [], torch.zeros(self.B, L, dtype=torch.float64, device=self.device)
        loss = 0.0
        for b, lam in enumerate(self.wls):
            pv = self.pvs[b]
            k0 = 2 * PI / lam
            bW, bV, Xs = [], [], []
            c, s = pv['c'], pv['s']
            for l in range(L):
                m = self.modes[b * L + l]
                bw, bv = A._rotate(m['W'], m['V'], c, s, N)
                bW.append(bw); bV.append(bv)
                Xs.append(torch.exp(-k0 * float(self.th[l]) * m['q']))
            C = A._incidence(pv, self.pol, N, self.device)
            cref, ctrn, sv = A.cascade_forward(bW, bV, Xs, pv, C)
            wr, wt = A._efficiency_weights(pv, self.pol, N)
            Rb, Tb = A.efficiencies(cref, ctrn, wr, wt, N)
            wRb = torch.as_tensor(wR[b], dtype=torch.float64, device=self.device)
            wTb = torch.as_tensor(wT[b], dtype=torch.float64, device=self.device)
            loss += float((wRb * Rb).sum() + (wTb * Tb).sum())
            gcref = torch.zeros_like(cref)
            gctrn = torch.zeros_like(ctrn)
            gcref[:, 0] = 2 * torch.cat([wRb, wRb]) * wr * cref[:, 0]
            gctrn[:, 0] = 2 * torch.cat([wTb, wTb]) * wt * ctrn[:, 0]
            gbW, gbV, gX = A.cascade_adjoint(gcref, gctrn, pv, sv)
            for l in range(L):
                m = self.modes[b * L + l]
                gq.append((-k0 * float(self.th[l]) * Xs[l]).conj() * gX[l])
                gth[b, l] = torch.real(((-k0 * m['q'] * Xs[l]).conj() * gX[l]).sum())
                gb, gv = gbW[l], gbV[l]
                gW.append(torch.cat([-s[:, None] * gb[:N] + c[:, None] * gb[N:], c[:, None] * gb[:N] + s[:, None] * gb[N:]], 0))
                gV.append(torch.cat([c[:, None] * gv[:N] - s[:, None] * gv[N:], s[:, None] * gv[:N] + c[:, None] * gv[N:]], 0))
        return loss, torch.stack(gW), torch.stack(gV), torch.stack(gq), gth

    def stage_b_torch(self, gW, gV, gq, gw=None):
        """Per-layer slot cotangents [(gepx, gepy, gepz)] (row-major) from the pairs' cotangents."""
        N, n, L = self.N, self.n, self.L
        g_conv = [[torch.zeros(N, N, dtype=torch.complex128, device=self.device) for _ in range(3)] for _ in range(L)]
        for p, m in enumerate(self.modes):
            l = p % L
            iq = 1.0 / m['q']
            gWp = gW[p] + A._H(m['omr']) @ (gV[p] * iq.conj()[None, :])
            gomr = (gV[p] * iq.conj()[None, :]) @ A._H(m['W'])
            giq = ((m['omr'] @ m['W']).conj() * gV[p]).sum(dim=0)
            gqp = gq[p] + (-(iq ** 2)).conj() * giq
            gwp = (1.0 / (2.0 * m['q'])).conj() * gqp
            if gw is not None:
                gwp = gwp + gw[p]
            gom2 = A.eig_adjoint(n, m['w'], m['W'], gwp, gWp)
            gx, gy, gz = A.layer_operator_adjoint(gom2, gomr, m['so'])
            g_conv[l][0] += gx; g_conv[l][1] += gy; g_conv[l][2] += gz
        return g_conv

    def stage_a_torch(self, g_conv):
        return torch.stack([A.li_conv_adjoint(g_conv[l], self.hu, self.hv, self.saved_a[l][1]) for l in range(self.L)])


def weights(case, seed=1):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((case.B, case.N)), rng.standard_normal((case.B, case.N))


def eff_cotangents(case, wR, wT):
    """(B, 3, N) cotangents of the entry points' R and T for the loss on the given polarization."""
    gR = np.zeros((case.B, 3, case.N)); gT = np.zeros((case.B, 3, case.N))
    gR[:, 0] = wR; gT[:, 0] = wT
    return gR, gT


def rel(a, b):
    a = a.detach().cpu() if torch.is_tensor(a) else torch.as_tensor(a)
    b = b.detach().cpu() if torch.is_tensor(b) else torch.as_tensor(b)
    return float((a - b).abs().max() / max(float(b.abs().max()), 1e-300))
