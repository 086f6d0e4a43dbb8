"""Gradient check of the adjoint on the adjoint-layer workload (one 220 nm layer, a 128x128
continuous raster, orders (9, 9), 32 wavelengths over 1000-1600 nm, p incidence, objective
sum_lambda T(0,0)): times one forward+reverse pass and compares the pixel and thickness
gradients with central finite differences (step 1e-6 on 16 seeded pixels) of the same forward.

    python -m wavebit_gb300.gradcheck [--wavelengths 32] [--pixels 16] [--orders 9] [--wavelength]

``--wavelength`` also checks d loss / d wavelength of the first wavelength (its forward tangent)
against a central difference of 1e-3 nm.
"""
import argparse
import json
import time

import numpy as np
import torch

from . import adjoint as AD
from . import workloads as WL


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--wavelengths', type=int, default=32)
    ap.add_argument('--pixels', type=int, default=16)
    ap.add_argument('--orders', type=int, default=9)
    ap.add_argument('--side', type=int, default=128)
    ap.add_argument('--wavelength', action='store_true', help='check d loss / d wavelength too')
    args = ap.parse_args()
    cfg = WL.adjoint_layer(side=args.side, n_wavelengths=args.wavelengths)
    h = args.orders
    N = (2 * h + 1) ** 2
    B = len(cfg['wavelengths'])
    wR = np.zeros((B, N))
    wT = np.zeros((B, N))
    wT[:, N // 2] = 1.0                       # sum over wavelengths of T(0, 0)
    kw = dict(wavelengths=cfg['wavelengths'], period=cfg['period'], hu=h, hv=h, theta=0.0, phi=0.0,
              eps_top=cfg['eps_top'], eps_bot=cfg['eps_bot'], pol=(0.0, 1.0), impl='gb300', device='cuda')
    eps, th = cfg['eps'], cfg['thickness']
    AD.solve_and_grad(eps, th, weights_R=wR, weights_T=wT, grad=False, **kw)      # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss, R, T, g_eps, g_th = AD.solve_and_grad(eps, th, weights_R=wR, weights_T=wT, **kw)
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    rng = np.random.default_rng(16)
    step = 1e-6
    worst = 0.0
    rows = []
    for _ in range(args.pixels):
        y, x = (int(v) for v in rng.integers(0, eps.shape[1], size=2))
        ep, em = eps.copy(), eps.copy()
        ep[0, y, x] += step
        em[0, y, x] -= step
        fp = AD.solve_and_grad(ep, th, weights_R=wR, weights_T=wT, grad=False, **kw)[0]
        fm = AD.solve_and_grad(em, th, weights_R=wR, weights_T=wT, grad=False, **kw)[0]
        fd = (fp - fm) / (2 * step)
        ad = float(g_eps[0, y, x])
        worst = max(worst, abs(fd - ad) / max(abs(fd), 1e-3 * float(g_eps.abs().max())))
        rows.append((y, x, fd, ad))
    tp, tm = th.copy(), th.copy()
    tp[0] += 1e-4
    tm[0] -= 1e-4
    fd_t = (AD.solve_and_grad(eps, tp, weights_R=wR, weights_T=wT, grad=False, **kw)[0]
            - AD.solve_and_grad(eps, tm, weights_R=wR, weights_T=wT, grad=False, **kw)[0]) / 2e-4
    out = {'workload': f'adjoint_layer {args.side}x{args.side}, orders ({h},{h}), {B} wavelengths, p, sum T(0,0)',
           'loss': loss, 'grad_seconds': t_grad, 'fd_pixels': args.pixels, 'fd_step': step,
           'max_rel_err_pixels': worst, 'thickness_grad': float(g_th[0]), 'thickness_fd': fd_t,
           'thickness_rel_err': abs(fd_t - float(g_th[0])) / max(abs(fd_t), 1e-300),
           'samples': [dict(y=r[0], x=r[1], fd=r[2], adjoint=r[3]) for r in rows[:4]]}
    if args.wavelength:
        t0 = time.perf_counter()
        g_wl = AD.solve_and_grad(eps, th, weights_R=wR, weights_T=wT, grad=False, grad_wavelength=True, **kw)[5]
        torch.cuda.synchronize()
        h_wl = 1e-3
        wl0 = list(cfg['wavelengths'])

        def at(lam):
            return AD.solve_and_grad(eps, th, weights_R=wR, weights_T=wT, grad=False,
                                     **dict(kw, wavelengths=[lam] + wl0[1:]))[0]
        fd_wl = (at(wl0[0] + h_wl) - at(wl0[0] - h_wl)) / (2 * h_wl)
        out.update(wavelength_grad=float(g_wl[0]), wavelength_fd=fd_wl,
                   wavelength_rel_err=abs(fd_wl - float(g_wl[0])) / max(abs(fd_wl), 1e-300),
                   wavelength_grad_seconds=time.perf_counter() - t0)
    print(json.dumps(out))


if __name__ == '__main__':
    main()
