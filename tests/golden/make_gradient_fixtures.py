"""Golden gradients from the reference's PyTorch backend (its differentiable path).

Run where the reference source tree is available (read-only)::

    PYTHONPATH=tests/golden/refshim python tests/golden/make_gradient_fixtures.py --reference <root>

It writes ``ref_gradient.npz``: for each case, the reference's public ``rcwa.run(...,
backend='torch')`` on a one-layer stack whose permittivity raster and thickness are leaf tensors.
The loss is the sum over wavelengths of the (0, 0)-order transmission, p incidence, normal
incidence, and ``loss.backward()`` gives its gradients with respect to every pixel and the
thickness.

* ``small`` -- a 32x32 raster of the adjoint-layer generator (eps = 1 + 11.25 sigmoid(8 g), g
  filtered noise), orders (5, 5), 4 wavelengths over 1000-1600 nm.
* ``layer`` -- the adjoint-layer workload itself: a 128x128 raster, 220 nm, orders (9, 9),
  32 wavelengths over 1000-1600 nm.

The rasters come from ``wavebit_gb300/workloads.py``'s seeded generator and are stored with the
results. The refshim package supplies the Array-API namespaces the reference imports.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import make_fixtures as MF  # noqa: E402
from wavebit_gb300 import workloads as WL  # noqa: E402


def reference_gradient(eps2d, thickness, wavelengths, orders, period=(1000.0, 1000.0), eps_bot=2.25):
    import torch
    from wavebit import Material, Units, rcwa
    eps = torch.tensor(np.asarray(eps2d).real, dtype=torch.float64, requires_grad=True)
    th = torch.tensor(float(thickness), dtype=torch.float64, requires_grad=True)
    prob = rcwa.Problem(
        units=Units(length='nm'),
        stack=rcwa.Stack(period=period, top=Material(epsilon=1.0), bottom=Material(epsilon=eps_bot),
                         layers=(rcwa.Layer(thickness=th, epsilon=eps),)),
        excitation=rcwa.Excitation(wavelength=tuple(float(w) for w in wavelengths),
                                   sources=(rcwa.PlaneWave(polarization='p', theta=0.0, phi=0.0),)))
    res = rcwa.run(prob, numerics=rcwa.Numerics(orders=orders), backend='torch')
    hu, hv = orders
    loss = res.T[:, hv, hu].sum()
    loss.backward()
    return float(loss.detach()), eps.grad.numpy().copy(), float(th.grad), res.T.detach().numpy()


def main():
    MF.use_reference()
    out = {}
    cases = [('small', 32, 5, 4), ('layer', 128, 9, 32)]
    for name, side, h, nw in cases:
        cfg = WL.adjoint_layer(side=side, n_wavelengths=nw)
        t0 = time.time()
        loss, g_eps, g_th, T = reference_gradient(cfg['eps'][0], cfg['thickness'][0], cfg['wavelengths'], (h, h),
                                                  cfg['period'], cfg['eps_bot'])
        out[f'{name}__eps'] = cfg['eps'][0].real
        out[f'{name}__thickness'] = np.asarray(cfg['thickness'][0])
        out[f'{name}__wavelengths'] = np.asarray(cfg['wavelengths'])
        out[f'{name}__orders'] = np.asarray((h, h))
        out[f'{name}__loss'] = np.asarray(loss)
        out[f'{name}__grad_eps'] = g_eps
        out[f'{name}__grad_thickness'] = np.asarray(g_th)
        out[f'{name}__T'] = T
        print(name, 'loss', loss, 'max |grad eps|', np.abs(g_eps).max(), 'grad th', g_th,
              f'{time.time() - t0:.1f} s', flush=True)
    out['names'] = np.array([c[0] for c in cases])
    np.savez_compressed(os.path.join(HERE, 'ref_gradient.npz'), **out)
    print('ref_gradient.npz written')


if __name__ == '__main__':
    main()
