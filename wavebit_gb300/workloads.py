"""Seeded synthetic stacks with the shapes of the benchmark configurations.

No dataset is involved anywhere in this path: every workload is generated here from a fixed
seed, with the sizes, value sets and distributions the configurations state.

* ``grating_1d``  — 1 x 4 raster [1, 1, 12.25, 12.25], 300 nm, period 700 nm, orders (10, 0),
  900 nm, normal incidence, s.
* ``crossed_sweep`` — three 256 x 256 binary rasters (eps 1 / 12.25, 1-4 seeded rectangles and
  discs) of thickness U(100, 400) nm, plus a uniform eps = -20+1.5j layer of 50 nm; period
  1000 nm, substrate 2.25, orders (7, 7), 128 wavelengths over 400-1000 nm, normal incidence.
* ``mixed_sweep`` — the same generator with 4 patterned layers, orders (12, 12), 256
  wavelengths x theta in {0, 0.2, 0.4, 0.6}, phi = 0.
* ``serving_stream`` — requests with orders in {(5,5),(8,8),(11,11),(15,15)}, 1-6 layers of side
  {64,128,256}, eps in {1, 2.25, 12.25, -20+1.5j}, d in U(50, 400), wavelength U(400, 1600),
  theta U(0, pi/3), phi U(0, 2 pi), random s/p, Poisson arrival times.
"""
import math

import numpy as np


def binary_raster(rng, side, eps_hi=12.25, eps_lo=1.0, n_min=1, n_max=4):
    """``side x side`` raster of eps_lo holding 1-4 axis-aligned rectangles and discs."""
    a = np.full((side, side), eps_lo, dtype=np.complex128)
    yy, xx = np.mgrid[0:side, 0:side]
    for _ in range(int(rng.integers(n_min, n_max + 1))):
        if rng.random() < 0.5:
            h, w = (int(v) for v in rng.integers(side // 8, side // 2 + 1, size=2))
            y0, x0 = (int(v) for v in rng.integers(0, side, size=2))
            ys = (np.arange(y0, y0 + h) % side)[:, None]
            xs = (np.arange(x0, x0 + w) % side)[None, :]
            a[ys, xs] = eps_hi
        else:
            r = rng.uniform(side / 10, side / 4)
            cy, cx = rng.uniform(0, side, size=2)
            dy = np.minimum(np.abs(yy + 0.5 - cy), side - np.abs(yy + 0.5 - cy))
            dx = np.minimum(np.abs(xx + 0.5 - cx), side - np.abs(xx + 0.5 - cx))
            a[dy * dy + dx * dx < r * r] = eps_hi
    return a


def grating_1d():
    return dict(name='grating_1d', eps=np.array([[[1., 1., 12.25, 12.25]]], np.complex128),
                thickness=np.array([300.]), period=(700., 700.), orders=(10, 0),
                wavelengths=np.array([900.]), thetas=np.array([0.]), phis=np.array([0.]),
                pols=['s'], eps_top=1.0, eps_bot=2.25)


def _patterned_stack(rng, n_patterned, side, absorber):
    layers = [binary_raster(rng, side) for _ in range(n_patterned)]
    thick = list(rng.uniform(100., 400., size=n_patterned))
    if absorber:
        layers.append(np.full((side, side), -20 + 1.5j, np.complex128))
        thick.append(50.)
    return np.stack(layers), np.array(thick)


def crossed_sweep(seed=2, n_wavelengths=128):
    rng = np.random.default_rng(seed)
    eps, thick = _patterned_stack(rng, 3, 256, absorber=True)
    wl = np.linspace(400., 1000., n_wavelengths)
    return dict(name='crossed_sweep', eps=eps, thickness=thick, period=(1000., 1000.), orders=(7, 7),
                wavelengths=wl, thetas=np.zeros_like(wl), phis=np.zeros_like(wl), pols=['s', 'p'],
                eps_top=1.0, eps_bot=2.25)


def mixed_sweep(seed=3, n_wavelengths=256, thetas=(0.0, 0.2, 0.4, 0.6)):
    rng = np.random.default_rng(seed)
    eps, thick = _patterned_stack(rng, 4, 256, absorber=False)
    wl = np.linspace(400., 1000., n_wavelengths)
    W, Th = np.meshgrid(wl, np.asarray(thetas), indexing='ij')
    return dict(name='mixed_sweep', eps=eps, thickness=thick, period=(1000., 1000.), orders=(12, 12),
                wavelengths=W.reshape(-1), thetas=Th.reshape(-1), phis=np.zeros(W.size), pols=['s', 'p'],
                eps_top=1.0, eps_bot=2.25)


def adjoint_layer(seed=4, side=128, n_wavelengths=32):
    """One 220 nm layer, eps(x, y) = 1 + 11.25 sigmoid(8 g), g seeded N(0, 1) noise Gaussian-
    filtered at sigma = 4 px (periodic) and normalised to unit variance; substrate 2.25; orders
    (9, 9); wavelengths over 1000-1600 nm; normal incidence, p; objective sum of T(0,0)."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    g = gaussian_filter(rng.standard_normal((side, side)), sigma=4.0, mode='wrap')
    g = (g - g.mean()) / g.std()
    eps = 1.0 + 11.25 / (1.0 + np.exp(-8.0 * g))
    return dict(name='adjoint_layer', eps=eps[None].astype(np.complex128), thickness=np.array([220.0]),
                period=(1000., 1000.), orders=(9, 9), wavelengths=np.linspace(1000., 1600., n_wavelengths),
                theta=0.0, phi=0.0, pol='p', eps_top=1.0, eps_bot=2.25)


ORDER_CHOICES = ((5, 5), (8, 8), (11, 11), (15, 15))
EPS_CHOICES = (1.0, 2.25, 12.25, -20 + 1.5j)


def serving_request(rng, idx, orders_choices=ORDER_CHOICES, sides=(64, 128, 256), max_layers=6):
    orders = orders_choices[int(rng.integers(0, len(orders_choices)))]
    L = int(rng.integers(1, max_layers + 1))
    side = int(sides[int(rng.integers(0, len(sides)))])
    layers = []
    for _ in range(L):
        hi = EPS_CHOICES[int(rng.integers(0, len(EPS_CHOICES)))]
        lo = EPS_CHOICES[int(rng.integers(0, len(EPS_CHOICES)))]
        layers.append(binary_raster(rng, side, eps_hi=hi, eps_lo=lo))
    return dict(id=idx, eps=np.stack(layers), thickness=rng.uniform(50., 400., size=L),
                orders=orders, period=(1000., 1000.), wavelength=float(rng.uniform(400., 1600.)),
                theta=float(rng.uniform(0., math.pi / 3)), phi=float(rng.uniform(0., 2 * math.pi)),
                pol='s' if rng.random() < 0.5 else 'p', eps_top=1.0, eps_bot=2.25)


def serving_stream(n_requests=4096, rate_hz=50.0, seed=5):
    """Requests with Poisson arrival times (exponential gaps at ``rate_hz``)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate_hz, size=n_requests))
    reqs = [serving_request(rng, i) for i in range(n_requests)]
    for r, ti in zip(reqs, t):
        r['arrival'] = float(ti)
    return reqs


def pol_pair(p):
    """(a_s, a_p) as the reference resolves 's' (psi = pi/2) and 'p' (psi = 0)."""
    if p == 's':
        return (1.0 + 0j, complex(math.cos(math.pi / 2)))
    return (0j, 1.0 + 0j)
