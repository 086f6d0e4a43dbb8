"""Golden per-order efficiencies of the benchmark configurations, from the reference itself.

Run where the reference source tree is available (read-only)::

    PYTHONPATH=tests/golden/refshim python tests/golden/make_config_fixtures.py --reference <root>

It writes ``ref_configs.npz``, the reference's public ``rcwa.run`` (NumPy backend, SMM, sampled
Li, fixed nesting, complex128) on the workloads the benchmark measures, at their full sizes:

* ``grating_1d`` -- the quickstart 1D grating (orders (10, 0), s);
* ``crossed_slice`` -- four of the 128 wavelengths of the crossed-grating sweep: the three
  seeded 256x256 binary rasters and the 50 nm eps = -20+1.5j layer, orders (7, 7) (N = 225,
  450x450 mode matrices), s and p;
* ``mixed_points`` -- two of the 1024 (wavelength, theta) points of the orders-(12, 12) sweep:
  four seeded 256x256 binary rasters (N = 625, 1250x1250 mode matrices), s and p.

and ``ref_graze.npz``, the reference's outcome on its own exact-graze 2D stacks (an order on a
spacer layer's light line): refused or solved at the exact point, and R/T 1e-8 away.

The rasters come from the seeded generators of ``wavebit_gb300/workloads.py`` and are stored with
the results (compressed: they are a few rectangles and discs), so the tests need neither the
generator's arithmetic nor the reference. Layers are stored in kernel order (entry face first).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import make_fixtures as MF  # noqa: E402
from wavebit_gb300 import workloads as WL  # noqa: E402

#: wavelength indices of the crossed-grating sweep's slice (of 128 over 400-1000 nm)
CROSSED_INDICES = (0, 41, 86, 127)
#: (wavelength index of 256, theta index of {0, 0.2, 0.4, 0.6}) of the orders-(12, 12) points
MIXED_POINTS = ((37, 3), (201, 1))


def _case(name, eps, thickness, wavelength, orders, theta, eps_top, eps_bot, period):
    return dict(name=name, structure=np.asarray(eps, complex), thickness=list(thickness),
                wavelength=float(wavelength), period=tuple(period), orders=tuple(orders), theta=float(theta),
                phi=0.0, eps_top=eps_top, eps_bot=eps_bot)


def config_cases():
    cases = []
    g = WL.grating_1d()
    cases.append(_case('grating_1d', g['eps'], g['thickness'], g['wavelengths'][0], g['orders'], 0.0,
                       g['eps_top'], g['eps_bot'], g['period']))
    c = WL.crossed_sweep()
    for i in CROSSED_INDICES:
        cases.append(_case(f'crossed_{i}', c['eps'], c['thickness'], c['wavelengths'][i], c['orders'], 0.0,
                           c['eps_top'], c['eps_bot'], c['period']))
    m = WL.mixed_sweep()
    for wi, ti in MIXED_POINTS:
        p = wi * 4 + ti
        cases.append(_case(f'mixed_{wi}_{ti}', m['eps'], m['thickness'], m['wavelengths'][p], m['orders'],
                           m['thetas'][p], m['eps_top'], m['eps_bot'], m['period']))
    return cases


def main():
    MF.use_reference()
    out = {}
    names = []
    stacks = {}
    for case in config_cases():
        n = case['name']
        names.append(n)
        key = n.split('_')[0]
        if key not in stacks:
            stacks[key] = case['structure']
            out[f'{key}__structure'] = case['structure']
        for k in ('thickness', 'wavelength', 'period', 'orders', 'theta', 'phi', 'eps_top', 'eps_bot'):
            out[f'{n}__{k}'] = np.asarray(case[k])
        out[f'{n}__stack'] = np.asarray(key)
        for pol in ('s', 'p'):
            R, T, _ = MF.run_ref(case, pol)
            out[f'{n}__R_{pol}'] = R
            out[f'{n}__T_{pol}'] = T
        print(n, 'R+T =', float(out[f'{n}__R_s'].sum() + out[f'{n}__T_s'].sum()), flush=True)
    out['names'] = np.array(names)
    np.savez_compressed(os.path.join(HERE, 'ref_configs.npz'), **out)
    print('ref_configs.npz:', len(names), 'cases')




def graze_cases():
    """The reference's exact-graze 2D stacks (tests/rcwa/test_rayleigh_guard.py of the reference):
    a uniform spacer of index 2.0 or 1.5 over a 20-pixel pillar row, period 1000 nm, 500 nm, orders
    (5, 1), where order m = 4 (kx = 2.0) or m = 3 (kx = 1.5) sits on the spacer's light line."""
    out = []
    for n_sp in (2.0, 1.5):
        pillar = np.ones((2, 20), complex)
        pillar[:, 6:14] = 12.25
        st = np.stack([np.full((2, 20), n_sp ** 2, complex), pillar])
        out.append(dict(name=f'graze_{n_sp}', structure=st, thickness=[300.0, 200.0], wavelength=500.0,
                        period=(1000., 1000.), orders=(5, 1), theta=0.0, phi=0.0, eps_top=1.0, eps_bot=2.25))
    return out


def make_graze():
    """``ref_graze.npz``: each exact-graze stack's inputs, the reference's outcome at the exact
    point (refused with its error code, or its R/T) and its R/T at 1e-8 relative detuning."""
    MF.use_reference()
    out = {}
    for case in graze_cases():
        n = case['name']
        for k in ('structure', 'thickness', 'wavelength', 'period', 'orders', 'theta', 'phi', 'eps_top', 'eps_bot'):
            out[f'{n}__{k}'] = np.asarray(case[k])
        try:
            R, T, _ = MF.run_ref(case, 's')
            out[f'{n}__exact_refused'] = np.asarray(False)
            out[f'{n}__R_exact'], out[f'{n}__T_exact'] = R, T
        except Exception as exc:
            out[f'{n}__exact_refused'] = np.asarray(True)
            out[f'{n}__exact_code'] = np.asarray(getattr(exc, 'code', type(exc).__name__))
        far = dict(case, wavelength=case['wavelength'] * (1 + 1e-8))
        R, T, _ = MF.run_ref(far, 's')
        out[f'{n}__R_far'], out[f'{n}__T_far'] = R, T
        out[f'{n}__wavelength_far'] = np.asarray(far['wavelength'])
        print(n, 'refused' if out[f'{n}__exact_refused'] else 'solved', 'R_far', R.sum())
    out['names'] = np.array([c['name'] for c in graze_cases()])
    np.savez_compressed(os.path.join(HERE, 'ref_graze.npz'), **out)


if __name__ == '__main__':
    main()
    make_graze()
