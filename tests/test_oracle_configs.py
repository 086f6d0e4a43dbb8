"""The oracle against the reference's runs at the benchmark's own sizes (``golden/ref_configs.npz``):
the quickstart 1D grating and one wavelength of the orders-(7, 7) crossed-grating sweep on its
256x256 rasters, s and p, per-order R/T within 1e-11 of the largest efficiency. (The orders-(12, 12)
points are held by the GPU tests; the oracle would take about half a minute per point here.)"""
import os

import numpy as np
import pytest

from oracle import rcwa_oracle as O

FIX = os.path.join(os.path.dirname(__file__), 'golden', 'ref_configs.npz')


def _case(name):
    d = np.load(FIX)
    c = {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}
    c['structure'] = d[f"{str(c['stack'])}__structure"]
    return c


def test_fixture_lists_the_benchmark_points():
    names = [str(n) for n in np.load(FIX)['names']]
    assert names[0] == 'grating_1d'
    assert sum(n.startswith('crossed_') for n in names) == 4
    assert sum(n.startswith('mixed_') for n in names) == 2
    d = np.load(FIX)
    assert d['crossed__structure'].shape == (4, 256, 256)
    assert d['mixed__structure'].shape == (4, 256, 256)


@pytest.mark.parametrize('name', ['grating_1d', 'crossed_0'])
def test_oracle_matches_reference_at_benchmark_size(name):
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    for pol in ('s', 'p'):
        o = O.solve_stack(c['structure'], np.asarray(c['thickness'], float), float(c['wavelength']),
                          tuple(np.asarray(c['period'], float)), hu, hv, float(c['theta']), float(c['phi']),
                          complex(c['eps_top']), complex(c['eps_bot']), pol)
        scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
        assert np.abs(o['R'][0] - c[f'R_{pol}']).max() <= 1e-11 * scale, (name, pol)
        assert np.abs(o['T'][0] - c[f'T_{pol}']).max() <= 1e-11 * scale, (name, pol)
