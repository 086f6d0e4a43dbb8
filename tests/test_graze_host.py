"""The host rebuild of a grazing cluster (wavebit_gb300/graze.py) against the oracle's own
restatement of the reference's (solve_2d.py:118-222), on the reference's exact-graze stacks:
same refusal, or the same modes' physics. And the layer factors multiply to the operator."""
import os

import numpy as np
import pytest

from oracle import rcwa_oracle as O
from wavebit_gb300 import graze as G

FIX = os.path.join(os.path.dirname(__file__), 'golden', 'ref_graze.npz')


def _layer(name, wavelength_key='wavelength'):
    d = np.load(FIX)
    c = {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}
    hu, hv = (int(v) for v in c['orders'])
    conv = O.to_conv_mat_raster_sampled(c['structure'], hu, hv)
    kx, ky = O.separable_kxy(float(c[wavelength_key]), (1000.0, 1000.0), O.incident_kxy(0.0, 0.0, 1.0), hu, hv)
    kxg, kyg = O.order_grid(kx, ky)
    return kxg, kyg, [s[0] for s in conv]       # the spacer (entry layer)


def test_the_factors_multiply_to_the_layer_operator():
    kxg, kyg, (epx, epy, epz) = _layer('graze_2.0')
    om2, om_r = O.layer_operator(kxg, kyg, epx, epy, epz)
    om_l, om_r2 = G.layer_factors(kxg.real, kyg.real, epx, epy, epz)
    assert np.abs(om_r2 - om_r).max() == 0.0
    assert np.abs(om_l @ om_r2 - om2).max() <= 1e-12 * np.abs(om2).max()


@pytest.mark.parametrize('name', ['graze_2.0', 'graze_1.5'])
def test_host_rebuild_agrees_with_the_oracle(name):
    kxg, kyg, (epx, epy, epz) = _layer(name)
    om2, om_r = O.layer_operator(kxg, kyg, epx, epy, epz)
    w, W = np.linalg.eig(om2)
    q = O.mode_q(w)
    V = (om_r @ W) / q
    om_l, _ = G.layer_factors(kxg.real, kyg.real, epx, epy, epz)
    assert G.grazing(w)
    outs = []
    for fn in (lambda: G.rebuild_grazing_cluster(w, W, V, q, om_l, om_r),
               lambda: O.rebuild_grazing_cluster(w, W, V, q, O.left_factor(kxg, kyg, epz), om_r)):
        try:
            outs.append(fn())
        except FloatingPointError:
            outs.append('refused')
    assert (outs[0] == 'refused') == (outs[1] == 'refused')
    if outs[0] != 'refused' and outs[0] is not None:
        for a, b in zip(outs[0], outs[1]):
            assert np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(b).max())
