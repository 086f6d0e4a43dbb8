"""Admission of the lifecycle mirror on the CPU: what the GB300 path accepts, and the reference's
error classes and codes for what it refuses (no GPU calls: resolution happens on the host)."""
import math

import numpy as np
import pytest

from wavebit_gb300 import rcwa


def _problem(**kw):
    layers = kw.pop('layers', (rcwa.Layer(thickness=120.0, epsilon=np.array([[1.0, 12.25], [12.25, 1.0]])),
                               rcwa.Layer(thickness=80.0, epsilon=2.25)))
    stack = rcwa.Stack(layers=layers, top=kw.pop('top', rcwa.Material(1.0)),
                       bottom=kw.pop('bottom', rcwa.Material(2.25)), period=kw.pop('period', (500.0, 600.0)),
                       lattice=kw.pop('lattice', None))
    src = kw.pop('source', rcwa.PlaneWave(polarization='p', theta=0.3, phi=0.1))
    return rcwa.Problem(stack=stack, excitation=rcwa.Excitation(kw.pop('wavelength', 640.0), (src,)),
                        units=rcwa.Units('nm'))


def test_a_plain_problem_resolves_in_kernel_order():
    r = rcwa._resolve(_problem(), rcwa.Numerics(orders=(3, 2)))
    # the public stack lists the bottom layer first; kernels take the entry (top) face first
    assert r['rasters'][0].shape == (1, 1) and r['rasters'][1].shape == (2, 2)
    assert np.allclose(r['thickness'], [80.0, 120.0])
    assert r['orders'] == (3, 2) and r['period'] == (500.0, 600.0)
    assert r['eps_top'] == 1 and r['eps_bot'] == 2.25
    assert r['pol'] == (0j, 1 + 0j)
    assert np.array_equal(r['wavelengths'], [640.0])


def test_polarization_pairs_are_normalised():
    r = rcwa._resolve(_problem(source=rcwa.PlaneWave(polarization=(3.0, 4.0))), rcwa.Numerics())
    assert abs(r['pol'][0] - 0.6) < 1e-15 and abs(r['pol'][1] - 0.8) < 1e-15
    r = rcwa._resolve(_problem(source=rcwa.PlaneWave(polarization='s')), rcwa.Numerics())
    assert r['pol'][0] == 1 and abs(r['pol'][1] - math.cos(math.pi / 2)) == 0


@pytest.mark.parametrize('kw,error,code,path', [
    (dict(lattice=((1, 0), (0.5, 1))), rcwa.UnsupportedFeatureError, 'feature.unsupported', 'stack.lattice'),
    (dict(layers=()), rcwa.ValidationError, 'input.invalid', 'stack.layers'),
    (dict(layers=(rcwa.Layer(thickness=50.0, epsilon=2.0, regions=('disc',)),)), rcwa.UnsupportedFeatureError,
     'feature.unsupported', 'stack.layers[0]'),
    (dict(layers=(rcwa.Layer(thickness=50.0, epsilon=2.0, mu=2.0),)), rcwa.UnsupportedFeatureError,
     'feature.unsupported', 'stack.layers[0].mu'),
    (dict(layers=(rcwa.Layer(thickness=-1.0, epsilon=2.0),)), rcwa.ValidationError, 'input.invalid',
     'stack.layers[0].thickness'),
    (dict(layers=(rcwa.Layer(thickness=10.0, epsilon=np.array([[np.nan, 1.0]])),)), rcwa.ValidationError,
     'input.invalid', 'stack.layers[0].epsilon'),
    (dict(top=rcwa.Material(2.0 + 0.1j)), rcwa.UnsupportedFeatureError, 'feature.unsupported', 'stack.top'),
    (dict(bottom=rcwa.Material(2.0, mu=3.0)), rcwa.UnsupportedFeatureError, 'feature.unsupported', 'stack.bottom'),
    (dict(top=rcwa.Material(lambda wl: 2.0)), rcwa.UnsupportedFeatureError, 'feature.unsupported', 'stack.top'),
    (dict(wavelength=-5.0), rcwa.ValidationError, 'input.invalid', 'excitation.wavelength'),
    (dict(source=rcwa.PlaneWave(side='bottom')), rcwa.UnsupportedFeatureError, 'feature.unsupported',
     'excitation.sources[0]'),
    (dict(source=rcwa.PlaneWave(kx=0.1)), rcwa.UnsupportedFeatureError, 'feature.unsupported',
     'excitation.sources[0]'),
    (dict(source=rcwa.PlaneWave(theta=2.0)), rcwa.ValidationError, 'input.invalid', 'excitation.sources[0].theta'),
])
def test_refusals_carry_the_reference_classes_and_codes(kw, error, code, path):
    with pytest.raises(error) as e:
        rcwa._resolve(_problem(**kw), rcwa.Numerics(orders=(1, 1)))
    assert e.value.code == code and e.value.path == path


@pytest.mark.parametrize('numerics,path', [
    (rcwa.Numerics(orders=(-1, 2)), 'numerics.orders'),
    (rcwa.Numerics(orders=(2,)), 'numerics.orders'),
])
def test_bad_orders_are_refused(numerics, path):
    with pytest.raises(rcwa.ValidationError) as e:
        rcwa._resolve(_problem(), numerics)
    assert e.value.path == path


@pytest.mark.parametrize('field,value', [('algorithm', 'etm'), ('fourier_coefficients', 'integrated'),
                                         ('factorization', 'nvf'), ('li_nesting', 'alternating')])
def test_numerics_outside_the_path_are_unsupported(field, value):
    num = rcwa.Numerics(orders=(1, 1), **{field: value})
    with pytest.raises(rcwa.UnsupportedFeatureError):
        rcwa._resolve(_problem(), num)
