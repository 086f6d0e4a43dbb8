"""Incidence given as a wavevector (``PlaneWave(kx=, ky=)``, rad per length unit): the in-plane
wavevector is fixed across wavelengths, so the angle in the lit medium changes with the
wavelength. Held to the reference's own runs (``ref_direct.npz``), lit from either side and at
exactly normal incidence."""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from oracle import rcwa_oracle as O
from wavebit_gb300 import rcwa

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
NAMES = list(np.load(os.path.join(GOLDEN, 'ref_direct.npz'))['names'])
POLS = (('s', 's'), ('mix', (0.6, 0.8j)))


def _case(name):
    d = np.load(os.path.join(GOLDEN, 'ref_direct.npz'))
    return {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}


def _problem(c, pol, **source):
    st, th = np.asarray(c['structure'], complex), np.asarray(c['thickness'], float)
    layers = tuple(rcwa.Layer(thickness=float(t), epsilon=e) for e, t in zip(st[::-1], th[::-1]))
    src = dict(side=str(c['side']), polarization=pol, kx=float(c['kx']), ky=float(c['ky']))
    src.update(source)
    return rcwa.Problem(units=rcwa.Units('nm'),
                        stack=rcwa.Stack(period=tuple(float(p) for p in c['period']),
                                         top=rcwa.Material(epsilon=complex(c['eps_top'])),
                                         bottom=rcwa.Material(epsilon=complex(c['eps_bot'])), layers=layers),
                        excitation=rcwa.Excitation(wavelength=np.asarray(c['wavelengths'], float),
                                                   sources=(rcwa.PlaneWave(**src),)))


def _check(res, c, tag, tol, name):
    np_ = lambda t: t.detach().cpu().numpy()
    for key, got in (('R', res.R), ('T', res.T)):
        want = c[f'{key}_{tag}']
        assert np.abs(np_(got) - want).max() <= tol * np.abs(want).max(), (name, tag, key)
    for port in ('reflected', 'transmitted'):
        o = res.outputs[port]
        sp = np.abs(np.stack([c[f'{tag}_{port}_s'], c[f'{tag}_{port}_p']])).max()
        for comp in ('s', 'p'):
            got = np_(getattr(o, f'amplitude_ratio_{comp}'))
            assert np.abs(got - c[f'{tag}_{port}_{comp}']).max() <= tol * sp, (name, tag, port, comp)
        want = c[f'{tag}_{port}_k_parallel']
        assert np.abs(np_(o.k_parallel) - want).max() <= 1e-13 * max(np.abs(want).max(), 1e-3), (name, port)


@pytest.mark.parametrize('name', NAMES)
def test_direct_wavevector_resolves_to_one_angle_per_wavelength(name):
    """sin(theta) = |k_par| / (k0 n) in the lit medium, phi = atan2(ky, kx); the oracle's solve at
    those angles (of the mirrored scene when lit from below) is the reference's run."""
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    r = rcwa._resolve(_problem(c, 's'), rcwa.Numerics(orders=(hu, hv)))
    wls = np.asarray(c['wavelengths'], float)
    n = np.sqrt(r['eps_top'].real)
    kx, ky = float(c['kx']), float(c['ky'])
    assert np.allclose(n * np.sin(r['thetas']), np.hypot(kx, ky) * wls / (2 * np.pi), rtol=1e-15, atol=1e-17)
    st, th = np.asarray(r['rasters']), np.asarray(r['thickness'])
    for tag, pol in POLS:
        for b, wl in enumerate(wls):
            o = O.solve_stack(st, th, wl, tuple(r['period']), hu, hv, float(r['thetas'][b]), r['phi'],
                              r['eps_top'], r['eps_bot'], pol)
            for key in ('R', 'T'):
                want = c[f'{key}_{tag}'][b]
                assert np.abs(o[key][0] - want).max() <= 1e-12 * np.abs(want).max(), (name, tag, b, key)


@pytest.mark.parametrize('name', NAMES)
def test_lifecycle_with_a_direct_wavevector_on_the_cpu(name, monkeypatch):
    """The lifecycle over two wavelengths (the ETM over the oracle's modes in place of the stage-B
    kernel): R, T, the amplitude ratios and the orders' wavevectors against the reference's run."""
    from wavebit_gb300 import engine
    from test_fields import use_cpu_stages
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    use_cpu_stages(monkeypatch)
    num = rcwa.Numerics(orders=(hu, hv), algorithm='etm')
    for tag, pol in POLS:
        r = rcwa._resolve(_problem(c, pol), num)
        conv_np = O.to_conv_mat_raster_sampled(np.stack(r['rasters']), hu, hv)
        conv = engine.ConvStack.from_matrices(*(torch.as_tensor(a) for a in conv_np), hu, hv)
        p = rcwa.Prepared.__new__(rcwa.Prepared)
        p.handle, p.numerics, p.precision = None, num, 'double'
        B = len(r['wavelengths'])
        res = p._solve_etm(r, conv, np.tile(np.arange(len(r['rasters'])), (B, 1)))
        _check(res, c, tag, 1e-11, name)
        # one wavelength of the two, with its own reference entries
        one = res.reflection.at_wavelength_index(1)
        assert one.wavelengths == res.wavelengths[1:] and torch.equal(one.power, res.reflection.power[1:])
        assert len(one.reference['incident_power']) == 1 and len(one.reference['plane']) == 1
        with pytest.raises(IndexError):
            res.reflection.at_wavelength_index(2)


def test_direct_wavevector_refusals():
    c = _case(NAMES[0])
    with pytest.raises(rcwa.ValidationError) as e:
        rcwa._resolve(_problem(c, 's', theta=0.1), rcwa.Numerics(orders=(1, 1)))
    assert e.value.code == 'source.direction_ambiguous'
    with pytest.raises(rcwa.UnsupportedFeatureError):          # past the light line: evanescent incidence
        rcwa._resolve(_problem(c, 's', kx=1.0), rcwa.Numerics(orders=(1, 1)))
    with pytest.raises(rcwa.ValidationError):
        rcwa._resolve(_problem(c, 's', kx=float('nan')), rcwa.Numerics(orders=(1, 1)))


@pytest.mark.gpu
@pytest.mark.parametrize('name', NAMES)
def test_lifecycle_with_a_direct_wavevector_on_the_gpu(name):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    for tag, pol in POLS:
        res = rcwa.run(_problem(c, pol), numerics=rcwa.Numerics(orders=(hu, hv)))
        _check(res, c, tag, 1e-10, name)
