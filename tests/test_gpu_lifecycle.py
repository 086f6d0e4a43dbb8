"""The rcwa.check -> prepare -> run mirror against the reference's own run (fixtures)."""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


def _rcwa():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import rcwa
    return rcwa


def _problem(rcwa, c, pol):
    # fixtures store layers entry face first; the public stack lists them bottom to top
    st = np.asarray(c['structure'])[::-1]
    th = list(c['thickness'])[::-1]
    layers = tuple(rcwa.Layer(thickness=float(t), epsilon=e) for e, t in zip(st, th))
    return rcwa.Problem(
        stack=rcwa.Stack(layers=layers, top=rcwa.Material(complex(c['eps_top'])),
                         bottom=rcwa.Material(complex(c['eps_bot'])), period=tuple(c['period'])),
        excitation=rcwa.Excitation(wavelength=float(c['wavelength']), sources=(
            rcwa.PlaneWave(polarization=pol, theta=float(c['theta']), phi=float(c['phi'])),)),
        units=rcwa.Units('nm'))


def test_run_matches_reference_fixtures():
    rcwa = _rcwa()
    d = np.load(os.path.join(GOLDEN, 'ref_cases.npz'))
    for name in d['names']:
        c = {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(str(name) + '__')}
        for pol in ('s', 'p'):
            res = rcwa.run(_problem(rcwa, c, pol), numerics=rcwa.Numerics(orders=tuple(int(v) for v in c['orders'])))
            R, T = res.R[0].cpu().numpy(), res.T[0].cpu().numpy()
            scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
            assert R.shape == c[f'R_{pol}'].shape
            assert np.abs(R - c[f'R_{pol}']).max() <= 1e-10 * scale, (name, pol)
            assert np.abs(T - c[f'T_{pol}']).max() <= 1e-10 * scale, (name, pol)


def test_check_reports_without_solving():
    rcwa = _rcwa()
    prob = rcwa.Problem(stack=rcwa.Stack(layers=(rcwa.Layer(100.0, np.ones((8, 8)) * 4.0),), period=(500.0, 500.0)),
                        excitation=rcwa.Excitation(600.0, (rcwa.PlaneWave(),)))
    rep = rcwa.check(prob, numerics=rcwa.Numerics(orders=(3, 2)))
    assert rep.estimates['retained_spatial_modes'] == 35
    assert rep.resolved['solve_path'] == '2d'


def test_prepared_run_reuses_assembly_across_wavelengths():
    rcwa = _rcwa()
    rng = np.random.default_rng(3)
    ras = np.where(rng.random((12, 12)) < 0.5, 12.25, 1.0)
    prob = rcwa.Problem(stack=rcwa.Stack(layers=(rcwa.Layer(150.0, ras),), bottom=rcwa.Material(2.25),
                                         period=(700.0, 700.0)),
                        excitation=rcwa.Excitation(np.linspace(600, 900, 7), (rcwa.PlaneWave(polarization='p'),)))
    prep = rcwa.prepare(prob, numerics=rcwa.Numerics(orders=(2, 2)))
    a = prep.run()
    b = prep.run(prob)
    assert a.R.shape == (7, 5, 5)
    assert torch.equal(a.R, b.R) and torch.equal(a.T, b.T)
    # lossless: R + T = 1
    tot = (a.R.sum((1, 2)) + a.T.sum((1, 2))).cpu().numpy()
    assert np.abs(tot - 1).max() < 1e-12


def test_unsupported_numerics_are_refused():
    rcwa = _rcwa()
    prob = rcwa.Problem(stack=rcwa.Stack(layers=(rcwa.Layer(100.0, np.ones((4, 4))),)),
                        excitation=rcwa.Excitation(600.0, (rcwa.PlaneWave(),)))
    with pytest.raises(rcwa.UnsupportedFeatureError):
        rcwa.run(prob, numerics=rcwa.Numerics(orders=(1, 1), factorization='nvf'))
    with pytest.raises(rcwa.ValidationError):
        rcwa.run(prob, numerics=rcwa.Numerics(orders=(1, 1)), device='cpu')
