"""Correct or loud at an exact graze (an order on a layer's light line), the reference's contract
(rcwa/_engine/solve_2d.py:118-222, :2463-2488; its tests/rcwa/test_rayleigh_guard.py).

``golden/ref_graze.npz`` holds the reference's own exact-graze 2D stacks: its outcome at the
exact point (refused or solved) and its R/T at 1e-8 relative detuning. At the exact point, an
answer is either a refusal (``FloatingPointError`` in the oracle, ``NumericalError('rcwa.singular')``
through the lifecycle) or within 1e-4 of the detuned truth with R + T = 1 to 1e-4. Quietly wrong
is never allowed. Which of the two a stack gets depends on the platform's round-off in the
cluster, so the assertions are on the pair of outcomes, as the reference's are.
"""
import os

import numpy as np
import pytest

from oracle import rcwa_oracle as O

FIX = os.path.join(os.path.dirname(__file__), 'golden', 'ref_graze.npz')
NAMES = [str(n) for n in np.load(FIX)['names']]


def _case(name):
    d = np.load(FIX)
    return {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}


def _oracle(c, wavelength, rebuild):
    hu, hv = (int(v) for v in c['orders'])
    return O.solve_stack(c['structure'], np.asarray(c['thickness'], float), float(wavelength), (1000.0, 1000.0), hu,
                         hv, 0.0, 0.0, 1.0, 2.25, 's', rebuild_grazing=rebuild)


@pytest.mark.parametrize('name', NAMES)
def test_oracle_detuned_matches_the_reference(name):
    c = _case(name)
    o = _oracle(c, c['wavelength_far'], False)
    assert np.abs(o['R'][0] - c['R_far']).max() < 1e-11 and np.abs(o['T'][0] - c['T_far']).max() < 1e-11


@pytest.mark.parametrize('name', NAMES)
def test_oracle_exact_graze_is_correct_or_loud(name):
    c = _case(name)
    assert bool(c['exact_refused']) and str(c['exact_code']) == 'rcwa.singular'
    try:
        o = _oracle(c, c['wavelength'], True)
    except FloatingPointError:
        return
    R, T = o['R'][0].sum(), o['T'][0].sum()
    assert abs(R - c['R_far'].sum()) < 1e-4 and abs(R + T - 1.0) < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize('name', NAMES)
def test_lifecycle_exact_graze_is_correct_or_loud_on_the_gpu(name):
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import rcwa
    from wavebit_gb300.rcwa import NumericalError
    c = _case(name)

    def problem(wl):
        st = c['structure'][::-1]
        layers = tuple(rcwa.Layer(thickness=float(t), epsilon=np.asarray(e))
                       for e, t in zip(st, list(np.asarray(c['thickness'], float))[::-1]))
        return rcwa.Problem(units=rcwa.Units(length='nm'),
                            stack=rcwa.Stack(period=(1000.0, 1000.0), top=rcwa.Material(epsilon=1.0),
                                             bottom=rcwa.Material(epsilon=2.25), layers=layers),
                            excitation=rcwa.Excitation(wavelength=float(wl), sources=(
                                rcwa.PlaneWave(polarization='s', theta=0.0, phi=0.0),)))
    num = rcwa.Numerics(orders=tuple(int(v) for v in c['orders']))
    far = rcwa.run(problem(c['wavelength_far']), numerics=num)
    assert np.abs(far.R.cpu().numpy()[0] - c['R_far']).max() < 1e-10
    try:
        res = rcwa.run(problem(c['wavelength']), numerics=num)
    except NumericalError as exc:
        assert exc.code == 'rcwa.singular' and 'detuning' in str(exc)
        return
    R, T = float(res.R.sum()), float(res.T.sum())
    assert abs(R - c['R_far'].sum()) < 1e-4 and abs(R + T - 1.0) < 1e-4
