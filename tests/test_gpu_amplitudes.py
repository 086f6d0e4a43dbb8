"""The published per-order readings through the CUDA path: rcwa.run keeps the efficiency kernel's
Fresnel amplitudes, and outputs['reflected'|'transmitted'] carry them about the cell centre, with
the Cartesian ratios, the per-order powers and the wavevectors, against the reference's own run."""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
NAMES = list(np.load(os.path.join(GOLDEN, 'ref_amplitudes.npz'))['names'])


@pytest.mark.parametrize('name', NAMES)
def test_gpu_amplitude_ratios_match_the_reference(name):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import rcwa
    d = np.load(os.path.join(GOLDEN, 'ref_amplitudes.npz'))
    c = {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}
    hu, hv = (int(v) for v in c['orders'])
    st, th = np.asarray(c['structure'], complex), np.asarray(c['thickness'], float)
    layers = tuple(rcwa.Layer(thickness=float(t), epsilon=e) for e, t in zip(st[::-1], th[::-1]))
    for tag, pol in (('p', 'p'), ('mix', (0.6, 0.8j))):
        prob = rcwa.Problem(units=rcwa.Units('nm'),
                            stack=rcwa.Stack(period=tuple(float(p) for p in c['period']),
                                             top=rcwa.Material(epsilon=complex(c['eps_top'])),
                                             bottom=rcwa.Material(epsilon=complex(c['eps_bot'])), layers=layers),
                            excitation=rcwa.Excitation(wavelength=float(c['wavelength']), sources=(
                                rcwa.PlaneWave(polarization=pol, theta=float(c['theta']), phi=float(c['phi'])),)))
        res = rcwa.run(prob, numerics=rcwa.Numerics(orders=(hu, hv)))
        for port in ('reflected', 'transmitted'):
            o = res.outputs[port]
            for comp, got in (('s', o.amplitude_ratio_s), ('p', o.amplitude_ratio_p)):
                want = c[f'{tag}_{port}_{comp}']
                assert np.abs(got[0].cpu().numpy() - want).max() <= 1e-10 * max(1.0, np.abs(want).max()), \
                    (name, tag, port, comp)
        # the other readings, in micrometres with a 2.5 V/m source
        um = 1e-3
        layers_um = tuple(rcwa.Layer(thickness=float(t) * um, epsilon=e) for e, t in zip(st[::-1], th[::-1]))
        prob = rcwa.Problem(units=rcwa.Units('um'),
                            stack=rcwa.Stack(period=tuple(float(p) * um for p in c['period']),
                                             top=rcwa.Material(epsilon=complex(c['eps_top'])),
                                             bottom=rcwa.Material(epsilon=complex(c['eps_bot'])), layers=layers_um),
                            excitation=rcwa.Excitation(wavelength=float(c['wavelength']) * um, sources=(
                                rcwa.PlaneWave(polarization=pol, theta=float(c['theta']), phi=float(c['phi']),
                                               amplitude=2.5),)))
        res = rcwa.run(prob, numerics=rcwa.Numerics(orders=(hu, hv)))
        p_inc = float(c[f'{tag}_reflected_incident_power'][0])
        for port in ('reflected', 'transmitted'):
            o = res.outputs[port]
            key = f'{tag}_{port}'
            assert abs(float(o.reference['incident_power'][0]) - p_inc) <= 1e-10 * p_inc
            assert np.abs(o.power[0].cpu().numpy() - c[f'{key}_power']).max() <= 1e-10 * p_inc, (name, key)
            for field_ in ('amplitude_ratio_xyz', 'k_parallel', 'k_normal'):
                want = c[f'{key}_{field_}']
                got = getattr(o, field_)[0].cpu().numpy()
                assert np.abs(got - want).max() <= 1e-10 * max(1.0, np.abs(want).max()), (name, key, field_)
