"""The ETM connecting algorithm (``Numerics(algorithm='etm')``): the device-agnostic recursion of
``wavebit_gb300.etm`` on the CPU with the oracle's modes, the lifecycle bookkeeping on the CPU
with the stage-B kernel replaced by the oracle, and the whole path on a GPU -- each against the
reference's own ETM runs and the SMM."""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from oracle import rcwa_oracle as O
from wavebit_gb300 import etm as E
from wavebit_gb300 import rcwa
from wavebit_gb300.adjoint import ports

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
NAMES = list(np.load(os.path.join(GOLDEN, 'ref_etm.npz'))['names'])


def _case(name):
    d = np.load(os.path.join(GOLDEN, 'ref_etm.npz'))
    return {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}


def _check(R, T, c, tol, label):
    for col, pol in ((1, 's'), (2, 'p')):
        scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
        assert np.abs(R[col] - c[f'R_{pol}']).max() <= tol * scale, (label, pol)
        assert np.abs(T[col] - c[f'T_{pol}']).max() <= tol * scale, (label, pol)


@pytest.mark.parametrize('name', NAMES)
def test_etm_recursion_matches_the_reference_on_the_cpu(name):
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    st = np.asarray(c['structure'], complex)
    wl = float(c['wavelength'])
    pv = ports(wl, tuple(float(p) for p in c['period']), float(c['theta']), float(c['phi']),
               complex(c['eps_top']), complex(c['eps_bot']), hu, hv, 'cpu')
    conv = O.to_conv_mat_raster_sampled(st, hu, hv)
    modes = []
    for i in range(st.shape[0]):
        W, V, q, _, _ = O.layer_modes_2d(pv['kx'].numpy() + 0j, pv['ky'].numpy() + 0j, conv[0][i], conv[1][i], conv[2][i])
        modes.append(tuple(torch.as_tensor(a) for a in (W, V, q)))
    R, T = E.etm_solve(modes, np.asarray(c['thickness'], float), 2 * np.pi / wl, pv, O.polarization_pair('s'),
                       2 * hu + 1, 2 * hv + 1)
    _check(R.numpy(), T.numpy(), c, 1e-12, name)


@pytest.mark.parametrize('name', ['crossed_1', 'crossed_4', 'metal_substrate', 'tir'])
def test_etm_amplitudes_are_the_smm_fresnel_amplitudes(name):
    """etm_solve(amplitudes=True): the final matching's unknowns, as the efficiency kernel's
    Fresnel amplitudes (r_s, r_p, t_s, t_p about the cell corner), equal the oracle's SMM ones
    under mixed incidence; the pure-s and pure-p columns too."""
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    st, th = np.asarray(c['structure'], complex), np.asarray(c['thickness'], float)
    wl, per = float(c['wavelength']), tuple(float(p) for p in c['period'])
    pol = (0.6, 0.8j)
    o = O.solve_stack(st, th, wl, per, hu, hv, float(c['theta']), float(c['phi']), complex(c['eps_top']),
                      complex(c['eps_bot']), pol)
    pv = ports(wl, per, float(c['theta']), float(c['phi']), complex(c['eps_top']), complex(c['eps_bot']), hu, hv, 'cpu')
    conv = O.to_conv_mat_raster_sampled(st, hu, hv)
    modes = []
    for i in range(st.shape[0]):
        W, V, q, _, _ = O.layer_modes_2d(pv['kx'].numpy() + 0j, pv['ky'].numpy() + 0j, conv[0][i], conv[1][i], conv[2][i])
        modes.append(tuple(torch.as_tensor(a) for a in (W, V, q)))
    _, _, amps = E.etm_solve(modes, th, 2 * np.pi / wl, pv, O.polarization_pair(pol), 2 * hu + 1, 2 * hv + 1,
                             amplitudes=True)
    want = np.stack([np.stack([a[col].reshape(-1) for a in o['amps']]) for col in range(3)])
    assert amps.shape == want.shape
    assert np.abs(amps.numpy() - want).max() <= 1e-12 * np.abs(want).max(), name


def _problem(c, **kw):
    st, th = np.asarray(c['structure'], complex), np.asarray(c['thickness'], float)
    layers = tuple(rcwa.Layer(thickness=float(t), epsilon=e) for e, t in zip(st[::-1], th[::-1]))
    return rcwa.Problem(units=rcwa.Units('nm'),
                        stack=rcwa.Stack(period=tuple(float(p) for p in c['period']),
                                         top=rcwa.Material(epsilon=complex(c['eps_top'])),
                                         bottom=rcwa.Material(epsilon=complex(c['eps_bot'])), layers=layers),
                        excitation=rcwa.Excitation(wavelength=float(c['wavelength']), sources=(
                            rcwa.PlaneWave(polarization='s', theta=float(c['theta']), phi=float(c['phi'])),)),
                        **kw)


def test_etm_refuses_a_scattering_matrix():
    """The ETM never forms a both-sides operator (scattering.py:482-495; _lifecycle.py:130-132)."""
    c = _case(NAMES[0])
    p = _problem(c, outputs=rcwa.Outputs(scattering=True))
    with pytest.raises(rcwa.UnsupportedFeatureError) as e:
        rcwa._resolve(p, rcwa.Numerics(orders=(1, 1), algorithm='etm'))
    assert e.value.code == 'rcwa.scattering_algorithm'


@pytest.mark.parametrize('name', ['crossed_1', 'symmetric_pillar'])
def test_lifecycle_etm_on_the_cpu(name, monkeypatch):
    """Prepared._solve_etm with the stage-B kernel replaced by the oracle on the CPU."""
    from wavebit_gb300 import engine
    from test_fields import use_cpu_stages
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    st = np.asarray(c['structure'], complex)
    conv_np = O.to_conv_mat_raster_sampled(st, hu, hv)
    conv = engine.ConvStack.from_matrices(*(torch.as_tensor(a) for a in conv_np), hu, hv)
    use_cpu_stages(monkeypatch)
    num = rcwa.Numerics(orders=(hu, hv), algorithm='etm')
    r = rcwa._resolve(_problem(c), num)
    p = rcwa.Prepared.__new__(rcwa.Prepared)
    p.handle, p.numerics, p.precision = None, num, 'double'
    res = p._solve_etm(r, conv, np.tile(np.arange(st.shape[0]), (1, 1)))
    assert res.diagnostics['algorithm'] == 'etm'
    _check(np.stack([res.R[0].numpy(), res.outputs['s_inc']['R'][0].numpy(), res.outputs['p_inc']['R'][0].numpy()]),
           np.stack([res.T[0].numpy(), res.outputs['s_inc']['T'][0].numpy(), res.outputs['p_inc']['T'][0].numpy()]),
           c, 1e-12, name)
    # the lifecycle's per-order readings: powers add up to the efficiencies times the incident power
    refl, trans = res.reflection, res.transmission
    p_inc = float(refl.reference['incident_power'][0])
    assert refl.reference['length_units'] == 'nm' and refl.k_normal.shape == refl.efficiency.shape
    assert res.provenance['solver'] == 'rcwa' and res.provenance['length_units'] == 'nm'
    assert res.provenance['requested_wavelengths'] == res.wavelengths
    assert res.diagnostics['effective_theta'] == (float(c['theta']),) and bool(res.diagnostics['efficiency_defined'].all())
    assert float(refl.power.sum()) == pytest.approx(float(res.R.sum()) * p_inc, rel=1e-10)
    assert float(trans.power.sum()) == pytest.approx(float(res.T.sum()) * p_inc, rel=1e-10)


@pytest.mark.gpu
@pytest.mark.parametrize('name', NAMES)
def test_lifecycle_etm_matches_the_reference_on_the_gpu(name):
    """rcwa.run(..., Numerics(algorithm='etm')) with the kernels' modes against the reference's
    ETM runs, and against this package's own SMM run of the same problem."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    etm = rcwa.run(_problem(c), numerics=rcwa.Numerics(orders=(hu, hv), algorithm='etm'))
    smm = rcwa.run(_problem(c), numerics=rcwa.Numerics(orders=(hu, hv)))
    R = np.stack([etm.R[0].cpu().numpy()] + [etm.outputs[k]['R'][0].cpu().numpy() for k in ('s_inc', 'p_inc')])
    T = np.stack([etm.T[0].cpu().numpy()] + [etm.outputs[k]['T'][0].cpu().numpy() for k in ('s_inc', 'p_inc')])
    _check(R, T, c, 1e-10, name)
    assert np.abs(etm.R.cpu().numpy() - smm.R.cpu().numpy()).max() <= 1e-10
    for port in ('reflected', 'transmitted'):
        for key in ('amplitude_ratio_s', 'amplitude_ratio_p', 'power'):
            a, b = getattr(etm.outputs[port], key), getattr(smm.outputs[port], key)
            scale = torch.abs(b).max().item() if key == 'power' else max(1.0, torch.abs(b).max().item())
            assert torch.abs(a - b).max().item() <= 1e-9 * scale, (name, port, key)


def _given_modes(c, wavelengths, device):
    """(W, V, q, inp) of the case at several wavelengths, the oracle's modes, on `device`."""
    from wavebit_gb300 import engine
    hu, hv = (int(v) for v in c['orders'])
    st, th = np.asarray(c['structure'], complex), np.asarray(c['thickness'], float)
    per = tuple(float(p) for p in c['period'])
    conv = O.to_conv_mat_raster_sampled(st, hu, hv)
    Ws, Vs, qs = [], [], []
    for wl in wavelengths:
        pv = ports(wl, per, float(c['theta']), float(c['phi']), complex(c['eps_top']), complex(c['eps_bot']), hu, hv,
                   'cpu')
        for i in range(st.shape[0]):
            W, V, q, _, _ = O.layer_modes_2d(pv['kx'].numpy() + 0j, pv['ky'].numpy() + 0j, conv[0][i], conv[1][i],
                                             conv[2][i])
            Ws.append(W); Vs.append(V); qs.append(q)
    B, L = len(wavelengths), st.shape[0]
    inp = engine.BatchInputs(np.tile(np.arange(L), (B, 1)), np.tile(th, (B, 1)), wavelengths, np.tile(per, (B, 1)),
                             np.full(B, float(c['theta'])), np.full(B, float(c['phi'])),
                             np.full(B, complex(c['eps_top'])), np.full(B, complex(c['eps_bot'])),
                             np.tile([0.6, 0.8j], (B, 1)), device=device)
    return tuple(torch.as_tensor(np.stack(a), device=device) for a in (Ws, Vs, qs)) + (inp,)


@pytest.mark.gpu
@pytest.mark.parametrize('name', ['crossed_1', 'crossed_4', 'metal_substrate', 'tir'])
def test_etm_kernels_match_the_torch_recursion(name):
    """wb_etm_solve (the library's LU and GEMM kernels) against the torch restatement of the same
    recursion on the same modes, three wavelengths in one batch: R, T and the Fresnel amplitudes
    to 1e-12."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import engine
    from test_fields import _torch_etm_solve
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    wls = [float(c['wavelength']) * f for f in (1.0, 1.07, 0.93)]
    W, V, q, inp = _given_modes(c, wls, 'cuda')
    R, T, st, amps = engine.etm_solve(W, V, q, inp, hu, hv, amplitudes=True)
    W0, V0, q0, inp0 = _given_modes(c, wls, 'cpu')
    R0, T0, _, a0 = _torch_etm_solve(W0, V0, q0, inp0, hu, hv, amplitudes=True)
    assert int(st.abs().sum()) == 0
    scale = max(float(R0.abs().max()), float(T0.abs().max()))
    assert float((R.cpu() - R0).abs().max()) <= 1e-12 * scale, name
    assert float((T.cpu() - T0).abs().max()) <= 1e-12 * scale, name
    assert float((amps.cpu() - a0).abs().max()) <= 1e-12 * float(a0.abs().max()), name
