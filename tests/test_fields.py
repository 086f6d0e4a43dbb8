"""Field reconstruction (``Outputs(fields=True)``, ``Result.field``): the device-agnostic state
and synthesis of ``wavebit_gb300.fields`` on the CPU with the oracle's modes, and the whole
lifecycle on a GPU with the kernels' modes, both against the reference's ``result.field``."""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from oracle import rcwa_oracle as O
from wavebit_gb300 import fields as F
from wavebit_gb300 import rcwa
from wavebit_gb300.adjoint import ports

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
NAMES = list(np.load(os.path.join(GOLDEN, 'ref_fields.npz'))['names'])


def _case(name):
    d = np.load(os.path.join(GOLDEN, 'ref_fields.npz'))
    return {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}


def _check(got, want, tol, label):
    for part in (slice(0, 3), slice(3, 6)):
        scale = np.abs(want[..., part]).max()
        assert np.abs(got[..., part] - want[..., part]).max() <= tol * scale, (label, part)


@pytest.mark.parametrize('name', NAMES)
def test_state_and_synthesis_match_the_reference_on_the_cpu(name):
    """build_state + synthesize on CPU tensors, fed the oracle's Cartesian modes and slots."""
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    st = np.asarray(c['structure'], complex)
    th = np.asarray(c['thickness'], float)
    wl, per = float(c['wavelength']), tuple(float(p) for p in c['period'])
    pv = ports(wl, per, float(c['theta']), float(c['phi']), complex(c['eps_top']), complex(c['eps_bot']), hu, hv, 'cpu')
    kxg, kyg = pv['kx'].numpy(), pv['ky'].numpy()
    conv = O.to_conv_mat_raster_sampled(st, hu, hv)
    modes, epz = [], []
    for i in range(st.shape[0]):
        W, V, q, _, _ = O.layer_modes_2d(kxg + 0j, kyg + 0j, conv[0][i], conv[1][i], conv[2][i])
        modes.append(tuple(torch.as_tensor(a) for a in (W, V, q)))
        epz.append(torch.as_tensor(conv[2][i]))
    for pol in ('s', 'p'):
        state = F.build_state(modes, epz, th, wl, pv, O.polarization_pair(pol), hu, hv)
        z, owner, depth = F.height_points(c['z'], th)
        got = F.synthesize(state, owner, depth, c['x'], c['y'], float(c[f'amplitude_{pol}'])).numpy()
        _check(got, c[f'field_{pol}'][0], 1e-12, (name, pol))


def test_height_rules():
    """Faces belong to the layer above; counts give every layer both of its faces."""
    th = np.array([30.0, 50.0, 20.0])                     # top layer first; bottom layer is 20 thick
    owner, depth = F.heights(th, [0.0, 20.0, 70.0, 100.0, 45.0])
    assert owner.tolist() == [2, 1, 0, 0, 1]
    assert np.allclose(depth, [20.0, 50.0, 30.0, 0.0, 25.0])
    z, owner, depth = F.height_points(3, th)
    assert np.allclose(z, [0, 10, 20, 20, 45, 70, 70, 85, 100])
    assert owner.tolist() == [2, 2, 2, 1, 1, 1, 0, 0, 0]
    assert np.allclose(depth, [20, 10, 0, 50, 25, 0, 30, 15, 0])
    with pytest.raises(ValueError):
        F.heights(th, [-1.0])
    with pytest.raises(ValueError):
        F.heights(th, [100.5])
    assert np.allclose(F.axis_points(3, 500.0, 'x'), [-250.0, 0.0, 250.0])


def test_a_result_without_fields_refuses_to_sample():
    res = rcwa.Result(None, None, (None, None), (None, None), None, (), {})
    with pytest.raises(rcwa.UnsupportedFeatureError) as e:
        res.field(x=[0.0], y=[0.0], z=[0.0])
    assert e.value.code == 'outputs.unavailable' and e.value.path == 'outputs.fields'


def _problem(c, pol):
    st, th = np.asarray(c['structure'], complex), np.asarray(c['thickness'], float)
    layers = tuple(rcwa.Layer(thickness=float(t), epsilon=e) for e, t in zip(st[::-1], th[::-1]))
    return rcwa.Problem(units=rcwa.Units('nm'),
                        stack=rcwa.Stack(period=tuple(float(p) for p in c['period']),
                                         top=rcwa.Material(epsilon=complex(c['eps_top'])),
                                         bottom=rcwa.Material(epsilon=complex(c['eps_bot'])), layers=layers),
                        excitation=rcwa.Excitation(wavelength=float(c['wavelength']), sources=(
                            rcwa.PlaneWave(polarization=pol, theta=float(c['theta']), phi=float(c['phi']),
                                           amplitude=float(c[f'amplitude_{pol}'])),)),
                        outputs=rcwa.Outputs(fields=True))


@pytest.mark.gpu
@pytest.mark.parametrize('name', NAMES)
def test_lifecycle_fields_match_the_reference(name):
    """rcwa.run(..., Outputs(fields=True)).field(x=, y=, z=) with the kernels' modes, within
    1e-10 of the reference's own phasors (E and H each against their largest magnitude)."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    for pol in ('s', 'p'):
        res = rcwa.run(_problem(c, pol), numerics=rcwa.Numerics(orders=(hu, hv)))
        f = res.field(x=c['x'], y=c['y'], z=c['z'])
        assert f.values.shape == (1, len(c['z']), len(c['y']), len(c['x']), 6)
        assert f.values.device.type == 'cuda' and f.components == F.COMPONENTS
        _check(f.values[0].cpu().numpy(), c[f'field_{pol}'][0], 1e-10, (name, pol))
        fl = res.field(x=c['x'], y=c['y'], z=c['z'], reconstruction='lalanne')
        _check(fl.values[0].cpu().numpy(), c[f'field_lalanne_{pol}'][0], 1e-10, (name, pol, 'lalanne'))
        for side in ('top', 'bottom'):
            want = c[f'boundary_{side}_total_{pol}'][0]
            got = res.boundary_fields(side=side, x=c['x'], y=c['y']).values[0].cpu().numpy()
            _check(got, want, 1e-10, (name, pol, side))


def _oracle_layer_modes(conv, pair_layer, kx, ky, precision='double', handle=None):
    """A CPU stand-in for engine.layer_modes: the oracle's eigen-solve of each pair's layer."""
    out = [[], [], [], []]
    for p, l in enumerate(np.asarray(pair_layer).reshape(-1)):
        kxg, kyg = kx[p].numpy() + 0j, ky[p].numpy() + 0j
        W, V, q, w, _ = O.layer_modes_2d(kxg, kyg, *(conv.slot(k)[int(l)].numpy() for k in range(3)))
        for lst, a in zip(out, (w, q, W, V)):
            lst.append(torch.as_tensor(a))
    w, q, W, V = (torch.stack(x) for x in out)
    return w, q, W, V, torch.zeros(len(out[0]), dtype=torch.int32)


def _solve_ports(inp, b, hu, hv, device):
    from wavebit_gb300.adjoint import ports
    return ports(float(inp.wavelength[b]), tuple(float(v) for v in inp.period[b]), float(inp.theta[b]),
                 float(inp.phi[b]), complex(inp.eps_top[b]), complex(inp.eps_bot[b]), hu, hv, device)


def _torch_layer_amplitudes(W, V, q, inp, hu, hv, C, handle=None):
    """A CPU stand-in for engine.layer_amplitudes: the torch restatement, solve by solve."""
    B, L = inp.B, inp.L
    out = [[], [], [], [], []]
    for b in range(B):
        pv = _solve_ports(inp, b, hu, hv, W.device)
        modes = [(W[b * L + l], V[b * L + l], q[b * L + l]) for l in range(L)]
        faces, cref, ctrn = F.layer_faces(modes, inp.thickness[b].tolist(), 2 * np.pi / float(inp.wavelength[b]),
                                          pv, C[b])
        for j in range(3):
            out[j].append(torch.stack([f[j] for f in faces]))
        out[3].append(cref)
        out[4].append(ctrn)
    return tuple(torch.stack(x) for x in out) + (torch.zeros(B, dtype=torch.int32),)


def _torch_etm_solve(W, V, q, inp, hu, hv, amplitudes=False, handle=None):
    """A CPU stand-in for engine.etm_solve: the torch restatement of the ETM, solve by solve."""
    from wavebit_gb300 import etm as E
    B, L = inp.B, inp.L
    out = [[], [], []]
    for b in range(B):
        pv = _solve_ports(inp, b, hu, hv, W.device)
        modes = [(W[b * L + l], V[b * L + l], q[b * L + l]) for l in range(L)]
        res = E.etm_solve(modes, inp.thickness[b].tolist(), 2 * np.pi / float(inp.wavelength[b]), pv,
                          tuple(complex(v) for v in inp.pol[b]), 2 * hu + 1, 2 * hv + 1, amplitudes=True)
        for lst, a in zip(out, res):
            lst.append(a)
    R, T, amps = (torch.stack(x) for x in out)
    return (R, T, torch.zeros(B, dtype=torch.int32)) + ((amps,) if amplitudes else ())


def use_cpu_stages(monkeypatch):
    """Stand the oracle in for stage B and the torch restatements for the cascade kernels the
    lifecycle calls on given modes, so that its bookkeeping runs on the CPU."""
    from wavebit_gb300 import engine
    monkeypatch.setattr(engine, 'layer_modes', _oracle_layer_modes)
    monkeypatch.setattr(engine, 'layer_amplitudes', _torch_layer_amplitudes)
    monkeypatch.setattr(engine, 'etm_solve', _torch_etm_solve)


@pytest.mark.parametrize('name', ['crossed_0', 'symmetric_pillar'])
def test_lifecycle_field_states_on_the_cpu(name, monkeypatch):
    """Prepared._field_states and Result.field with the stage-B kernel replaced by the oracle on
    the CPU: the per-(wavelength, layer) bookkeeping, slots, heights and source amplitude."""
    from wavebit_gb300 import engine
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    st = np.asarray(c['structure'], complex)
    conv_np = O.to_conv_mat_raster_sampled(st, hu, hv)
    conv = engine.ConvStack.from_matrices(*(torch.as_tensor(a) for a in conv_np), hu, hv)
    use_cpu_stages(monkeypatch)
    for pol in ('s', 'p'):
        r = rcwa._resolve(_problem(c, pol), rcwa.Numerics(orders=(hu, hv)))
        p = rcwa.Prepared.__new__(rcwa.Prepared)
        p.handle = None
        L = st.shape[0]
        wl = np.asarray(r['wavelengths'], dtype=np.float64)
        th = np.full(len(wl), r['theta'])
        states = p._field_states(r, conv, np.tile(np.arange(L), (len(wl), 1)), wl, th)
        res = rcwa.Result(None, None, (None, None), (None, None), None, tuple(wl), {}, None, None, states,
                          (np.asarray(r['thickness']), r['period'], r['amplitude'], False, (hu, hv)))
        f = res.field(x=c['x'], y=c['y'], z=c['z'])
        _check(f.values[0].numpy(), c[f'field_{pol}'][0], 1e-12, (name, pol))
        with pytest.raises(rcwa.ValidationError) as e:
            res.field(x=c['x'], y=c['y'], z=[-5.0])
        assert e.value.code == 'field.coordinates'
        fl = res.field(x=c['x'], y=c['y'], z=c['z'], reconstruction='lalanne')
        _check(fl.values[0].numpy(), c[f'field_lalanne_{pol}'][0], 1e-12, (name, pol, 'lalanne'))
        assert fl.metadata['reconstruction'] == 'lalanne'
        with pytest.raises(rcwa.UnsupportedFeatureError) as e:
            res.field(x=c['x'], y=c['y'], z=c['z'], reconstruction='splitw')
        assert e.value.code == 'field.reconstruction'
        with pytest.raises(rcwa.ValidationError) as e:
            res.field(x=c['x'], y=c['y'], z=c['z'], reconstruction='li')
        assert e.value.code == 'field.reconstruction'
        counts = res.field(x=3, y=2, z=2)
        assert counts.values.shape == (1, 2 * L, 2, 3, 6)
        b = res.boundary_fields(side='top', x=c['x'], y=c['y'], part='outgoing')
        _check(b.values[0].numpy(), c[f'boundary_top_outgoing_{pol}'][0], 1e-12, (name, pol, 'boundary'))
        assert b.metadata['side'] == 'top' and b.values.shape == (1, len(c['y']), len(c['x']), 6)
        with pytest.raises(rcwa.ValidationError) as e:
            res.boundary_fields(side='left', x=c['x'], y=c['y'])
        assert e.value.code == 'field.side'


@pytest.mark.parametrize('name', NAMES)
def test_count_sampling_matches_the_reference_on_the_cpu(name):
    """x=3, y=2, z=3: a centred grid across the cell and every layer's own heights from its bottom
    face to its top face (an internal face twice, the lower layer's first), field_result.py:85-106,
    375-398 -- the heights and the phasors against the reference's."""
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    st = np.asarray(c['structure'], complex)
    th = np.asarray(c['thickness'], float)
    wl, per = float(c['wavelength']), tuple(float(p) for p in c['period'])
    pv = ports(wl, per, float(c['theta']), float(c['phi']), complex(c['eps_top']), complex(c['eps_bot']), hu, hv, 'cpu')
    conv = O.to_conv_mat_raster_sampled(st, hu, hv)
    modes, epz = [], []
    for i in range(st.shape[0]):
        W, V, q, _, _ = O.layer_modes_2d(pv['kx'].numpy() + 0j, pv['ky'].numpy() + 0j, conv[0][i], conv[1][i], conv[2][i])
        modes.append(tuple(torch.as_tensor(a) for a in (W, V, q)))
        epz.append(torch.as_tensor(conv[2][i]))
    for pol in ('s', 'p'):
        state = F.build_state(modes, epz, th, wl, pv, O.polarization_pair(pol), hu, hv)
        z, owner, depth = F.height_points(3, th)
        assert np.allclose(z, c[f'counts_z_{pol}'], rtol=0, atol=1e-9)
        got = F.synthesize(state, owner, depth, F.axis_points(3, per[0], 'x'), F.axis_points(2, per[1], 'y'),
                           float(c[f'amplitude_{pol}'])).numpy()
        _check(got, c[f'field_counts_{pol}'][0], 1e-12, (name, pol))


@pytest.mark.parametrize('name', NAMES)
def test_boundary_fields_match_the_reference_on_the_cpu(name):
    """The half-spaces' waves on both faces (incoming, outgoing, total) from the field state built
    on the CPU with the oracle's modes, against the reference's result.boundary_fields."""
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    st = np.asarray(c['structure'], complex)
    th = np.asarray(c['thickness'], float)
    wl, per = float(c['wavelength']), tuple(float(p) for p in c['period'])
    pv = ports(wl, per, float(c['theta']), float(c['phi']), complex(c['eps_top']), complex(c['eps_bot']), hu, hv, 'cpu')
    conv = O.to_conv_mat_raster_sampled(st, hu, hv)
    modes, epz = [], []
    for i in range(st.shape[0]):
        W, V, q, _, _ = O.layer_modes_2d(pv['kx'].numpy() + 0j, pv['ky'].numpy() + 0j, conv[0][i], conv[1][i], conv[2][i])
        modes.append(tuple(torch.as_tensor(a) for a in (W, V, q)))
        epz.append(torch.as_tensor(conv[2][i]))
    for pol in ('s', 'p'):
        state = F.build_state(modes, epz, th, wl, pv, O.polarization_pair(pol), hu, hv)
        for side in ('top', 'bottom'):
            for part in ('incoming', 'outgoing', 'total'):
                got = F.expand_boundary(state, side, part, c['x'], c['y'], float(c[f'amplitude_{pol}'])).numpy()
                want = c[f'boundary_{side}_{part}_{pol}'][0]
                if np.abs(want).max() == 0:
                    assert np.abs(got).max() == 0, (name, pol, side, part)
                else:
                    _check(got, want, 1e-12, (name, pol, side, part))


@pytest.mark.parametrize('name', NAMES)
def test_lalanne_rule_matches_the_reference_on_the_cpu(name):
    """reconstruction='lalanne' (E_x, E_y of patterned layers from the D series line by line,
    P. Lalanne and M. P. Jurek 1998) on the CPU with the oracle's modes, against the reference's."""
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    st = np.asarray(c['structure'], complex)
    th = np.asarray(c['thickness'], float)
    wl, per = float(c['wavelength']), tuple(float(p) for p in c['period'])
    pv = ports(wl, per, float(c['theta']), float(c['phi']), complex(c['eps_top']), complex(c['eps_bot']), hu, hv, 'cpu')
    conv = O.to_conv_mat_raster_sampled(st, hu, hv)
    modes, epz = [], []
    for i in range(st.shape[0]):
        W, V, q, _, _ = O.layer_modes_2d(pv['kx'].numpy() + 0j, pv['ky'].numpy() + 0j, conv[0][i], conv[1][i], conv[2][i])
        modes.append(tuple(torch.as_tensor(a) for a in (W, V, q)))
        epz.append(torch.as_tensor(conv[2][i]))
    for pol in ('s', 'p'):
        state = F.build_state(modes, epz, th, wl, pv, O.polarization_pair(pol), hu, hv, rasters=list(st))
        z, owner, depth = F.height_points(c['z'], th)
        got = F.synthesize(state, owner, depth, c['x'], c['y'], float(c[f'amplitude_{pol}']), 'lalanne', per,
                           (hu, hv)).numpy()
        _check(got, c[f'field_lalanne_{pol}'][0], 1e-11, (name, pol))
        # counts put x samples on both cell edges, and every internal face in both layers
        xs, ys = F.axis_points(3, per[0], 'x'), F.axis_points(2, per[1], 'y')
        _, owner, depth = F.height_points(3, th)
        got = F.synthesize(state, owner, depth, xs, ys, float(c[f'amplitude_{pol}']), 'lalanne', per,
                           (hu, hv)).numpy()
        _check(got, c[f'field_counts_lalanne_{pol}'][0], 1e-11, (name, pol, 'counts'))


def test_coordinate_rules_follow_the_reference():
    """Counts are positive integers; explicit coordinates are nonempty 1-D finite real arrays
    (a torch tensor too), and a complex value with an imaginary part is refused rather than
    truncated (results.py:47-69)."""
    assert np.array_equal(F.axis_points(torch.tensor([0.5, -1.0]), 2.0, 'x'), [0.5, -1.0])
    assert np.array_equal(F.axis_points(np.array([1 + 0j, 2 + 0j]), 2.0, 'x'), [1.0, 2.0])
    assert np.allclose(F.axis_points(3, 2.0, 'x'), [-1.0, 0.0, 1.0])
    for bad in ([1 + 1e-3j], [[0.0, 1.0]], [], [np.nan], ['a'], 0, True):
        with pytest.raises(ValueError):
            F.axis_points(bad, 2.0, 'x')
    for bad in ([[0.1, 0.2]], [0.1 + 1j]):
        with pytest.raises(ValueError):
            F.height_points(bad, np.array([1.0]))


@pytest.mark.gpu
@pytest.mark.parametrize('name', ['crossed_0', 'symmetric_pillar'])
def test_layer_amplitude_kernels_match_the_torch_recursion(name):
    """wb_layer_amplitudes (the cascade kernels' recursion with the per-layer amplitudes kept)
    against the torch restatement on the same modes, two wavelengths and three incidence columns
    in one batch: every layer's plus, minus_top and minus_bottom and the reflected and
    transmitted columns to 1e-12 of their largest entry."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import engine
    from test_etm import _given_modes
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    N = (2 * hu + 1) * (2 * hv + 1)
    wls = [float(np.asarray(c['wavelength']).reshape(-1)[0]) * f for f in (1.0, 1.11)]
    rng = np.random.default_rng(5)
    Cn = rng.standard_normal((2, 2 * N, 3)) + 1j * rng.standard_normal((2, 2 * N, 3))
    W, V, q, inp = _given_modes(c, wls, 'cuda')
    got = engine.layer_amplitudes(W, V, q, inp, hu, hv, torch.as_tensor(Cn, device='cuda'))
    W0, V0, q0, inp0 = _given_modes(c, wls, 'cpu')
    want = _torch_layer_amplitudes(W0, V0, q0, inp0, hu, hv, torch.as_tensor(Cn))
    assert int(got[5].abs().sum()) == 0
    for a, b, label in zip(got[:5], want[:5], ('plus', 'minus_top', 'minus_bottom', 'cref', 'ctrn')):
        assert a.shape == b.shape, label
        assert float((a.cpu() - b).abs().max()) <= 1e-12 * float(b.abs().max()), (name, label)
