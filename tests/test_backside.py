"""Incidence from below (``PlaneWave(side='bottom')``): the scene lit through its substrate,
angles in the substrate, R back into it, T into the superstrate. The lifecycle solves the
z-mirrored scene lit from above and maps fields and readings back; these tests hold it to the
reference's own bottom-lit runs (``ref_backside.npz``) and to RETICOLO's bottom-incidence orders."""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from oracle import rcwa_oracle as O
from wavebit_gb300 import rcwa

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
NAMES = list(np.load(os.path.join(GOLDEN, 'ref_backside.npz'))['names'])
RETICOLO = list(np.load(os.path.join(GOLDEN, 'reticolo_cases.npz'))['names'])
POLS = (('s', 's'), ('mix', (0.6, 0.8j)))


def _case(name, fixture='ref_backside.npz'):
    d = np.load(os.path.join(GOLDEN, fixture))
    return {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}


def _problem(c, pol, fields=True):
    st, th = np.asarray(c['structure'], complex), np.asarray(c['thickness'], float)
    layers = tuple(rcwa.Layer(thickness=float(t), epsilon=e) for e, t in zip(st[::-1], th[::-1]))
    return rcwa.Problem(units=rcwa.Units('nm'),
                        stack=rcwa.Stack(period=tuple(float(p) for p in c['period']),
                                         top=rcwa.Material(epsilon=complex(c['eps_top'])),
                                         bottom=rcwa.Material(epsilon=complex(c['eps_bot'])), layers=layers),
                        excitation=rcwa.Excitation(wavelength=float(c['wavelength']), sources=(
                            rcwa.PlaneWave(side='bottom', polarization=pol, theta=float(c['theta']),
                                           phi=float(c['phi']), amplitude=2.5),)),
                        outputs=rcwa.Outputs(fields=fields))


def _close(got, want, tol, label):
    scale = max(np.abs(want).max(), 1e-300)
    assert np.abs(got - want).max() <= tol * scale, label


def _check_fields(got, want, tol, label):
    for part in (slice(0, 3), slice(3, 6)):
        _close(got[..., part], want[..., part], tol, (label, part))


def _check_result(res, c, tag, tol, name):
    """R, T, every per-order reading, the fields at points and both faces' boundary waves."""
    dev_np = lambda t: t.detach().cpu().numpy()
    _close(dev_np(res.R[0]), c[f'R_{tag}'], tol, (name, tag, 'R'))
    _close(dev_np(res.T[0]), c[f'T_{tag}'], tol, (name, tag, 'T'))
    p_inc = float(c[f'{tag}_reflected_incident_power'][0])
    for port in ('reflected', 'transmitted'):
        o = res.outputs[port]
        key = f'{tag}_{port}'
        assert o.reference['port'] == str(c[f'{key}_port']) and o.reference['incident_port'] == 'bottom'
        assert o.reference['plane'][0] == pytest.approx(float(c[f'{key}_plane'][0]), abs=1e-9)
        assert abs(float(dev_np(o.reference['incident_power'])[0]) - p_inc) <= tol * p_inc
        # s and p ratios scaled together: a ratio the polarization leaves empty is round-off
        sp = np.abs(np.stack([c[f'{key}_amplitude_ratio_s'], c[f'{key}_amplitude_ratio_p']])).max()
        for comp in ('s', 'p'):
            got = dev_np(getattr(o, f'amplitude_ratio_{comp}')[0])
            assert np.abs(got - c[f'{key}_amplitude_ratio_{comp}']).max() <= tol * sp, (name, key, comp)
        for field_ in ('amplitude_ratio_xyz', 'k_parallel', 'k_normal'):
            _close(dev_np(getattr(o, field_)[0]), c[f'{key}_{field_}'], tol, (name, key, field_))
        assert np.abs(dev_np(o.power[0]) - c[f'{key}_power']).max() <= tol * p_inc, (name, key, 'power')
    f = res.field(x=c['x'], y=c['y'], z=c['z'])
    _check_fields(dev_np(f.values[0]), c[f'field_{tag}'][0], tol, (name, tag, 'field'))
    f = res.field(x=c['x'], y=c['y'], z=c['z'], reconstruction='lalanne')
    _check_fields(dev_np(f.values[0]), c[f'field_lalanne_{tag}'][0], 10 * tol, (name, tag, 'lalanne'))
    for side in ('top', 'bottom'):
        for part in ('incoming', 'outgoing'):
            b = res.boundary_fields(side=side, x=c['x'], y=c['y'], part=part)
            want = c[f'boundary_{side}_{part}_{tag}'][0]
            if np.abs(want).max() == 0:
                assert np.abs(dev_np(b.values[0])).max() == 0, (name, tag, side, part)
            else:
                _check_fields(dev_np(b.values[0]), want, tol, (name, tag, side, part))


@pytest.mark.parametrize('name', NAMES)
def test_the_mirrored_scene_is_the_reference_lit_from_below(name):
    """The oracle's solve of the z-mirrored scene (layers in reverse, half-spaces swapped, the same
    angles) against the reference's bottom-lit R and T (incidence_side contract)."""
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    st, th = np.asarray(c['structure'], complex), np.asarray(c['thickness'], float)
    for tag, pol in POLS:
        o = O.solve_stack(st[::-1], th[::-1], float(c['wavelength']), tuple(c['period']), hu, hv, float(c['theta']),
                          float(c['phi']), complex(c['eps_bot']), complex(c['eps_top']), pol)
        _close(o['R'][0], c[f'R_{tag}'], 1e-12, (name, tag))
        _close(o['T'][0], c[f'T_{tag}'], 1e-12, (name, tag))


@pytest.mark.parametrize('name', RETICOLO)
def test_the_mirrored_scene_matches_reticolo_from_below(name):
    """RETICOLO's own bottom-incidence orders (its inc_bottom, at the top side's in-plane
    wavevector: theta_bottom = asin(n_top sin(theta) / n_bot)); reflection goes back into the
    substrate, so its propagating orders are the top side's transmitted ones, and the reverse."""
    c = _case(name, 'reticolo_cases.npz')
    h, per = int(c['h']), float(c['period'])
    st = np.asarray(c['structure'], complex)
    n_top, n_bot = np.sqrt(complex(c['top'])).real, np.sqrt(complex(c['bot'])).real
    theta_b = float(np.arcsin(n_top * np.sin(float(c['theta'])) / n_bot))
    o = O.solve_stack(st[::-1], np.asarray(c['thickness'], float)[::-1], float(c['wavelength']), (per, per), h, 0,
                      theta_b, float(c['phi']), complex(c['bot']), complex(c['top']), str(c['pol']))
    for side, idx_key, arr in (('ri_bot', 'idx_ti', o['R'][0].ravel()), ('ti_bot', 'idx_ri', o['T'][0].ravel())):
        idx = c[idx_key]
        assert np.abs(arr[idx] - c[f'de_{side}']).max() < 1e-11, (name, side)
        assert np.abs(np.delete(arr, idx)).max(initial=0.0) < 1e-14, (name, side)


@pytest.mark.parametrize('name', NAMES)
def test_bottom_lit_scattering_matrix_is_the_mirrored_scenes(name):
    """The reference's S of a bottom-lit run is incidence-relative (its cascade's blocks read from
    the other end, the entry port in the substrate): the four blocks of the mirrored scene's
    cascade, as the lifecycle exports them, to 1e-12."""
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    st, th = np.asarray(c['structure'], complex), np.asarray(c['thickness'], float)
    o = O.solve_stack(st[::-1], th[::-1], float(c['wavelength']), tuple(c['period']), hu, hv, float(c['theta']),
                      float(c['phi']), complex(c['eps_bot']), complex(c['eps_top']), 's')
    for blk, m in zip(('S11', 'S12', 'S21', 'S22'), O.exported_scattering(o['S'], hu, hv)):
        assert np.abs(m - c[blk]).max() <= 1e-12 * max(1.0, np.abs(c[blk]).max()), (name, blk)
    assert complex(c['entry_index']) == pytest.approx(np.sqrt(complex(c['eps_bot'])), rel=1e-15)


def test_bottom_incidence_resolves_to_the_mirrored_scene():
    c = _case('crossed_1')
    r = rcwa._resolve(_problem(c, 's'), rcwa.Numerics(orders=(1, 1)))
    st, th = np.asarray(c['structure'], complex), np.asarray(c['thickness'], float)
    assert r['side'] == 'bottom' and r['eps_top'] == complex(c['eps_bot']) and r['eps_bot'] == complex(c['eps_top'])
    assert all(np.array_equal(a, b) for a, b in zip(r['rasters'], st[::-1]))
    assert np.array_equal(r['thickness'], th[::-1])


@pytest.mark.parametrize('name', NAMES)
def test_lifecycle_from_below_on_the_cpu(name, monkeypatch):
    """The whole bottom-lit lifecycle -- resolve, solve (the ETM over the oracle's modes in place of
    the stage-B kernel), amplitudes, readings, fields and boundary fields mapped back to the
    scene's frame -- against the reference's own bottom-lit run."""
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
        res = p._solve_etm(r, conv, np.tile(np.arange(len(r['rasters'])), (1, 1)), fields=True)
        _check_result(res, c, tag, 1e-11, name)


@pytest.mark.gpu
@pytest.mark.parametrize('name', NAMES)
def test_lifecycle_from_below_on_the_gpu(name):
    """rcwa.run of a bottom-lit scene through the kernels (FP64), against the reference's run."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    for tag, pol in POLS:
        res = rcwa.run(_problem(c, pol), numerics=rcwa.Numerics(orders=(hu, hv)))
        _check_result(res, c, tag, 1e-10, name)
    prob = _problem(c, 's', fields=False)
    prob = rcwa.Problem(units=prob.units, stack=prob.stack, excitation=prob.excitation,
                        outputs=rcwa.Outputs(scattering=True))
    S = rcwa.run(prob, numerics=rcwa.Numerics(orders=(hu, hv))).scattering[0]
    for blk in ('S11', 'S12', 'S21', 'S22'):
        want = c[blk]
        assert np.abs(getattr(S, blk).cpu().numpy() - want).max() <= 1e-10 * max(1.0, np.abs(want).max()), (name, blk)
    assert S.entry_port.refractive_index == pytest.approx(np.sqrt(complex(c['eps_bot'])), rel=1e-15)


def test_a_preparation_takes_the_same_scene_lit_from_the_other_side():
    """Which side the source lights is not structural: the layout a preparation fixes is read in
    the scene's own layer order, so a stack of rasters of different shapes lit from below keeps
    the layout of the same stack lit from above; a changed raster shape is still refused."""
    st = (rcwa.Layer(thickness=50.0, epsilon=np.ones((2, 3)) * 2.0), rcwa.Layer(thickness=60.0, epsilon=np.ones((4, 5))))

    def problem(side, layers=st):
        return rcwa.Problem(stack=rcwa.Stack(period=(400.0, 500.0), top=rcwa.Material(1.0),
                                             bottom=rcwa.Material(2.25), layers=layers),
                            excitation=rcwa.Excitation(wavelength=600.0, sources=(
                                rcwa.PlaneWave(side=side, theta=0.2),)))
    num = rcwa.Numerics(orders=(1, 1))
    top, bottom = problem('top'), problem('bottom')
    layout = rcwa.Prepared._layout
    assert layout(top, rcwa._resolve(top, num)) == layout(bottom, rcwa._resolve(bottom, num))
    other = problem('bottom', (st[0], rcwa.Layer(thickness=60.0, epsilon=np.ones((4, 4)))))
    assert layout(other, rcwa._resolve(other, num)) != layout(top, rcwa._resolve(top, num))


def test_the_operator_contract_is_the_scene_not_the_lit_side():
    from wavebit_gb300 import operators
    c = _case('crossed_1')
    lit_below = _problem(c, 's', fields=False)
    lit_above = rcwa.Problem(units=lit_below.units, stack=lit_below.stack, excitation=rcwa.Excitation(
        wavelength=lit_below.excitation.wavelength, sources=(rcwa.PlaneWave(side='top', theta=0.1),)))
    num = rcwa.Numerics(orders=(1, 1))
    assert operators._contract(lit_below, num) == operators._contract(lit_above, num)


@pytest.mark.gpu
def test_operators_keep_the_scenes_layer_order_from_below():
    """rcwa.operators.assemble lists the layers top first whichever side is lit, and solve with
    those operators is rcwa.run of the bottom-lit problem."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import operators
    c = _case('crossed_4')
    hu, hv = (int(v) for v in c['orders'])
    num = rcwa.Numerics(orders=(hu, hv))
    lit_below = _problem(c, 's', fields=False)
    lit_above = rcwa.Problem(units=lit_below.units, stack=lit_below.stack, excitation=rcwa.Excitation(
        wavelength=lit_below.excitation.wavelength, sources=(rcwa.PlaneWave(side='top', theta=0.1),)))
    ops_b, ops_t = operators.assemble(lit_below, numerics=num), operators.assemble(lit_above, numerics=num)
    for a, b in zip(ops_b.epsilon[0][:3], ops_t.epsilon[0][:3]):
        assert torch.equal(a, b)
    got = operators.solve(lit_below, ops_b)
    want = rcwa.run(lit_below, numerics=num)
    assert torch.abs(got.R - want.R).max().item() <= 1e-12 and torch.abs(got.T - want.T).max().item() <= 1e-12
