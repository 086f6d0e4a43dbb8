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
    (dict(source=rcwa.PlaneWave(side='left')), rcwa.ValidationError, 'source.side', 'source.side'),
    (dict(source=rcwa.PlaneWave(side='bottom'), bottom=rcwa.Material(-5.0 + 0.2j)), rcwa.UnsupportedFeatureError,
     'feature.unsupported', 'stack.bottom'),
    (dict(source=rcwa.PlaneWave(kx=0.1)), rcwa.UnsupportedFeatureError, 'feature.unsupported',
     'excitation.sources[0]'),
    (dict(source=rcwa.PlaneWave(theta=2.0)), rcwa.ValidationError, 'input.invalid', 'excitation.sources[0].theta'),
    (dict(source=rcwa.PlaneWave(phi=float('nan'))), rcwa.ValidationError, 'input.invalid', 'excitation.sources[0].phi'),
    (dict(source=rcwa.PlaneWave(polarization='x')), rcwa.ValidationError, 'input.invalid',
     'excitation.sources[0].polarization'),
    (dict(source=rcwa.PlaneWave(polarization=(0.0, 0.0))), rcwa.ValidationError, 'input.invalid',
     'excitation.sources[0].polarization'),
    (dict(wavelength=float('inf')), rcwa.ValidationError, 'input.invalid', 'excitation.wavelength'),
    (dict(wavelength=()), rcwa.ValidationError, 'input.invalid', 'excitation.wavelength'),
])
def test_refusals_carry_the_reference_classes_and_codes(kw, error, code, path):
    with pytest.raises(error) as e:
        rcwa._resolve(_problem(**kw), rcwa.Numerics(orders=(1, 1)))
    assert e.value.code == code and e.value.path == path


@pytest.mark.parametrize('numerics,path', [
    (rcwa.Numerics(orders=(-1, 2)), 'numerics.orders'),
    (rcwa.Numerics(orders=(2,)), 'numerics.orders'),
    (rcwa.Numerics(orders=(28, 28)), 'numerics.orders'),
    (rcwa.Numerics(orders=(0, 43)), 'numerics.orders'),
])
def test_bad_orders_are_refused(numerics, path):
    with pytest.raises(rcwa.ValidationError) as e:
        rcwa._resolve(_problem(), numerics)
    assert e.value.path == path


@pytest.mark.parametrize('field,value', [('algorithm', 'fdtd'), ('fourier_coefficients', 'shape'),
                                         ('factorization', 'nvf'), ('factorization', 'laurent'),
                                         ('li_nesting', 'alternating')])
def test_numerics_outside_the_path_are_unsupported(field, value):
    num = rcwa.Numerics(orders=(1, 1), **{field: value})
    with pytest.raises(rcwa.UnsupportedFeatureError):
        rcwa._resolve(_problem(), num)


@pytest.mark.parametrize('value', ['sampled', 'integrated', 'INTEGRATED', None])
def test_both_coefficient_rules_are_admitted(value):
    num = rcwa.Numerics(orders=(1, 1), fourier_coefficients=value)
    rcwa._resolve(_problem(), num)
    assert rcwa._integrated(num) == (value is not None and value.lower() == 'integrated')


@pytest.mark.parametrize('value', [True, 0, -1e-12, float('nan'), float('inf'), '1e-12'])
def test_detuning_is_a_positive_relative_step(value):
    """numerics.py:127-131 of the reference: None or a positive finite float / int."""
    with pytest.raises(rcwa.ValidationError) as e:
        rcwa._resolve(_problem(), rcwa.Numerics(orders=(1, 1), detuning=value))
    assert e.value.code == 'numerics.detuning' and e.value.path == 'numerics.detuning'


def test_a_detuning_step_is_admitted():
    rcwa._resolve(_problem(), rcwa.Numerics(orders=(1, 1), detuning=1e-12))
    rcwa._resolve(_problem(), rcwa.Numerics(orders=(1, 1), detuning=1))


def test_compression_matches_the_oracle_record():
    """The host compression of the integrated path against the oracle's restatement of
    compression_indices, on rasters with runs, isolated pixels and uniform layers."""
    from oracle import rcwa_oracle as O
    rng = np.random.default_rng(7)
    cells = [np.full((5, 7), 2.25 + 0j), np.array([[1.0, 12.25]]), np.ones((1, 1))]
    for _ in range(30):
        ny, nx = rng.integers(1, 25, size=2)
        base = np.where(rng.random((rng.integers(1, 5), rng.integers(1, 5))) < 0.5, 12.25, 1.0 + 0.5j)
        ry = np.sort(rng.integers(0, ny, size=base.shape[0] - 1))
        rx = np.sort(rng.integers(0, nx, size=base.shape[1] - 1))
        cells.append(base[np.searchsorted(ry, np.arange(ny), side='right')][:, np.searchsorted(rx, np.arange(nx), side='right')])
    cells.append(rng.standard_normal((9, 4)) + 0j)          # nothing to compress
    for cell in cells:
        comp, x, y = rcwa.compression(cell)
        ri, ci, ox, oy = O.compression_indices(cell)
        assert np.array_equal(comp, cell[np.ix_(ri, ci)])
        assert np.array_equal(x, ox) and np.array_equal(y, oy)       # bit-identical edges
        assert x[-1] == 1.0 and y[-1] == 1.0


class _FakeInputs:
    def __init__(self, li, th, wl, per, theta, phi, et, eb, pol, device=None):
        self.wl, self.theta = np.asarray(wl, float), np.asarray(theta, float)
        self.B = len(self.wl)


def _fake_solver(rule):
    """A stand-in for engine.solve_batch: R carries the wavelength, T the angle each solve used,
    and ``rule(wl, theta)`` decides its status word."""
    import torch

    def solve(conv, inp, precision='double', amplitudes=False, handle=None):
        R = torch.tensor(inp.wl, dtype=torch.float64).reshape(-1, 1, 1, 1).repeat(1, 3, 1, 1)
        T = torch.tensor(inp.theta, dtype=torch.float64).reshape(-1, 1, 1, 1).repeat(1, 3, 1, 1)
        st = torch.tensor([rule(w, t) for w, t in zip(inp.wl, inp.theta)], dtype=torch.int32)
        return R, T, st
    return solve


def _prepared(detuning):
    p = rcwa.Prepared.__new__(rcwa.Prepared)
    p.numerics, p.precision, p.handle = rcwa.Numerics(orders=(0, 0), detuning=detuning), 'double', None
    r = dict(wavelengths=np.array([600.0, 700.0, 800.0]), rasters=[np.ones((1, 1))], thickness=np.array([100.0]),
             period=(500.0, 500.0), theta=0.3, thetas=np.full(3, 0.3), phi=0.0, eps_top=1.0, eps_bot=1.0,
             pol=(1.0, 0.0), orders=(0, 0))
    return p, r


def test_auto_detune_ladder_moves_the_wavelength_then_the_angle(monkeypatch):
    from wavebit_gb300 import _lib
    g = _lib.WB_ST_GRAZING
    # 700 grazes exactly; 800 grazes until both the wavelength and the angle have moved
    rule = lambda w, t: g if (w == 700.0 or (w in (800.0, 800.0 * (1 + 1e-12)) and t == 0.3)) else 0
    monkeypatch.setattr(rcwa.engine, 'BatchInputs', _FakeInputs)
    monkeypatch.setattr(rcwa.engine, 'solve_batch', _fake_solver(rule))
    p, r = _prepared(rcwa._AUTO_DETUNE_REL)
    with pytest.warns(rcwa.AutoDetuneWarning):
        res = p._solve(r, None, np.zeros((3, 1), int))
    eff = res.diagnostics['effective_wavelengths']
    assert eff == (600.0, 700.0 * (1 + 1e-12), 800.0 * (1 + 1e-12))
    assert res.diagnostics['detuned'] == {1: ('wavelength',), 2: ('wavelength', 'theta')}
    assert not any(res.diagnostics['grazing'])
    assert float(res.R[2].max()) == 800.0 * (1 + 1e-12) and float(res.T[2].max()) == 0.3 * (1 + 1e-12)


def test_a_grazing_mode_without_detuning_warns(monkeypatch):
    """A grazing solve whose cluster the rebuild cannot take (its two products' clusters
    differ in size) keeps its flag and warns."""
    from wavebit_gb300 import _lib
    monkeypatch.setattr(rcwa.engine, 'BatchInputs', _FakeInputs)
    monkeypatch.setattr(rcwa.engine, 'solve_batch', _fake_solver(lambda w, t: _lib.WB_ST_GRAZING if w == 700.0 else 0))
    p, r = _prepared(None)
    seen = []
    monkeypatch.setattr(type(p), '_rebuild_grazing', lambda self, *a: seen.append(list(a[3])) or ())
    with pytest.warns(rcwa.RayleighPointWarning):
        res = p._solve(r, None, np.zeros((3, 1), int))
    assert seen == [[1]]
    assert res.diagnostics['grazing'] == (False, True, False) and res.diagnostics['detuned'] == {}
    assert res.diagnostics['grazing_rebuilt'] == ()


def test_a_defective_graze_is_refused_with_the_reference_code(monkeypatch):
    """A grazing cluster the rebuild finds numerically defective ends the run with the
    reference's NumericalError (rcwa.singular) and its detuning remedy."""
    from wavebit_gb300 import _lib, graze
    monkeypatch.setattr(rcwa.engine, 'BatchInputs', _FakeInputs)
    monkeypatch.setattr(rcwa.engine, 'solve_batch', _fake_solver(lambda w, t: _lib.WB_ST_GRAZING if w == 700.0 else 0))
    p, r = _prepared(None)

    def refuse(self, *a):
        raise rcwa.NumericalError(graze.DEFECTIVE_MESSAGE, code='rcwa.singular')
    monkeypatch.setattr(type(p), '_rebuild_grazing', refuse)
    with pytest.raises(rcwa.NumericalError) as e:
        p._solve(r, None, np.zeros((3, 1), int))
    assert e.value.code == 'rcwa.singular' and 'detuning' in str(e.value)


def test_a_failed_solve_is_a_numerical_error_with_the_reference_code(monkeypatch):
    from wavebit_gb300 import _lib
    monkeypatch.setattr(rcwa.engine, 'BatchInputs', _FakeInputs)
    monkeypatch.setattr(rcwa.engine, 'solve_batch', _fake_solver(lambda w, t: _lib.WB_ST_SINGULAR if w == 600.0 else 0))
    p, r = _prepared(None)
    with pytest.raises(rcwa.NumericalError) as e:
        p._solve(r, None, np.zeros((3, 1), int))
    assert e.value.code == 'rcwa.singular'


def test_check_reports_the_resolved_numerics_and_outputs_without_a_gpu():
    """rcwa.check resolves and estimates on the host (_lifecycle.py:380-420 of the reference):
    the coefficient rule, the connecting algorithm, what the outputs keep and what it costs."""
    p = _problem()
    p = rcwa.Problem(stack=p.stack, excitation=p.excitation, units=p.units,
                     outputs=rcwa.Outputs(fields=True, scattering=False))
    rep = rcwa.check(p, numerics=rcwa.Numerics(orders=(3, 2), fourier_coefficients='integrated',
                                               algorithm='etm'))
    res = rep.resolved
    assert res['fourier_coefficients'] == 'integrated' and res['algorithm'] == 'etm'
    assert res['retained_fields'] is True and res['retained_scattering'] is False
    assert res['length_units'] == 'nm' and res['layer_count'] == 2
    N = 7 * 5
    assert rep.estimates['retained_spatial_modes'] == N
    assert rep.estimates['retained_field_bytes'] == 16 * 1 * 2 * (2 * (2 * N) ** 2 + 4 * N)
    assert rep.estimates['retained_scattering_bytes'] == 0
    assert rep.estimates['device_workspace_bytes'] > 0
    # as in the reference, check reports a refusal as an issue instead of raising it
    rep = rcwa.check(rcwa.Problem(stack=p.stack, excitation=p.excitation, outputs=rcwa.Outputs(scattering=True)),
                     numerics=rcwa.Numerics(orders=(1, 1), algorithm='etm'))
    assert len(rep.issues) == 1 and rep.issues[0].code == 'rcwa.scattering_algorithm'
    assert rep.issues[0].path == 'outputs.scattering' and rep.issues[0].severity == 'error'
    assert rcwa.check(_problem(wavelength=-1.0)).issues[0].code == 'input.invalid'


def test_solve_batch_refuses_layer_indices_outside_the_convolution_stack():
    """The kernels index the convolution stack with layer_index: a batch that would read past it
    is refused on the host, before any device work (engine.solve_batch)."""
    import torch
    conv = rcwa.engine.ConvStack(torch.zeros((2, 3, 9, 9), dtype=torch.complex128), 1, 1)
    for bad in ([[0, 2]], [[-1, 0]]):
        inp = rcwa.engine.BatchInputs(bad, [[10.0, 10.0]], [600.0], [[500.0, 500.0]], [0.0], [0.0], [1.0], [1.0],
                                      [[1.0, 0.0]], device='cpu')
        with pytest.raises(ValueError, match='layer_index'):
            rcwa.engine.solve_batch(conv, inp)
    ok = rcwa.engine.BatchInputs([[0, 1]], [[10.0, 10.0]], [600.0], [[500.0, 500.0]], [0.0], [0.0], [1.0], [1.0],
                                 [[1.0, 0.0]], device='cpu')
    assert ok.index_range == (0, 1)
    with pytest.raises(ValueError, match='pair_layer'):
        rcwa.engine.layer_modes(conv, [0, 2], np.zeros((2, 9)), np.zeros((2, 9)))
    # given modes must cover every (solve, layer) pair the kernels read
    W = torch.zeros((1, 18, 18), dtype=torch.complex128)
    q = torch.zeros((1, 18), dtype=torch.complex128)
    for fn in (rcwa.engine.smm_solve, rcwa.engine.scattering_matrix):
        with pytest.raises(ValueError, match='modes must be'):
            fn(W, W, q, ok, 1, 1)


def test_a_stack_with_no_layers_is_the_bare_interface():
    """The reference solves a stack with no layers through one zero-thickness layer of the top
    medium (results.py:180-189); the mirror resolves it the same way."""
    r = rcwa._resolve(_problem(layers=()), rcwa.Numerics(orders=(1, 1)))
    assert r['bare_interface'] and r['thickness'].tolist() == [0.0]
    assert r['rasters'][0].shape == (1, 1) and r['rasters'][0][0, 0] == r['eps_top']
    res = rcwa.Result(None, None, (None, None), (None, None), None, (600.0,), {}, None, None, (object(),),
                      (r['thickness'], r['period'], 1.0, True))
    with pytest.raises(rcwa.ValidationError) as e:
        res.field(x=[0.0], y=[0.0], z=[0.0])
    assert e.value.code == 'field.coordinates'


def test_a_prepared_run_refuses_a_changed_layout_and_takes_new_values():
    """Prepared.run(problem) keeps the reference's reuse contract (_adapt.py:633-640): values are
    live, the declaration layout is not (code prepared.structure)."""
    base = _problem()
    p = rcwa.Prepared.__new__(rcwa.Prepared)
    p.problem, p.numerics = base, rcwa.Numerics(orders=(1, 1))
    p.resolved = rcwa._resolve(base, p.numerics)
    # new values in the same layout: accepted
    moved = _problem(wavelength=700.0, layers=(rcwa.Layer(thickness=150.0, epsilon=np.array([[1.0, 9.0], [9.0, 1.0]])),
                                               rcwa.Layer(thickness=60.0, epsilon=3.1)))
    p._check_layout(moved, rcwa._resolve(moved, p.numerics))
    for changed, path in ((_problem(layers=(rcwa.Layer(thickness=80.0, epsilon=2.25),)), 'stack.layers'),
                          (_problem(layers=(rcwa.Layer(thickness=120.0, epsilon=np.ones((3, 2))),
                                            rcwa.Layer(thickness=80.0, epsilon=2.25))), 'stack.layers'),
                          (_problem(wavelength=(600.0, 640.0)), 'excitation')):
        with pytest.raises(rcwa.IncompatibleProblemError) as e:
            p._check_layout(changed, rcwa._resolve(changed, p.numerics))
        assert e.value.code == 'prepared.structure' and e.value.path == path
    asked = rcwa.Problem(stack=base.stack, excitation=base.excitation, units=base.units,
                         outputs=rcwa.Outputs(fields=True))
    with pytest.raises(rcwa.IncompatibleProblemError) as e:
        p._check_layout(asked, rcwa._resolve(asked, p.numerics))
    assert e.value.path == 'outputs'


def test_validate_reports_instead_of_raising():
    base = _problem()
    p = rcwa.Prepared.__new__(rcwa.Prepared)
    p.problem, p.numerics, p.precision = base, rcwa.Numerics(orders=(1, 1)), 'double'
    p.resolved = rcwa._resolve(base, p.numerics)
    ok = p.validate(base)
    assert ok.issues == () and ok.resolved['layer_count'] == 2
    bad = p.validate(_problem(layers=(rcwa.Layer(thickness=80.0, epsilon=2.25),)))
    assert bad.issues[0].code == 'prepared.structure' and bad.issues[0].path == 'stack.layers'


def test_diffraction_orders_carry_the_reference_amplitude_ratios():
    """outputs['reflected'|'transmitted'] from amplitudes laid out as the efficiency kernel writes
    them (B, 3 columns, (r_s, r_p, t_s, t_p), N, about the corner), here the oracle's, against the
    reference's own published ratios (mixed (0.6, 0.8i) incidence)."""
    import os
    import torch
    from oracle import rcwa_oracle as O
    d = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'ref_amplitudes.npz'))
    for name in ('crossed_1', 'crossed_2'):
        c = {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}
        hu, hv = (int(v) for v in c['orders'])
        o = O.solve_stack(c['structure'], c['thickness'], float(c['wavelength']), tuple(c['period']), hu, hv,
                          float(c['theta']), float(c['phi']), complex(c['eps_top']), complex(c['eps_bot']),
                          (0.6, 0.8j))
        amps = torch.as_tensor(np.stack([np.stack([a[col].reshape(-1) for a in o['amps']]) for col in range(3)]))[None]
        R = torch.as_tensor(o['R'][0])[None]
        T = torch.as_tensor(o['T'][0])[None]
        refl, trans = rcwa._diffraction_orders(R, T, amps, (float(c['wavelength']),), hu, hv)
        assert refl.orders_u.tolist() == list(range(-hu, hu + 1)) and torch.equal(refl.efficiency, R)
        for got, key in ((refl.amplitude_ratio_s, 'reflected_s'), (refl.amplitude_ratio_p, 'reflected_p'),
                         (trans.amplitude_ratio_s, 'transmitted_s'), (trans.amplitude_ratio_p, 'transmitted_p')):
            want = c[f'mix_{key}']
            assert np.abs(got[0].numpy() - want).max() <= 1e-12 * max(1.0, np.abs(want).max()), (name, key)
    none = rcwa._diffraction_orders(R, T, None, (600.0,), hu, hv)
    assert none[0].amplitude_ratio_s is None and none[1].efficiency is T


def test_result_reports_power_entering_absorption_and_validity():
    import torch
    R = torch.tensor([[[0.1, 0.2]], [[0.3, 0.0]]], dtype=torch.float64)
    T = torch.tensor([[[0.5, 0.1]], [[0.6, 0.05]]], dtype=torch.float64)
    res = rcwa.Result(R, T, (R, R), (T, T), None, (600.0, 700.0), {}, orders=(0, 0))
    assert torch.allclose(res.outputs['power_entering'], torch.tensor([0.7, 0.7], dtype=torch.float64))
    assert torch.allclose(res.outputs['absorption'], torch.tensor([0.1, 0.05], dtype=torch.float64))
    assert torch.allclose(res.absorption, res.outputs['absorption'])
    assert res.validity['checks']['numerical_finite'] is True
    assert res.validity['convergence']['status'] == 'not assessed'


def test_sample_structure_returns_the_raster_the_solve_reads():
    p = _problem()
    # the public stack lists layers from the bottom: layer 0 is the raster, layer 1 the uniform one
    np.testing.assert_array_equal(rcwa.sample_structure(p, layer=0), np.array([[1.0, 12.25], [12.25, 1.0]]))
    np.testing.assert_array_equal(rcwa.sample_structure(p, layer=1), np.full((1, 1), 2.25 + 0j))
    for kw, code in ((dict(layer=2), 'structure.layer'), (dict(samples=0), 'structure.samples'),
                     (dict(quantity='chi'), 'structure.quantity'), (dict(wavelength_index=3), 'structure.wavelength')):
        with pytest.raises(rcwa.ValidationError) as e:
            rcwa.sample_structure(p, **kw)
        assert e.value.code == code
    with pytest.raises(rcwa.UnsupportedFeatureError):
        rcwa.sample_structure(p, quantity='mu')


def _amplitude_case(name):
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'ref_amplitudes.npz'))
    return {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}


@pytest.mark.parametrize('name', ['grating_1d', 'crossed_1', 'crossed_3', 'symmetric_pillar', 'lossy_substrate',
                                  'metal_substrate', 'tir', 'dense_superstrate', 'normal_rotated'])
def test_order_readings_match_the_reference(name):
    """outputs['reflected'|'transmitted'] beyond the ratios -- amplitude_ratio_xyz, power (W),
    k_parallel, k_normal, and the reference's plane, cell measure, medium and incident power --
    from the oracle's amplitudes, against the reference's own run in micrometres with a 2.5 V/m
    source (results.py:292-420)."""
    import torch
    from oracle import rcwa_oracle as O
    c = _amplitude_case(name)
    hu, hv = (int(v) for v in c['orders'])
    um = 1e-3
    wl, per = float(c['wavelength']) * um, tuple(float(p) * um for p in c['period'])
    th = np.asarray(c['thickness'], float) * um
    for tag, pol in (('p', 'p'), ('mix', (0.6, 0.8j))):
        o = O.solve_stack(c['structure'], th, wl, per, hu, hv, float(c['theta']), float(c['phi']),
                          complex(c['eps_top']), complex(c['eps_bot']), pol)
        amps = torch.as_tensor(np.stack([np.stack([a[col].reshape(-1) for a in o['amps']]) for col in range(3)]))[None]
        R, T = torch.as_tensor(o['R'][0])[None], torch.as_tensor(o['T'][0])[None]
        ports = dict(wavelengths=[wl], thetas=[float(c['theta'])], phi=float(c['phi']), period=per,
                     eps_top=complex(c['eps_top']), eps_bot=complex(c['eps_bot']), pol=O.polarization_pair(pol),
                     amplitude=2.5, length='um', top_plane=float(th.sum()))
        refl, trans = rcwa._diffraction_orders(R, T, amps, (wl,), hu, hv, ports=ports)
        p_inc = float(c[f'{tag}_reflected_incident_power'][0])
        assert abs(float(refl.reference['incident_power'][0]) - p_inc) <= 1e-13 * p_inc, (name, tag)
        for port, got in (('reflected', refl), ('transmitted', trans)):
            key = f'{tag}_{port}'
            for field_, tol in (('amplitude_ratio_xyz', 1e-11), ('k_parallel', 1e-13), ('k_normal', 1e-13)):
                want = c[f'{key}_{field_}']
                diff = np.abs(getattr(got, field_)[0].numpy() - want).max()
                assert diff <= tol * max(1.0, np.abs(want).max()), (name, key, field_, diff)
            assert np.abs(got.power[0].numpy() - c[f'{key}_power']).max() <= 1e-11 * p_inc, (name, key)
            assert np.abs(got.efficiency[0].numpy() - c[f'{key}_efficiency']).max() <= 1e-11, (name, key)
            assert got.reference['plane'][0] == pytest.approx(float(c[f'{key}_plane'][0]), rel=1e-14, abs=1e-18)
            assert got.reference['cell_measure'][0] == pytest.approx(float(c[f'{key}_cell_measure'][0]), rel=1e-14)
            assert got.reference['epsilon'][0] == complex(c[f'{key}_epsilon'][0])
            # the CW field is the ratio times the source, and one order reads the same arrays
            assert torch.equal(got.field_xyz, got.amplitude_ratio_xyz * 2.5)
            one = got.order(0, 0)
            assert one.k_normal.shape == (1,) and torch.equal(one.power, got.power[:, hv, hu])
        # the outgoing powers add up to the efficiencies times the incident power
        total = float(refl.power.sum() + trans.power.sum())
        assert total == pytest.approx(float(R.sum() + T.sum()) * p_inc, rel=1e-9, abs=1e-12 * p_inc)


def test_units_and_order_lookup_refusals():
    import torch
    with pytest.raises(rcwa.ValidationError) as e:
        rcwa.Units(length='inch')
    assert e.value.code == 'units.length'
    R = torch.zeros((1, 3, 5), dtype=torch.float64)
    refl, _ = rcwa._diffraction_orders(R, R, None, (1.0,), 2, 1)
    with pytest.raises(KeyError):
        refl.order(3, 0)
    assert refl.order(-2, 1).efficiency.shape == (1,) and refl.field_s is None


def test_numerics_the_path_does_not_implement_are_refused_not_ignored():
    """The second-order layer operator is what the kernels solve; a merge tolerance changes the
    problem. Both defaults pass, other values are refused with the option's path."""
    rcwa._numerics_orders(rcwa.Numerics(orders=(1, 1), formulation='second_order', half_space_merge_tolerance=0.0))
    for kw, path in ((dict(formulation='first_order'), 'numerics.formulation'),
                     (dict(half_space_merge_tolerance=1e-6), 'numerics.half_space_merge_tolerance')):
        with pytest.raises(rcwa.UnsupportedFeatureError) as e:
            rcwa._numerics_orders(rcwa.Numerics(orders=(1, 1), **kw))
        assert e.value.path == path


def test_other_illuminations_are_refused_not_read_as_a_plane_wave():
    """An incident-order set, a Gaussian beam and a dipole carry angle fields like a plane wave;
    they are refused by what defines them rather than solved as their central wave."""
    from dataclasses import dataclass

    @dataclass(frozen=True)
    class IncidentOrders:
        weights: tuple
        side: str = 'top'
        polarization: object = 's'
        amplitude: object = 1.0
        theta: object = 0.1
        phi: object = None
        kx: object = None
        ky: object = None

    @dataclass(frozen=True)
    class GaussianBeam:
        waist: object = 2.0
        side: str = 'top'
        polarization: object = 's'
        theta: object = None
        phi: object = None
        kx: object = None
        ky: object = None

    @dataclass(frozen=True)
    class ElectricDipole:
        position: tuple = (0.0, 0.0, 10.0)
        moment: tuple = (1.0, 0.0, 0.0)

    for src in (IncidentOrders(weights=(((0, 0), 1.0), ((1, 0), 0.5))), GaussianBeam(), ElectricDipole()):
        prob = rcwa.Problem(stack=rcwa.Stack(period=(500.0, 500.0), layers=(rcwa.Layer(thickness=50.0, epsilon=2.0),)),
                            excitation=rcwa.Excitation(wavelength=600.0, sources=(src,)))
        with pytest.raises(rcwa.UnsupportedFeatureError) as e:
            rcwa._resolve(prob, rcwa.Numerics(orders=(1, 1)))
        assert e.value.path == 'excitation.sources[0]'


def test_a_profiled_layer_is_refused():
    from dataclasses import dataclass

    @dataclass(frozen=True)
    class ProfiledLayer:
        thickness: object
        background: object = None
        regions: tuple = ()
        layers: tuple = ()

    prob = rcwa.Problem(stack=rcwa.Stack(period=(500.0, 500.0), layers=(ProfiledLayer(thickness=50.0, background=2.0),)),
                        excitation=rcwa.Excitation(wavelength=600.0, sources=(rcwa.PlaneWave(),)))
    with pytest.raises(rcwa.UnsupportedFeatureError) as e:
        rcwa._resolve(prob, rcwa.Numerics(orders=(1, 1)))
    assert e.value.path == 'stack.layers[0]'


def test_readings_without_amplitudes_keep_the_wavevectors():
    """run(amplitudes=False): the amplitude-derived readings are None, never zeros; the
    wavevectors and port references, which need no amplitude, are still given."""
    import torch
    R = torch.zeros((1, 3, 5), dtype=torch.float64)
    ports = dict(wavelengths=[600.0], thetas=[0.1], phi=0.0, period=(500.0, 500.0), eps_top=1.0, eps_bot=2.0,
                 pol=(1.0, 0.0), amplitude=1.0, length='nm', top_plane=10.0, side='top')
    refl, trans = rcwa._diffraction_orders(R, R, None, (600.0,), 2, 1, ports=ports)
    for o in (refl, trans):
        assert o.power is None and o.amplitude_ratio_xyz is None and o.amplitude_ratio_s is None
        assert o.k_normal.shape == (1, 3, 5) and o.reference['incident_power'] is None
    assert refl.reference['port'] == 'top' and trans.reference['plane'] == (0.0,)
