"""Explicit operators (rcwa.operators.assemble / solve): refusals on CPU, the solve on a GPU."""
import dataclasses

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from wavebit_gb300 import rcwa
from wavebit_gb300 import operators as OP


def _problem(raster, wavelength=(650.0, 820.0)):
    layers = (rcwa.Layer(thickness=220.0, epsilon=raster),
              rcwa.Layer(thickness=140.0, epsilon=np.full((12, 12), 4.0 + 0.2j)))
    return rcwa.Problem(units=rcwa.Units('nm'),
                        stack=rcwa.Stack(period=(700.0, 760.0), top=rcwa.Material(epsilon=1.0),
                                         bottom=rcwa.Material(epsilon=2.25), layers=layers),
                        excitation=rcwa.Excitation(wavelength=wavelength,
                                                   sources=(rcwa.PlaneWave(polarization='p', theta=0.2, phi=0.4),)))


def _raster(seed):
    rng = np.random.default_rng(seed)
    a = np.ones((12, 12), complex)
    a[rng.random((12, 12)) < 0.4] = 12.25
    return a


def test_solve_refuses_anything_but_assembled_operators_cpu():
    with pytest.raises(rcwa.ValidationError) as e:
        OP.solve(_problem(_raster(0)), object())
    assert e.value.code == 'operators.type'


def test_error_classes_follow_the_reference_cpu():
    err = rcwa.IncompatibleProblemError('x')
    assert isinstance(err, rcwa.ValidationError) and err.code == 'problem.incompatible'
    assert rcwa.ValidationError('y').code == 'input.invalid'
    assert rcwa.operators is OP


def test_frame_swap_is_an_involution_cpu():
    hu, hv = 2, 1
    N = (2 * hu + 1) * (2 * hv + 1)
    a = torch.randn(3, N, N, dtype=torch.complex128)
    assert torch.equal(OP._swap_frame(OP._swap_frame(a, hu, hv), hu, hv), a)


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')


@pytest.mark.gpu
def test_assembled_operators_solve_like_run_and_match_the_oracle():
    _gpu()
    from oracle import rcwa_oracle as O
    num = rcwa.Numerics(orders=(3, 2))
    p = _problem(_raster(1))
    ops = OP.assemble(p, numerics=num)
    res = OP.solve(p, ops)
    ref = rcwa.prepare(p, numerics=num).run()
    assert float((res.R - ref.R).abs().max()) <= 1e-12 and float((res.T - ref.T).abs().max()) <= 1e-12
    assert res.diagnostics['explicit_operators']
    # slots about the cell centre, entry face first (the public stack lists the bottom layer first)
    for li, raster in enumerate([_raster(1), np.full((12, 12), 4.0 + 0.2j)][::-1]):
        want = O.li_conv(raster, 3, 2)
        for k in range(3):
            got = ops.epsilon[0][k][li].cpu().numpy()
            w = O.swap_fourier_origin(want[k], 3, 2)
            assert np.abs(got - w).max() <= 1e-12 * np.abs(w).max()


@pytest.mark.gpu
def test_replaced_operator_arrays_are_what_is_solved():
    _gpu()
    num = rcwa.Numerics(orders=(3, 2))
    pa, pb = _problem(_raster(2)), _problem(_raster(3))
    ops_a, ops_b = OP.assemble(pa, numerics=num), OP.assemble(pb, numerics=num)
    swapped = dataclasses.replace(ops_a, epsilon=ops_b.epsilon)
    res = OP.solve(pa, swapped)
    ref = rcwa.prepare(pb, numerics=num).run()
    assert float((res.R - ref.R).abs().max()) <= 1e-12 and float((res.T - ref.T).abs().max()) <= 1e-12
    with pytest.raises(rcwa.IncompatibleProblemError) as e:
        OP.solve(pb, ops_a)
    assert e.value.code == 'operators.physical_contract'
