"""Integrated (closed-form segment) Li coefficients on the GPU path: the compressed-raster
assembly (wb_assemble_li_integrated) against the oracle and the reference's own operators and
runs with ``fourier_coefficients='integrated'``; the host-side refusals on the CPU."""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from oracle import rcwa_oracle as O
from wavebit_gb300 import engine as E
from wavebit_gb300 import rcwa

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
NAMES = list(np.load(os.path.join(GOLDEN, 'ref_integrated.npz'))['names'])


def _cuda():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')


def _case(name):
    d = np.load(os.path.join(GOLDEN, 'ref_integrated.npz'))
    return {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}


def _blocky(rng, ny, nx, values=(12.25 + 0.3j, 2.1, 1.0)):
    """A raster of a few rectangular blocks, so that compression has runs to merge."""
    by, bx = rng.integers(1, 5, size=2)
    base = rng.choice(np.asarray(values, complex), size=(by, bx))
    ry = np.sort(rng.integers(0, ny, size=by - 1))
    rx = np.sort(rng.integers(0, nx, size=bx - 1))
    return base[np.searchsorted(ry, np.arange(ny), side='right')][:, np.searchsorted(rx, np.arange(nx), side='right')]


@pytest.mark.parametrize('bad', ['shape', 'order', 'last', 'zero'])
def test_bad_block_edges_are_refused_before_any_device_work(bad):
    eps = np.ones((1, 2, 3), complex)
    x, y = np.array([[1 / 3, 2 / 3, 1.0]]), np.array([[0.5, 1.0]])
    if bad == 'shape':
        x = x[:, :2]
    elif bad == 'order':
        x = np.array([[2 / 3, 1 / 3, 1.0]])
    elif bad == 'last':
        y = np.array([[0.5, 0.99]])
    else:
        y = np.array([[0.0, 1.0]])
    with pytest.raises(ValueError):
        E.assemble(eps, 1, 1, edges=(x, y))


@pytest.mark.gpu
@pytest.mark.parametrize('hu,hv', [(3, 3), (2, 4), (5, 0), (0, 3)])
def test_integrated_assembly_matches_the_oracle(hu, hv):
    """Stacks whose layers compress to different shapes and edges (uniform, 1D, crossed),
    assembled layer group by layer group, against li_conv_integrated of each raw raster."""
    _cuda()
    rng = np.random.default_rng(10 * hu + hv)
    rasters = [_blocky(rng, 24, 24), _blocky(rng, 24, 24), np.full((24, 24), 6.25 + 0.1j),
               _blocky(rng, 1, 40), _blocky(rng, 17, 9)]
    conv = rcwa._assemble_layers(rasters, hu, hv, None, integrated=True)
    torch.cuda.synchronize()
    for i, raster in enumerate(rasters):
        want = O.li_conv_integrated(raster, hu, hv)
        for k, w in enumerate(want):
            got = conv.slot(k)[i].cpu().numpy()
            assert np.abs(got - w).max() <= 1e-12 * np.abs(w).max(), (i, k)


@pytest.mark.gpu
@pytest.mark.parametrize('name', NAMES)
def test_integrated_slots_match_the_reference_operators(name):
    """Centre-frame slots against the reference's rcwa.operators.assemble(...,
    fourier_coefficients='integrated')."""
    _cuda()
    c = _case(name)
    if 'epx' not in c:
        pytest.skip('no stored slots for this scene')
    hu, hv = (int(v) for v in c['orders'])
    conv = rcwa._assemble_layers(list(np.asarray(c['structure'], complex)), hu, hv, None, integrated=True)
    torch.cuda.synchronize()
    for k, slot in enumerate(('epx', 'epy', 'epz_i')):
        for i in range(conv.n_layers):
            got = O.swap_fourier_origin(conv.slot(k)[i].cpu().numpy(), hu, hv)
            want = c[slot][i]
            assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max(), (name, slot, i)


def _problem(c):
    st, th = np.asarray(c['structure'], complex), np.asarray(c['thickness'], float)
    layers = tuple(rcwa.Layer(thickness=float(t), epsilon=e) for e, t in zip(st[::-1], th[::-1]))
    return rcwa.Problem(units=rcwa.Units('nm'),
                        stack=rcwa.Stack(period=tuple(float(p) for p in c['period']),
                                         top=rcwa.Material(epsilon=complex(c['eps_top'])),
                                         bottom=rcwa.Material(epsilon=complex(c['eps_bot'])), layers=layers),
                        excitation=rcwa.Excitation(wavelength=float(c['wavelength']), sources=(
                            rcwa.PlaneWave(polarization='s', theta=float(c['theta']), phi=float(c['phi'])),)))


@pytest.mark.gpu
@pytest.mark.parametrize('name', NAMES)
def test_integrated_run_matches_the_reference_run(name):
    """Per-order R and T of rcwa.run(..., fourier_coefficients='integrated') within 1e-10
    (relative to the largest efficiency) of the reference's own run, for s and p."""
    _cuda()
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    res = rcwa.run(_problem(c), numerics=rcwa.Numerics(orders=(hu, hv), fourier_coefficients='integrated'))
    assert res.diagnostics is not None
    for key, pol in (('s_inc', 's'), ('p_inc', 'p')):
        R = res.outputs[key]['R'][0].cpu().numpy()
        T = res.outputs[key]['T'][0].cpu().numpy()
        scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
        assert np.abs(R - c[f'R_{pol}']).max() <= 1e-10 * scale, (name, pol)
        assert np.abs(T - c[f'T_{pol}']).max() <= 1e-10 * scale, (name, pol)


@pytest.mark.gpu
def test_integrated_and_sampled_agree_on_a_raster_that_does_not_compress():
    """With no equal neighbours the segments are the pixels, and the two coefficient rules
    compute the same staircase series (factorization.py:289-501): the slots agree to round-off."""
    _cuda()
    rng = np.random.default_rng(3)
    raster = rng.standard_normal((11, 13)) + 4.0 + 0.2j
    a = rcwa._assemble_layers([raster], 3, 2, None, integrated=True)
    b = rcwa._assemble_layers([raster], 3, 2, None, integrated=False)
    torch.cuda.synchronize()
    for k in range(3):
        x, y = a.slot(k)[0].cpu().numpy(), b.slot(k)[0].cpu().numpy()
        assert np.abs(x - y).max() <= 1e-11 * np.abs(y).max(), k
