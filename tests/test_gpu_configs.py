"""Parity of the CUDA path at the benchmark's own sizes, against the reference's runs.

``golden/ref_configs.npz`` holds the reference's ``rcwa.run`` (NumPy, complex128) on the
quickstart 1D grating, on four wavelengths of the orders-(7, 7) crossed-grating sweep (three
256x256 binary rasters and a metallic film; 450x450 mode matrices) and on two (wavelength, theta)
points of the orders-(12, 12) sweep (four 256x256 binary rasters; 1250x1250 mode matrices), each
for s and p incidence. The plain FP64 form must match per-order R and T within 1e-10 of the
largest efficiency; the mixed form within 1e-6 (the stated precision target), and every result
must come back without a status flag.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
FIX = os.path.join(GOLDEN, 'ref_configs.npz')

#: quickstart values of the 1D grating (README of the reference, s incidence at 900 nm)
QUICKSTART_R = 0.2053316282584904
QUICKSTART_T = 0.7946683717415131


def _engine():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import engine
    return engine


def _cases(prefix):
    d = np.load(FIX)
    names = [str(n) for n in d['names'] if str(n).startswith(prefix)]
    out = []
    for n in names:
        c = {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(n + '__')}
        c['structure'] = d[f"{str(c['stack'])}__structure"]
        c['name'] = n
        out.append(c)
    return out


def _solve(E, cases, precision):
    """One batch over the cases (they share one stack): R, T as (B, 3, n_v, n_u), status."""
    c0 = cases[0]
    hu, hv = (int(v) for v in c0['orders'])
    st = np.ascontiguousarray(c0['structure'])
    L = st.shape[0]
    conv = E.assemble(torch.as_tensor(st, device='cuda'), hu, hv)
    B = len(cases)
    inp = E.BatchInputs([list(range(L))] * B, [list(np.asarray(c['thickness'], float)) for c in cases],
                        [float(c['wavelength']) for c in cases], [list(np.asarray(c['period'], float)) for c in cases],
                        [float(c['theta']) for c in cases], [float(c['phi']) for c in cases],
                        [complex(c['eps_top']) for c in cases], [complex(c['eps_bot']) for c in cases],
                        [[1.0 + 0j, 0j]] * B)
    R, T, status = E.solve_batch(conv, inp, precision=precision)
    torch.cuda.synchronize()
    return R.cpu().numpy(), T.cpu().numpy(), status.cpu().numpy()


def _worst(cases, R, T):
    """max |dR|, |dT| over orders, both polarizations and the batch, relative to the largest
    efficiency of each reference answer."""
    worst = 0.0
    for b, c in enumerate(cases):
        for col, pol in ((1, 's'), (2, 'p')):
            for got, want in ((R[b, col], c[f'R_{pol}']), (T[b, col], c[f'T_{pol}'])):
                scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
                worst = max(worst, np.abs(got - want).max() / scale)
    return worst


def test_quickstart_grating_fp64():
    E = _engine()
    cases = _cases('grating_1d')
    R, T, st = _solve(E, cases, 'double')
    assert not (st & ~8).any(), st
    assert abs(R[0, 1].sum() - QUICKSTART_R) < 1e-12
    assert abs(T[0, 1].sum() - QUICKSTART_T) < 1e-12
    assert _worst(cases, R, T) < 1e-10


@pytest.mark.parametrize('precision,tol', [('double', 1e-10), ('mixed', 1e-6)])
def test_crossed_sweep_slice_full_size(precision, tol):
    """Four wavelengths of the orders-(7, 7) sweep on its own 256x256 rasters (n = 450)."""
    E = _engine()
    cases = _cases('crossed_')
    assert len(cases) == 4
    R, T, st = _solve(E, cases, precision)
    assert not (st & ~8).any(), st
    err = _worst(cases, R, T)
    assert err < tol, (precision, err)


@pytest.mark.parametrize('precision,tol', [('double', 1e-10), ('mixed', 1e-6)])
def test_orders_12_points_full_size(precision, tol):
    """Two (wavelength, theta) points of the orders-(12, 12) sweep (n = 1250)."""
    E = _engine()
    cases = _cases('mixed_')
    assert len(cases) == 2
    R, T, st = _solve(E, cases, precision)
    assert not (st & ~8).any(), st
    err = _worst(cases, R, T)
    assert err < tol, (precision, err)
    # lossless stack: every answer balances energy
    for b in range(len(cases)):
        for col in (1, 2):
            assert abs(1.0 - R[b, col].sum() - T[b, col].sum()) < (1e-9 if precision == 'double' else 1e-6)
