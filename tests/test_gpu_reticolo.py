"""RETICOLO's per-order efficiencies of twelve 1D gratings (tests/references/test_reticolo_golden.py
of the reference) through the CUDA path: wb_assemble_li and wb_solve_batch, FP64."""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from oracle import rcwa_oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
NAMES = list(np.load(os.path.join(GOLDEN, 'reticolo_cases.npz'))['names'])


@pytest.mark.parametrize('name', NAMES)
def test_gpu_matches_reticolo_orders(name):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import engine as E
    d = np.load(os.path.join(GOLDEN, 'reticolo_cases.npz'))
    c = {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}
    h, per = int(c['h']), float(c['period'])
    st = np.asarray(c['structure'], complex)
    L = st.shape[0]
    conv = E.assemble(torch.as_tensor(st, device='cuda'), h, 0)
    inp = E.BatchInputs([list(range(L))], [list(c['thickness'])], [float(c['wavelength'])], [[per, per]],
                        [float(c['theta'])], [float(c['phi'])], [complex(c['top'])], [complex(c['bot'])],
                        [list(O.polarization_pair(str(c['pol'])))])
    R, T, status = E.solve_batch(conv, inp)
    torch.cuda.synchronize()
    assert int(status[0].item()) & ~8 == 0
    for side, arr in (('ri', R[0, 0].cpu().numpy().ravel()), ('ti', T[0, 0].cpu().numpy().ravel())):
        idx = c[f'idx_{side}']
        assert np.abs(arr[idx] - c[f'de_{side}']).max() < 1e-10, (name, side)
        assert np.abs(np.delete(arr, idx)).max(initial=0.0) < 1e-12, (name, side)


@pytest.mark.parametrize('name', NAMES)
def test_gpu_matches_reticolo_orders_from_below(name):
    """RETICOLO's bottom-incidence orders through the kernels: the mirrored scene (layers in
    reverse, half-spaces swapped) lit from above at the substrate angle of the same in-plane
    wavevector."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import engine as E
    d = np.load(os.path.join(GOLDEN, 'reticolo_cases.npz'))
    c = {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}
    h, per = int(c['h']), float(c['period'])
    st = np.asarray(c['structure'], complex)[::-1].copy()   # a fresh array: positive strides even for one layer
    L = st.shape[0]
    n_top, n_bot = np.sqrt(complex(c['top'])).real, np.sqrt(complex(c['bot'])).real
    theta_b = float(np.arcsin(n_top * np.sin(float(c['theta'])) / n_bot))
    conv = E.assemble(torch.as_tensor(st, device='cuda'), h, 0)
    inp = E.BatchInputs([list(range(L))], [list(np.asarray(c['thickness'], float)[::-1])], [float(c['wavelength'])],
                        [[per, per]], [theta_b], [float(c['phi'])], [complex(c['bot'])], [complex(c['top'])],
                        [list(O.polarization_pair(str(c['pol'])))])
    R, T, status = E.solve_batch(conv, inp)
    torch.cuda.synchronize()
    assert int(status[0].item()) & ~8 == 0
    for side, idx_key, arr in (('ri_bot', 'idx_ti', R[0, 0].cpu().numpy().ravel()),
                               ('ti_bot', 'idx_ri', T[0, 0].cpu().numpy().ravel())):
        idx = c[idx_key]
        assert np.abs(arr[idx] - c[f'de_{side}']).max() < 1e-10, (name, side)
        assert np.abs(np.delete(arr, idx)).max(initial=0.0) < 1e-12, (name, side)
