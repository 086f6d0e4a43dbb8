"""The half-space branches through the CUDA path: a lossy and a metallic substrate, total internal
reflection and a denser superstrate, against the reference's own run (wb_assemble_li and
wb_solve_batch, FP64)."""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from oracle import rcwa_oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
NAMES = list(np.load(os.path.join(GOLDEN, 'ref_halfspace.npz'))['names'])


@pytest.mark.parametrize('name', NAMES)
def test_gpu_matches_the_reference_half_space_branches(name):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import engine as E
    d = np.load(os.path.join(GOLDEN, 'ref_halfspace.npz'))
    c = {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}
    hu, hv = (int(v) for v in c['orders'])
    st = np.asarray(c['structure'], complex)
    L = st.shape[0]
    conv = E.assemble(torch.as_tensor(st, device='cuda'), hu, hv)
    inp = E.BatchInputs([list(range(L))], [list(c['thickness'])], [float(c['wavelength'])], [list(c['period'])],
                        [float(c['theta'])], [float(c['phi'])], [complex(c['eps_top'])], [complex(c['eps_bot'])],
                        [list(O.polarization_pair('s'))])
    R, T, status = E.solve_batch(conv, inp)
    torch.cuda.synchronize()
    assert int(status[0].item()) & ~8 == 0
    for col, pol in ((1, 's'), (2, 'p')):
        scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
        assert np.abs(R[0, col].cpu().numpy() - c[f'R_{pol}']).max() <= 1e-10 * scale, (name, pol)
        assert np.abs(T[0, col].cpu().numpy() - c[f'T_{pol}']).max() <= 1e-10 * scale, (name, pol)
