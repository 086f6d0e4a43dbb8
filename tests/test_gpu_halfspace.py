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


@pytest.mark.parametrize('name', list(np.load(os.path.join(GOLDEN, 'ref_bare.npz'))['names']))
def test_gpu_bare_interface_matches_the_reference(name):
    """rcwa.run on a stack with no layers (the bare interface) against the reference's own run."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import rcwa
    d = np.load(os.path.join(GOLDEN, 'ref_bare.npz'))
    c = {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}
    hu, hv = (int(v) for v in c['orders'])
    prob = rcwa.Problem(units=rcwa.Units('nm'),
                        stack=rcwa.Stack(period=tuple(float(p) for p in c['period']),
                                         top=rcwa.Material(epsilon=complex(c['eps_top'])),
                                         bottom=rcwa.Material(epsilon=complex(c['eps_bot'])), layers=()),
                        excitation=rcwa.Excitation(wavelength=float(c['wavelength']), sources=(
                            rcwa.PlaneWave(polarization='s', theta=float(c['theta']), phi=float(c['phi'])),)))
    res = rcwa.run(prob, numerics=rcwa.Numerics(orders=(hu, hv)))
    for key, pol in (('s_inc', 's'), ('p_inc', 'p')):
        scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
        assert np.abs(res.outputs[key]['R'][0].cpu().numpy() - c[f'R_{pol}']).max() <= 1e-10 * scale
        assert np.abs(res.outputs[key]['T'][0].cpu().numpy() - c[f'T_{pol}']).max() <= 1e-10 * scale
