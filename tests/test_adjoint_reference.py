"""The hand-written adjoint against the reference's own gradient.

``golden/ref_gradient.npz`` holds the reference PyTorch backend's ``loss.backward()`` (its
differentiable path, ``rcwa.run(..., backend='torch')``) for the loss sum over wavelengths of the
(0, 0)-order transmission, p incidence:

* ``small``: a 32x32 continuous raster, orders (5, 5), 4 wavelengths;
* ``layer``: the adjoint-layer workload, a 128x128 raster at orders (9, 9) and 32 wavelengths.

Our gradient comes from ``solve_and_grad``: the torch pass on the CPU for the small case, and
the CUDA kernels' forward with the hand-written reverse pass on the GPU for the full workload.
The loss must agree to 1e-10 relative, and every pixel's and the thickness's gradient to 1e-7 of
the largest pixel gradient (1e-8 and 1e-6 with the mixed form's eigen-solve).
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from wavebit_gb300 import adjoint as AD

FIX = os.path.join(os.path.dirname(__file__), 'golden', 'ref_gradient.npz')


def _case(name):
    d = np.load(FIX)
    return {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}


def _ours(c, impl, device, modes='double'):
    h = int(c['orders'][0])
    N = (2 * h + 1) ** 2
    B = len(c['wavelengths'])
    wR, wT = np.zeros((B, N)), np.zeros((B, N))
    wT[:, N // 2] = 1.0
    loss, R, T, g_eps, g_th = AD.solve_and_grad(
        c['eps'][None].astype(np.complex128), np.array([float(c['thickness'])]), c['wavelengths'], (1000.0, 1000.0),
        h, h, wR, wT, theta=0.0, phi=0.0, eps_top=1.0, eps_bot=2.25, pol=(0.0, 1.0), impl=impl, device=device,
        modes=modes)
    return loss, np.asarray(g_eps.cpu())[0], float(g_th.cpu()[0])


def _check(c, loss, g_eps, g_th, tol=1e-7, loss_tol=1e-10):
    assert abs(loss - float(c['loss'])) <= loss_tol * abs(float(c['loss']))
    scale = np.abs(c['grad_eps']).max()
    assert np.abs(g_eps - c['grad_eps']).max() <= tol * scale
    assert abs(g_th - float(c['grad_thickness'])) <= tol * max(scale, abs(float(c['grad_thickness'])))


def test_torch_adjoint_matches_the_reference_gradient():
    c = _case('small')
    _check(c, *_ours(c, 'torch', 'cpu'))


@pytest.mark.gpu
@pytest.mark.parametrize('modes,tol,loss_tol', [('double', 1e-7, 1e-10), ('mixed', 1e-6, 1e-8)])
def test_kernel_adjoint_matches_the_reference_gradient_on_the_adjoint_layer_workload(modes, tol, loss_tol):
    """The kernel path (every stage and reverse pass on the library's kernels) with the FP64
    eigen-solve (loss 1e-10 relative, gradient 1e-7 of the largest pixel gradient) and with the
    FP32 eigen-solve refined by Newton steps, held to the mixed form's own accuracy (loss 1e-8,
    gradient 1e-6; measured 3e-10 and 1.1e-7 on a GB300)."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    c = _case('layer')
    _check(c, *_ours(c, 'gb300', 'cuda', modes), tol=tol, loss_tol=loss_tol)
