"""d loss / d wavelength with the CUDA kernels' eigenpairs against the torch reference pass."""
import numpy as np
import pytest

torch = pytest.importorskip('torch')

from wavebit_gb300 import adjoint as AD

pytestmark = pytest.mark.gpu


def test_wavelength_gradient_gb300_matches_the_torch_reference():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    rng = np.random.default_rng(4)
    eps = (1.0 + 11.25 / (1 + np.exp(-3 * rng.standard_normal((1, 8, 8))))).astype(complex)
    th = np.array([140.0])
    kw = dict(wavelengths=[620.0, 710.0], period=(700.0, 650.0), hu=2, hv=2, theta=0.2, phi=0.3,
              eps_top=1.0, eps_bot=2.25, pol=(0.6, 0.8))
    wR, wT = rng.standard_normal((2, 25)), rng.standard_normal((2, 25))
    a = AD.solve_and_grad(eps, th, impl='gb300', weights_R=wR, weights_T=wT, grad_wavelength=True, **kw)
    b = AD.solve_and_grad(eps, th, impl='torch', device='cpu', weights_R=wR, weights_T=wT, grad_wavelength=True, **kw)
    ga, gb = a[5].cpu().numpy(), b[5].numpy()
    assert np.abs(ga - gb).max() <= 1e-7 * np.abs(gb).max()
