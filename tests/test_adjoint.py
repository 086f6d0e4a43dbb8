"""The hand-written adjoint against central finite differences (CPU, torch reference forward)
and, on a GPU, with the forward of stages A and B on the CUDA kernels."""
import numpy as np
import pytest

torch = pytest.importorskip('torch')

from wavebit_gb300 import adjoint as AD


def _case(seed, L=2, ny=5, nx=6):
    rng = np.random.default_rng(seed)
    eps = 1.0 + 11.25 / (1 + np.exp(-3 * rng.standard_normal((L, ny, nx))))
    th = rng.uniform(80, 200, size=L)
    return eps.astype(complex), th


def _loss(eps, th, impl, **kw):
    return AD.solve_and_grad(eps, th, impl=impl, **kw)


KW = dict(wavelengths=[620.0, 710.0], period=(700.0, 650.0), hu=1, hv=1,
          theta=0.2, phi=0.3, eps_top=1.0, eps_bot=2.25, pol=(0.6, 0.8))


def _weights(N, B=2, seed=1):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((B, N)), rng.standard_normal((B, N))


@pytest.mark.parametrize('seed', [0, 1])
def test_adjoint_matches_finite_differences_cpu(seed):
    eps, th = _case(seed)
    N = 9
    wR, wT = _weights(N, seed=seed)
    loss, R, T, g_eps, g_th = _loss(eps, th, 'torch', weights_R=wR, weights_T=wT, **KW)
    h = 1e-6
    rng = np.random.default_rng(seed + 10)
    for _ in range(4):
        l, y, x = rng.integers(0, eps.shape[0]), rng.integers(0, eps.shape[1]), rng.integers(0, eps.shape[2])
        ep, em = eps.copy(), eps.copy()
        ep[l, y, x] += h; em[l, y, x] -= h
        fd = (_loss(ep, th, 'torch', weights_R=wR, weights_T=wT, **KW)[0]
              - _loss(em, th, 'torch', weights_R=wR, weights_T=wT, **KW)[0]) / (2 * h)
        assert abs(fd - float(g_eps[l, y, x])) <= 1e-6 * max(1.0, abs(fd)), (fd, float(g_eps[l, y, x]))
    for l in range(eps.shape[0]):
        tp, tm = th.copy(), th.copy()
        tp[l] += 1e-4; tm[l] -= 1e-4
        fd = (_loss(eps, tp, 'torch', weights_R=wR, weights_T=wT, **KW)[0]
              - _loss(eps, tm, 'torch', weights_R=wR, weights_T=wT, **KW)[0]) / 2e-4
        assert abs(fd - float(g_th[l])) <= 1e-6 * max(1.0, abs(fd)), (fd, float(g_th[l]))


def test_adjoint_forward_matches_the_oracle_cpu():
    from oracle import rcwa_oracle as O
    eps, th = _case(3)
    wR, wT = _weights(9)
    _, R, T, _, _ = _loss(eps, th, 'torch', weights_R=wR, weights_T=wT, **KW)
    for b, lam in enumerate(KW['wavelengths']):
        o = O.solve_stack(eps, th, lam, KW['period'], 1, 1, KW['theta'], KW['phi'], 1.0, 2.25, KW['pol'])
        assert np.abs(R[b].numpy() - o['R'][0].reshape(-1)).max() < 1e-12
        assert np.abs(T[b].numpy() - o['T'][0].reshape(-1)).max() < 1e-12


@pytest.mark.gpu
def test_adjoint_gb300_matches_the_torch_reference():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    eps, th = _case(4, L=1, ny=8, nx=8)
    kw = dict(KW, hu=2, hv=2)
    N = 25
    wR, wT = _weights(N)
    a = _loss(eps, th, 'gb300', weights_R=wR, weights_T=wT, **kw)
    b = _loss(eps, th, 'torch', weights_R=wR, weights_T=wT, device='cpu', **kw)
    assert abs(a[0] - b[0]) < 1e-10 * max(1, abs(b[0]))
    ga, gb = a[3].cpu().numpy(), b[3].numpy()
    assert np.abs(ga - gb).max() <= 1e-7 * np.abs(gb).max()
    assert np.abs(a[4].cpu().numpy() - b[4].numpy()).max() <= 1e-7 * np.abs(b[4].numpy()).max()


def test_autograd_function_matches_solve_and_grad_cpu():
    eps, th = _case(6, L=1)
    wR, wT = _weights(9)
    e = torch.tensor(eps.real, requires_grad=True)
    t = torch.tensor(th, requires_grad=True)
    spec = dict(KW, impl='torch')
    loss = AD.efficiency_loss(e, t, wR, wT, **spec)
    loss.backward()
    ref = _loss(eps, th, 'torch', weights_R=wR, weights_T=wT, **KW)
    assert abs(float(loss.detach()) - ref[0]) < 1e-12
    assert torch.allclose(e.grad, ref[3], rtol=0, atol=1e-14)
    assert torch.allclose(t.grad, ref[4], rtol=0, atol=1e-14)


def test_chunked_stage_b_gives_the_same_gradient_cpu():
    """A budget that admits one wavelength's eigenpairs at a time (recomputed per chunk, never all
    resident) gives the same loss and gradients as the unchunked pass."""
    eps, th = _case(4)
    kw = dict(KW, wavelengths=[600.0, 650.0, 710.0])
    wR, wT = _weights(9, B=3, seed=4)
    full = _loss(eps, th, 'torch', weights_R=wR, weights_T=wT, **kw)
    n = 18
    one = _loss(eps, th, 'torch', weights_R=wR, weights_T=wT, hbm_budget=8 * 16 * n * n * eps.shape[0], **kw)
    assert AD._chunk_size(eps.shape[0], n, 8 * 16 * n * n * eps.shape[0], 'cpu') == 1
    assert abs(full[0] - one[0]) <= 1e-12 * abs(full[0])
    for a, b in zip(full[1:], one[1:]):
        assert float((a - b).abs().max()) <= 1e-12 * max(1.0, float(a.abs().max()))


@pytest.mark.parametrize('case', ['oblique_crossed', 'normal_degenerate'])
def test_wavelength_gradient_matches_finite_differences_cpu(case):
    """d loss / d wavelength by the forward tangent (wavelength_tangent) against a central
    difference, including normal incidence on a symmetric cell, whose eigenvalues are exactly
    degenerate (the broadened gaps) and whose specular order sits on the kx = 0 branch."""
    if case == 'oblique_crossed':
        eps, th = _case(4)
        kw = dict(KW, wavelengths=[620.0, 710.0])
        wR, wT = _weights(9, B=2, seed=2)
    else:
        eps = np.ones((1, 8, 8), complex)
        eps[0, 2:6, 2:6] = 9.0
        th = np.array([150.0])
        kw = dict(KW, wavelengths=[655.0], theta=0.0, phi=0.0, pol=(1.0, 0.0), period=(700.0, 700.0), hu=2, hv=2)
        wR, wT = _weights(25, B=1, seed=3)
    out = AD.solve_and_grad(eps, th, impl='torch', device='cpu', weights_R=wR, weights_T=wT, grad_wavelength=True,
                            **kw)
    assert len(out) == 6
    for b, lam in enumerate(kw['wavelengths']):
        h = 1e-3

        def f(x):
            wl = list(kw['wavelengths'])
            wl[b] = x
            return AD.solve_and_grad(eps, th, impl='torch', device='cpu', weights_R=wR, weights_T=wT, grad=False,
                                     **dict(kw, wavelengths=wl))[0]
        fd = (f(lam + h) - f(lam - h)) / (2 * h)
        assert abs(float(out[5][b]) - fd) <= 1e-6 * abs(fd), (case, b)


def test_autograd_function_carries_the_wavelength_gradient_cpu():
    eps, th = _case(6, L=1)
    wR, wT = _weights(9, B=2, seed=5)
    e = torch.tensor(eps.real, requires_grad=True)
    t = torch.tensor(th, requires_grad=True)
    wl = torch.tensor(KW['wavelengths'], dtype=torch.float64, requires_grad=True)
    spec = dict(KW, impl='torch', wavelengths=wl)
    loss = AD.efficiency_loss(e, t, wR, wT, **spec)
    loss.backward()
    ref = AD.solve_and_grad(eps, th, impl='torch', device='cpu', weights_R=wR, weights_T=wT, grad_wavelength=True,
                            **KW)
    assert torch.allclose(wl.grad, ref[5], rtol=0, atol=1e-14)
    assert torch.allclose(e.grad, ref[3], rtol=0, atol=1e-14)


def test_integrated_coefficients_take_the_same_pass_cpu():
    """Over one segment per pixel the integrated series is the sampled one, so a differentiated
    raster with fourier_coefficients='integrated' has the oracle's integrated solve as its loss."""
    from oracle import rcwa_oracle as O
    eps, th = _case(7, L=1)
    wR, wT = _weights(9)
    a = _loss(eps, th, 'torch', weights_R=wR, weights_T=wT, fourier_coefficients='integrated', **KW)
    b = _loss(eps, th, 'torch', weights_R=wR, weights_T=wT, **KW)
    assert a[0] == b[0] and torch.equal(a[3], b[3])
    conv = O.to_conv_mat_raster_integrated(eps, 1, 1)
    ref = 0.0
    for bi, lam in enumerate(KW['wavelengths']):
        o = O.solve_stack(eps, th, lam, KW['period'], 1, 1, KW['theta'], KW['phi'], 1.0, 2.25, KW['pol'], conv=conv)
        ref += float((wR[bi] * o['R'][0].reshape(-1)).sum() + (wT[bi] * o['T'][0].reshape(-1)).sum())
    assert abs(a[0] - ref) < 1e-12
    with pytest.raises(ValueError):
        _loss(eps, th, 'torch', weights_R=wR, weights_T=wT, fourier_coefficients='laurent', **KW)
