"""A finite gain film (``Im eps < 0`` under exp(-i omega t)) between passive half-spaces against the
closed-form Airy film (test_gain_film.py of the reference): in a finite film the field
``a exp(i k0 q z) + b exp(-i k0 q z)`` is unchanged by ``q -> -q`` with ``a <-> b``, so the answer
needs no root choice, and ``R + T > 1`` is the pump's power. Loss, lossless and gain films, normal
and oblique incidence, s and p, lit from either side; the oracle, the lifecycle on the CPU (the
ETM over the oracle's modes) and the lifecycle through the kernels."""
import numpy as np
import pytest

torch = pytest.importorskip('torch')

from oracle import rcwa_oracle as O
from wavebit_gb300 import rcwa

WL, D, PERIOD = 1.0, 0.2, (0.45, 0.55)
EPS_UP, EPS_DOWN = 1.0, 2.25
ETAS = (0.03, 0.003, 0.0, -0.003, -0.03)        # loss, lossless, gain
THETAS = (0.0, 0.5)


def _airy(eps1, eps2, eps3, kx, k0d, pol):
    """Specular R, T of a slab eps2 lit from the eps1 side (exp(-i w t)); branch-free for a finite film."""
    kz = [np.sqrt(complex(e) - kx ** 2) for e in (eps1, eps2, eps3)]
    kz = [k if k.imag > 0 or (k.imag == 0 and k.real >= 0) else -k for k in kz]
    y = kz if pol == 's' else [k / e for k, e in zip(kz, (eps1, eps2, eps3))]
    r12, r23 = (y[0] - y[1]) / (y[0] + y[1]), (y[1] - y[2]) / (y[1] + y[2])
    t12, t23 = 2 * y[0] / (y[0] + y[1]), 2 * y[1] / (y[1] + y[2])
    ph = np.exp(1j * kz[1] * k0d)
    den = 1 + r12 * r23 * ph ** 2
    r, t = (r12 + r23 * ph ** 2) / den, t12 * t23 * ph / den
    return abs(r) ** 2, (y[2].real / y[0].real) * abs(t) ** 2


def _want(eta, theta, pol, side):
    eps2 = 2.25 + 1j * eta
    lit, far = (EPS_UP, EPS_DOWN) if side == 'top' else (EPS_DOWN, EPS_UP)
    return _airy(lit, eps2, far, np.sqrt(lit) * np.sin(theta), 2 * np.pi / WL * D, pol)


def _problem(eta, theta, pol, side):
    layer = rcwa.Layer(thickness=D, epsilon=np.full((3, 3), 2.25 + 1j * eta))
    return rcwa.Problem(units=rcwa.Units('um'),
                        stack=rcwa.Stack(period=PERIOD, top=rcwa.Material(epsilon=EPS_UP),
                                         bottom=rcwa.Material(epsilon=EPS_DOWN), layers=(layer,)),
                        excitation=rcwa.Excitation(wavelength=WL, sources=(
                            rcwa.PlaneWave(side=side, polarization=pol, theta=theta, phi=0.0),)))


def _check(R, T, eta, theta, pol, side, tol):
    """The specular order carries the Airy film's R and T; every other order is empty."""
    Rw, Tw = _want(eta, theta, pol, side)
    R, T = np.asarray(R), np.asarray(T)
    spec = (R.shape[0] // 2, R.shape[1] // 2)
    assert abs(R[spec] - Rw) <= tol and abs(T[spec] - Tw) <= tol, (eta, theta, pol, side, R[spec], Rw, T[spec], Tw)
    others = np.ones(R.shape, bool)
    others[spec] = False
    assert np.abs(R[others]).max() <= tol and np.abs(T[others]).max() <= tol


@pytest.mark.parametrize('eta', ETAS)
@pytest.mark.parametrize('theta', THETAS)
@pytest.mark.parametrize('pol', ['s', 'p'])
def test_the_oracle_gain_film_is_the_airy_film(eta, theta, pol):
    for side in ('top', 'bottom'):
        lit, far = (EPS_UP, EPS_DOWN) if side == 'top' else (EPS_DOWN, EPS_UP)
        o = O.solve_stack(np.full((1, 3, 3), 2.25 + 1j * eta), np.array([D]), WL, PERIOD, 1, 1, theta, 0.0,
                          lit, far, pol)
        _check(o['R'][0], o['T'][0], eta, theta, pol, side, 1e-12)
    if eta < 0:
        R, T = _want(eta, theta, pol, 'top')
        assert R + T > 1.0                     # the pump's power, not a broken balance


@pytest.mark.parametrize('eta', ETAS)
@pytest.mark.parametrize('side', ['top', 'bottom'])
def test_lifecycle_gain_film_on_the_cpu(eta, side, monkeypatch):
    """rcwa's resolve and the ETM over the oracle's modes in place of the stage-B kernel."""
    from wavebit_gb300 import engine
    from test_fields import use_cpu_stages
    use_cpu_stages(monkeypatch)
    num = rcwa.Numerics(orders=(1, 1), algorithm='etm')
    for theta in THETAS:
        for pol in ('s', 'p'):
            r = rcwa._resolve(_problem(eta, theta, pol, side), num)
            conv_np = O.to_conv_mat_raster_sampled(np.stack(r['rasters']), 1, 1)
            conv = engine.ConvStack.from_matrices(*(torch.as_tensor(a) for a in conv_np), 1, 1)
            p = rcwa.Prepared.__new__(rcwa.Prepared)
            p.handle, p.numerics, p.precision = None, num, 'double'
            res = p._solve_etm(r, conv, np.zeros((1, 1), int))
            _check(res.R[0].numpy(), res.T[0].numpy(), eta, theta, pol, side, 1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize('eta', ETAS)
def test_lifecycle_gain_film_on_the_gpu(eta):
    """The SMM through the kernels, FP64: loss, lossless and gain films, both sides."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    for side in ('top', 'bottom'):
        for theta in THETAS:
            for pol in ('s', 'p'):
                res = rcwa.run(_problem(eta, theta, pol, side), numerics=rcwa.Numerics(orders=(1, 1)))
                _check(res.R[0].cpu().numpy(), res.T[0].cpu().numpy(), eta, theta, pol, side, 1e-10)
