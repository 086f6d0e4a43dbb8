"""The reverse passes on the GPU through the C ABI (wb_smm_solve_vjp, wb_layer_modes_vjp,
wb_assemble_li_vjp), each against the hand-written torch restatement (wavebit_gb300/adjoint.py)
evaluated on the kernels' own forward (their slots and eigenpairs), and the gradient path built
on them (solve_and_grad with impl='gb300') against the torch path. The full adjoint-layer
workload against the reference's own gradient is tests/test_adjoint_reference.py."""
import numpy as np
import pytest

torch = pytest.importorskip('torch')

from vjp_case import Case, eff_cotangents, rel, weights  # noqa: E402
from wavebit_gb300 import adjoint as A  # noqa: E402

pytestmark = pytest.mark.gpu


def _case(**kw):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    return Case(device='cuda', kernels=True, **kw)


def _inputs(case):
    from wavebit_gb300 import engine
    sa = case.solve_arrays()
    return engine.BatchInputs([list(range(case.L))] * case.B, sa['thickness'], sa['wavelength'], sa['period'],
                              sa['theta'], sa['phi'], sa['eps_top'], sa['eps_bot'], sa['pol'])


def _modes(case):
    return case.pairs('W'), case.pairs('V'), case.pairs('q')


@pytest.mark.parametrize('kw', [dict(seed=0), dict(seed=3, L=3, hu=3, hv=2, wavelengths=(540.0, 600.0, 655.0))])
def test_smm_solve_vjp_matches_the_torch_cascade_adjoint(kw):
    from wavebit_gb300 import engine
    case = _case(**kw)
    wR, wT = weights(case, 4)
    _, gW_t, gV_t, gq_t, gth_t = case.stage_c_torch(wR, wT)
    gR, gT = eff_cotangents(case, wR, wT)
    W, V, q = _modes(case)
    gW, gV, gq, gth, st = engine.smm_solve_vjp(W, V, q, _inputs(case), case.hu, case.hv, gR, gT)
    torch.cuda.synchronize()
    assert int(st.abs().sum()) == 0
    assert rel(gW, gW_t) < 1e-10
    assert rel(gV, gV_t) < 1e-10
    assert rel(gq, gq_t) < 1e-10
    assert rel(gth, gth_t) < 1e-10


@pytest.mark.parametrize('kw', [dict(seed=0), dict(seed=4, L=3, hu=3, hv=3)])
def test_layer_modes_vjp_matches_the_torch_eigen_adjoint(kw):
    from wavebit_gb300 import engine
    case = _case(**kw)
    rng = np.random.default_rng(8)
    Pn, n = case.B * case.L, case.n
    cz = lambda *s: torch.as_tensor(rng.standard_normal(s) + 1j * rng.standard_normal(s), device='cuda')  # noqa: E731
    gW, gV, gq, gw = cz(Pn, n, n), cz(Pn, n, n), cz(Pn, n), cz(Pn, n)
    want = case.stage_b_torch(gW, gV, gq, gw)
    kx, ky = case.kxy()
    W, V, q = _modes(case)
    g, st = engine.layer_modes_vjp(case.cs, np.tile(np.arange(case.L), case.B), kx, ky, case.pairs('w'), q, W, V,
                                   g_w=gw, g_q=gq, g_W=gW, g_V=gV)
    torch.cuda.synchronize()
    assert int(st.abs().sum()) == 0
    for l in range(case.L):
        for k in range(3):
            assert rel(g.slot(k)[l], want[l][k]) < 1e-9, (l, k)


def test_assemble_li_vjp_matches_the_torch_li_adjoint():
    from wavebit_gb300 import engine
    case = _case(seed=2, ny=24, nx=20, hu=4, hv=3)
    rng = np.random.default_rng(12)
    cz = lambda *s: torch.as_tensor(rng.standard_normal(s) + 1j * rng.standard_normal(s), device='cuda')  # noqa: E731
    g_conv = [[cz(case.N, case.N) for _ in range(3)] for _ in range(case.L)]
    want = case.stage_a_torch(g_conv)
    g = engine.ConvStack.from_matrices(*(torch.stack([g_conv[l][k] for l in range(case.L)]) for k in range(3)),
                                       case.hu, case.hv)
    got = engine.assemble_vjp(case.eps, case.cs, g)
    torch.cuda.synchronize()
    assert rel(got, want) < 1e-10


@pytest.mark.parametrize('kw', [dict(seed=1), dict(seed=6, L=3, ny=32, nx=32, hu=4, hv=4,
                                                   wavelengths=(600.0, 640.0, 700.0, 760.0))])
def test_kernel_gradient_path_matches_the_torch_path(kw):
    """solve_and_grad(impl='gb300') runs every stage and reverse pass on the kernels; its loss,
    R, T and gradients equal the torch restatement's."""
    case = _case(**kw)
    wR, wT = weights(case, 5)
    common = dict(theta=case.theta, phi=case.phi, eps_top=case.eps_top, eps_bot=case.eps_bot, pol=case.pol)
    lk, Rk, Tk, gk, thk = A.solve_and_grad(case.eps_np, case.th, case.wls, case.period, case.hu, case.hv, wR, wT,
                                           impl='gb300', device='cuda', **common)
    lt, Rt, Tt, gt, tht = A.solve_and_grad(case.eps_np, case.th, case.wls, case.period, case.hu, case.hv, wR, wT,
                                           impl='torch', device='cuda', **common)
    assert abs(lk - lt) <= 1e-10 * abs(lt)
    assert rel(Rk, Rt) < 1e-10 and rel(Tk, Tt) < 1e-10
    assert rel(gk, gt) < 1e-8
    assert rel(thk, tht) < 1e-8


def test_kernel_gradient_path_in_chunks_equals_one_chunk():
    """A budget that holds one wavelength's modes at a time gives the same gradient."""
    case = _case(seed=7, wavelengths=(610.0, 650.0, 690.0))
    wR, wT = weights(case, 6)
    common = dict(theta=case.theta, phi=case.phi, eps_top=case.eps_top, eps_bot=case.eps_bot, pol=case.pol,
                  impl='gb300', device='cuda')
    one = A.solve_and_grad(case.eps_np, case.th, case.wls, case.period, case.hu, case.hv, wR, wT, **common)
    per = 8 * 16 * case.n * case.n * case.L
    many = A.solve_and_grad(case.eps_np, case.th, case.wls, case.period, case.hu, case.hv, wR, wT, hbm_budget=per,
                            **common)
    assert abs(one[0] - many[0]) <= 1e-12 * abs(one[0])
    assert rel(many[3], one[3]) < 1e-12 and rel(many[4], one[4]) < 1e-12
