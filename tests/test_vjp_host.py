"""The reverse-pass drivers of the C ABI's wb_*_vjp entry points (wavebit_gb300/csrc/wb_vjp.h),
compiled on the CPU over a C++ stand-in of the device primitives (tests/vjp_host/host_ops.cpp),
against the hand-written torch adjoint (wavebit_gb300/adjoint.py, itself held to central finite
differences and to the reference PyTorch backend's gradient). This checks the drivers' index,
stride, transpose and conjugation logic without a GPU; the same source runs on the device
kernels in tests/test_gpu_vjp.py."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from vjp_case import Case, eff_cotangents, rel, rowmajor, weights  # noqa: E402
from wavebit_gb300 import adjoint as A  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, 'tests', 'vjp_host', 'host_ops.cpp')


def _cuda_include():
    for base in (os.environ.get('CUDA_HOME'), os.environ.get('CUDA_PATH'), '/usr/local/cuda'):
        if base and os.path.exists(os.path.join(base, 'include', 'vector_types.h')):
            return os.path.join(base, 'include')
    return None


@pytest.fixture(scope='module')
def host(tmp_path_factory):
    gxx = shutil.which('g++')
    inc = _cuda_include()
    if not gxx or not inc:
        pytest.skip('g++ and the CUDA headers (vector_types.h) are needed to build the host drivers')
    out = str(tmp_path_factory.mktemp('vjp') / 'libwbvjp_host.so')
    cmd = [gxx, '-O2', '-std=c++17', '-shared', '-fPIC', '-I', os.path.join(ROOT, 'wavebit_gb300', 'csrc'),
           '-I', inc, SRC, '-o', out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(out)
    vp, i = ctypes.c_void_p, ctypes.c_int
    lib.host_layer_modes_vjp.argtypes = [i, i, i] + [vp] * 14
    lib.host_smm_vjp.argtypes = [i, i, i] + [vp] * 31
    lib.host_assemble_vjp.argtypes = [i, i, i, i, i] + [vp] * 8
    return lib


def P(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def run_stage_c(lib, case, gR, gT):
    pa = case.port_arrays()
    sa = case.solve_arrays()
    W = torch.stack([m['W'].T.contiguous() for m in case.modes])
    V = torch.stack([m['V'].T.contiguous() for m in case.modes])
    q = case.pairs('q').contiguous()
    Pn = case.B * case.L
    gW = torch.zeros(Pn, case.n, case.n, dtype=torch.complex128)
    gV = torch.zeros_like(gW)
    gq = torch.zeros(Pn, case.n, dtype=torch.complex128)
    gth = torch.zeros(case.B, case.L, dtype=torch.float64)
    st = torch.zeros(case.B, dtype=torch.int32)
    gRt = torch.as_tensor(gR, dtype=torch.float64).contiguous()
    gTt = torch.as_tensor(gT, dtype=torch.float64).contiguous()
    rc = lib.host_smm_vjp(case.B, case.L, case.N, *[P(pa[k]) for k in ('kx', 'ky', 'c', 's', 'kzt', 'kzb', 'wg', 'vg',
                                                                       'r11', 'r12', 'r21', 'r22', 't11', 't21',
                                                                       'nt', 'nb')],
                          P(W), P(V), P(q), P(sa['thickness']), P(sa['wavelength']), P(sa['eps_top']),
                          P(sa['eps_bot']), P(sa['pol']), P(gRt), P(gTt), P(gW), P(gV), P(gq), P(gth), P(st))
    assert rc == 0 and int(st.abs().sum()) == 0
    return rowmajor(gW), rowmajor(gV), gq, gth


def run_stage_b(lib, case, gW, gV, gq, gw=None):
    conv = case.conv_buf()
    kx, ky = case.kxy()
    pl = torch.tensor([p % case.L for p in range(case.B * case.L)], dtype=torch.int32)
    w, q = case.pairs('w').contiguous(), case.pairs('q').contiguous()
    W = torch.stack([m['W'].T.contiguous() for m in case.modes])
    V = torch.stack([m['V'].T.contiguous() for m in case.modes])
    gconv = torch.zeros(case.L, 3, case.N, case.N, dtype=torch.complex128)
    st = torch.zeros(case.B * case.L, dtype=torch.int32)
    # every buffer stays referenced until the call returns
    gWc, gVc, gqc = gW.transpose(-1, -2).contiguous(), gV.transpose(-1, -2).contiguous(), gq.contiguous()
    gwc = None if gw is None else gw.contiguous()
    rc = lib.host_layer_modes_vjp(case.B * case.L, case.N, case.L, P(conv), P(pl), P(kx), P(ky), P(w), P(q), P(W), P(V),
                                  P(gwc), P(gqc), P(gWc), P(gVc), P(gconv), P(st))
    assert rc == 0 and int(st.abs().sum()) == 0
    return [[rowmajor(gconv[l, k]) for k in range(3)] for l in range(case.L)]


def run_stage_a(lib, case, g_conv):
    eps = case.eps.contiguous()
    epx, epz = case.slot_planes(0), case.slot_planes(2)
    g = [torch.stack([g_conv[l][k].T.contiguous() for l in range(case.L)]) for k in range(3)]
    g_eps = torch.zeros(case.L, case.ny, case.nx, dtype=torch.complex128)
    st = torch.zeros(1, dtype=torch.int32)
    rc = lib.host_assemble_vjp(case.L, case.ny, case.nx, case.hu, case.hv, P(eps), P(epx), P(epz), P(g[0]), P(g[1]),
                               P(g[2]), P(g_eps), P(st))
    assert rc == 0 and int(st.item()) == 0
    return g_eps


@pytest.mark.parametrize('seed', [0, 3])
def test_stage_c_reverse_matches_the_torch_cascade_adjoint(host, seed):
    case = Case(seed=seed)
    wR, wT = weights(case, seed)
    _, gW_t, gV_t, gq_t, gth_t = case.stage_c_torch(wR, wT)
    gR, gT = eff_cotangents(case, wR, wT)
    gW, gV, gq, gth = run_stage_c(host, case, gR, gT)
    assert rel(gW, gW_t) < 1e-10
    assert rel(gV, gV_t) < 1e-10
    assert rel(gq, gq_t) < 1e-10
    assert rel(gth, gth_t) < 1e-10


def test_stage_c_reverse_of_the_pure_polarization_columns(host):
    """Cotangents on the pure-s and pure-p columns equal the given-polarization cotangents of the
    same loss run with pol = (1, 0) and (0, 1)."""
    case = Case(seed=5)
    wR, wT = weights(case, 9)
    gR = np.zeros((case.B, 3, case.N)); gT = np.zeros((case.B, 3, case.N))
    gR[:, 1] = wR; gT[:, 2] = wT
    gW, gV, gq, gth = run_stage_c(host, case, gR, gT)
    s_case = Case(seed=5, pol=(1.0, 0.0))
    p_case = Case(seed=5, pol=(0.0, 1.0))
    _, gWs, gVs, gqs, gths = s_case.stage_c_torch(wR, np.zeros_like(wT))
    _, gWp, gVp, gqp, gthp = p_case.stage_c_torch(np.zeros_like(wR), wT)
    assert rel(gW, gWs + gWp) < 1e-9
    assert rel(gV, gVs + gVp) < 1e-9
    assert rel(gth, gths + gthp) < 1e-9


@pytest.mark.parametrize('seed', [0, 4])
def test_stage_b_reverse_matches_the_torch_eigen_adjoint(host, seed):
    case = Case(seed=seed)
    rng = np.random.default_rng(seed + 7)
    Pn, n = case.B * case.L, case.n
    cz = lambda *s: torch.as_tensor(rng.standard_normal(s) + 1j * rng.standard_normal(s))  # noqa: E731
    gW, gV, gq, gw = cz(Pn, n, n), cz(Pn, n, n), cz(Pn, n), cz(Pn, n)
    want = case.stage_b_torch(gW, gV, gq, gw)
    got = run_stage_b(host, case, gW, gV, gq, gw)
    for l in range(case.L):
        for k in range(3):
            assert rel(got[l][k], want[l][k]) < 1e-9, (l, k)


def test_stage_a_reverse_matches_the_torch_li_adjoint(host):
    case = Case(seed=2, ny=7, nx=5, hu=2, hv=2)
    rng = np.random.default_rng(11)
    cz = lambda *s: torch.as_tensor(rng.standard_normal(s) + 1j * rng.standard_normal(s))  # noqa: E731
    g_conv = [[cz(case.N, case.N) for _ in range(3)] for _ in range(case.L)]
    want = case.stage_a_torch(g_conv)
    got = run_stage_a(host, case, g_conv)
    assert rel(got, want) < 1e-10


@pytest.mark.parametrize('kw', [dict(seed=1), dict(seed=8, L=3, ny=5, nx=7, hu=1, hv=2,
                                                   wavelengths=(560.0, 610.0, 690.0), theta=0.4, phi=-0.7),
                                dict(seed=9, L=1, ny=4, nx=4, hu=3, hv=0, wavelengths=(640.0,), theta=0.0,
                                     phi=0.0, pol=(1.0, 0.0))])
def test_three_reverse_passes_compose_to_the_adjoint_gradient(host, kw):
    """Stages C, B and A chained as a host of the C ABI would chain wb_smm_solve_vjp,
    wb_layer_modes_vjp and wb_assemble_li_vjp give solve_and_grad's raster and thickness
    gradient (crossed and 1D windows, one and three layers, oblique and normal incidence)."""
    case = Case(**kw)
    wR, wT = weights(case, 2)
    gR, gT = eff_cotangents(case, wR, wT)
    gW, gV, gq, gth = run_stage_c(host, case, gR, gT)
    g_conv = run_stage_b(host, case, gW, gV, gq)
    g_eps = run_stage_a(host, case, g_conv)
    loss, _, _, g_eps_t, g_th_t = A.solve_and_grad(case.eps_np, case.th, case.wls, case.period, case.hu, case.hv, wR, wT,
                                                   theta=case.theta, phi=case.phi, eps_top=case.eps_top,
                                                   eps_bot=case.eps_bot, pol=case.pol, impl='torch')
    assert rel(g_eps.real, g_eps_t) < 1e-9
    assert rel(gth.sum(0), g_th_t) < 1e-9
