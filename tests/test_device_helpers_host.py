"""The device code's complex helpers (wb_common.cuh, host- and device-callable) compiled for the
host with nvcc and compared with NumPy: the principal square root and its branch cut, the
half-space kz rule of ports_kernel (sqrt(n^2 - k_par^2), flipped where Re + Im < 0; the oracle's
boundary_kz, conventions.py:655-760 of the reference), Smith's division and the exponential."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import rcwa_oracle as O

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'wavebit_gb300', 'csrc')

HARNESS = r'''
#include "wb_common.cuh"
extern "C" void sqrt_host(const double* z, long long n, double* out) {
  for (long long i = 0; i < n; ++i) { cplx r = csqrt_p(cmk(z[2*i], z[2*i+1])); out[2*i] = r.x; out[2*i+1] = r.y; }
}
// ports_kernel's kz: csqrt_p(nn - kpar), negated where Re + Im < 0
extern "C" void kz_host(const double* nn, const double* kpar, long long n, double* out) {
  for (long long i = 0; i < n; ++i) {
    cplx k = csqrt_p(csub(cmk(nn[2*i], nn[2*i+1]), cmk(kpar[i], 0.0)));
    if (k.x + k.y < 0.0) k = cneg(k);
    out[2*i] = k.x; out[2*i+1] = k.y;
  }
}
extern "C" void div_host(const double* a, const double* b, long long n, double* out) {
  for (long long i = 0; i < n; ++i) { cplx r = cdiv(cmk(a[2*i], a[2*i+1]), cmk(b[2*i], b[2*i+1])); out[2*i] = r.x; out[2*i+1] = r.y; }
}
extern "C" void exp_host(const double* z, long long n, double* out) {
  for (long long i = 0; i < n; ++i) { cplx r = cexp_(cmk(z[2*i], z[2*i+1])); out[2*i] = r.x; out[2*i+1] = r.y; }
}
'''


@pytest.fixture(scope='module')
def lib(tmp_path_factory):
    nvcc = shutil.which('nvcc') or ('/usr/local/cuda/bin/nvcc' if os.path.exists('/usr/local/cuda/bin/nvcc') else None)
    if nvcc is None:
        pytest.skip('nvcc is not available')
    d = tmp_path_factory.mktemp('helpers_host')
    (d / 'h.cu').write_text(HARNESS)
    so = d / 'libh.so'
    subprocess.run([nvcc, '-O2', '-std=c++17', '-Xcompiler', '-fPIC', '-shared', '-I', CSRC, '-o', str(so),
                    str(d / 'h.cu')], check=True, capture_output=True)
    h = ctypes.CDLL(str(so))
    P, LL = ctypes.c_void_p, ctypes.c_longlong
    for name, nargs in (('sqrt_host', 1), ('kz_host', 2), ('div_host', 2), ('exp_host', 1)):
        getattr(h, name).argtypes = [P] * nargs + [LL, P]
    return h


def _call(fn, *arrays):
    arrays = [np.ascontiguousarray(a) for a in arrays]
    n = arrays[0].shape[0]
    out = np.zeros(n, np.complex128)
    fn(*[a.ctypes.data for a in arrays], n, out.ctypes.data)
    return out


def _samples():
    rng = np.random.default_rng(0)
    z = rng.standard_normal(2000) * 10 ** rng.uniform(-3, 3, 2000) + 1j * rng.standard_normal(2000)
    edge = np.array([-4.0 + 0j, -4.0 - 0j, complex(-4.0, -0.0), complex(-4.0, 1e-300), 4 + 0j, 0j,
                     complex(0.0, -0.0), 1j, -1j, complex(-1e-20, 1e-20), complex(-2.5, -1e-16)])
    return np.concatenate([z, edge])


def test_principal_square_root_matches_numpy_including_the_branch_cut(lib):
    z = _samples()
    got = _call(lib.sqrt_host, z)
    want = np.sqrt(z)
    assert np.allclose(got, want, rtol=4e-16 * 4, atol=0)
    # on the cut the sign of the zero imaginary part picks the side, as in C99 csqrt:
    # sqrt(-4 + 0i) = +2i and sqrt(-4 - 0i) = -2i
    cut = {i: got[i] for i in range(2000, 2003)}
    assert cut[2000] == 2j and cut[2001] == 2j and cut[2002] == -2j


def test_half_space_kz_is_the_oracle_boundary_kz(lib):
    rng = np.random.default_rng(1)
    eps = np.concatenate([rng.uniform(0.5, 13, 300) + 1j * rng.uniform(0, 2, 300),      # lossy dielectrics
                          -rng.uniform(1, 30, 100) + 1j * rng.uniform(0, 3, 100),      # metals
                          np.array([1.0, 2.25, 12.25 + 0j])])
    kpar = rng.uniform(0, 4, eps.shape[0]) ** 2
    kpar[-3:] = [1.0, 2.25, 0.0]                                        # exactly at cutoff, and normal
    got = _call(lib.kz_host, eps, kpar)
    want = O.boundary_kz(eps, kpar)
    assert np.abs(got - want).max() <= 1e-15 * np.abs(want).max()
    assert np.all(got.real + got.imag >= 0)


def test_division_and_exponential_match_numpy(lib):
    rng = np.random.default_rng(2)
    a = rng.standard_normal(1000) + 1j * rng.standard_normal(1000)
    b = (rng.standard_normal(1000) + 1j * rng.standard_normal(1000)) * 10 ** rng.uniform(-150, 150, 1000)
    q = _call(lib.div_host, a, b)
    assert np.allclose(q, a / b, rtol=1e-15, atol=0)
    z = rng.uniform(-50, 5, 1000) + 1j * rng.uniform(-30, 30, 1000)
    assert np.allclose(_call(lib.exp_host, z), np.exp(z), rtol=1e-14, atol=0)
