"""The integrated series' device code on the CPU: ``wb_series.cuh`` is host- and device-callable,
so a small host harness compiled here with nvcc drives ``segment_series_at`` over every thread
index of stage A's three series launches (column series of eps and 1/eps, the row series of the
inner inverses, the direct rule), with the other stage-A steps restated in NumPy on the kernels'
buffer layouts; the slots must equal the oracle's integrated Li slots."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import rcwa_oracle as O

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), 'wavebit_gb300', 'csrc')

HARNESS = r'''
#include "wb_series.cuh"
extern "C" void seg_launch_host(const double* in, long long n_lines, int lpg, long long gs, long long ls,
                                long long ps, int npts, int h, int rec, const double* edges, long long lps,
                                int nrows, double* out) {
  const long long total = n_lines * (4 * h + 1);
  for (long long i = 0; i < total; ++i)
    wb::segment_series_at(i, (const cplx*)in, lpg, gs, ls, ps, npts, h, rec, edges, lps, nrows, (cplx*)out);
}
'''


@pytest.fixture(scope='module')
def lib(tmp_path_factory):
    nvcc = shutil.which('nvcc') or ('/usr/local/cuda/bin/nvcc' if os.path.exists('/usr/local/cuda/bin/nvcc') else None)
    if nvcc is None:
        pytest.skip('nvcc is not available')
    d = tmp_path_factory.mktemp('series_host')
    src = d / 'harness.cu'
    src.write_text(HARNESS)
    so = d / 'libharness.so'
    subprocess.run([nvcc, '-O2', '-std=c++17', '-Xcompiler', '-fPIC', '-shared', '-I', CSRC, '-o', str(so), str(src)],
                   check=True, capture_output=True)
    h = ctypes.CDLL(str(so))
    P, LL, I = ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int
    h.seg_launch_host.argtypes = [P, LL, I, LL, LL, LL, I, I, I, P, LL, I, P]
    return h


def _launch(lib, buf, n_lines, lpg, gs, ls, ps, npts, h, rec, edges, lps, nrows, out, out_off):
    o = out.reshape(-1)[out_off:]
    lib.seg_launch_host(buf.ctypes.data, n_lines, lpg, gs, ls, ps, npts, h, rec, edges.ctypes.data, lps, nrows,
                        o.ctypes.data)


def _assemble(lib, eps, xe, ye, hu, hv):
    """assemble_li with edges (wb_assemble.cu), the series on the harness."""
    L, ny, nx = eps.shape
    nu, nv, nku, nkv = 2 * hu + 1, 2 * hv + 1, 4 * hu + 1, 4 * hv + 1
    N = nu * nv
    eps, xe, ye = (np.ascontiguousarray(a) for a in (eps.astype(complex), xe.astype(float), ye.astype(float)))
    cv = np.zeros(2 * L * nx * nkv, complex)
    for rec in range(2):
        _launch(lib, eps, L * nx, nx, ny * nx, 1, nx, ny, hv, rec, ye, nx, L, cv, rec * L * nx * nkv)
    inner = np.zeros(2 * L * nv * nv * nx, complex)
    pos = np.arange(nv)[:, None] - np.arange(nv)[None, :] + 2 * hv
    for line in range(2 * L * nx):
        g, x = divmod(line, nx)
        Ti = np.linalg.inv(cv[line * nkv:(line + 1) * nkv][pos])
        inner[(g * nv * nv + np.arange(nv * nv)) * nx + x] = Ti.reshape(-1)
    cu = np.zeros(2 * L * nv * nv * nku, complex)
    _launch(lib, inner, 2 * L * nv * nv, 1, nx, 0, 1, nx, hu, 0, xe, nv * nv, L, cu, 0)
    c2 = np.zeros(L * nkv * nku, complex)
    _launch(lib, cv, L * nkv, nkv, nx * nkv, 1, nkv, nx, hu, 0, xe, nkv, L, c2, 0)
    i = np.arange(N)
    r, m = np.divmod(i, nu)
    out = []
    for l in range(L):
        du = (m[:, None] - m[None, :] + 2 * hu)
        pre = cu[((l * nv + r[:, None]) * nv + r[None, :]) * nku + du]
        epy = cu[(((L + l) * nv + r[:, None]) * nv + r[None, :]) * nku + du]
        direct = c2[(l * nkv + (r[:, None] - r[None, :] + 2 * hv)) * nku + du]
        out.append((np.linalg.inv(pre), epy, np.linalg.inv(direct)))
    return out


def _blocky(rng, ny, nx):
    by, bx = rng.integers(1, 5, size=2)
    base = rng.choice(np.array([12.25 + 0.3j, 2.1, 1.0]), size=(by, bx))
    ry, rx = np.sort(rng.integers(0, ny, size=by - 1)), np.sort(rng.integers(0, nx, size=bx - 1))
    return base[np.searchsorted(ry, np.arange(ny), side='right')][:, np.searchsorted(rx, np.arange(nx), side='right')]


@pytest.mark.parametrize('hu,hv', [(3, 3), (2, 4), (5, 0), (0, 3)])
def test_device_series_code_builds_the_oracle_slots(lib, hu, hv):
    rng = np.random.default_rng(100 * hu + hv)
    cells = [_blocky(rng, 20, 24) for _ in range(3)]
    comp = [O.compression_indices(c) for c in cells]
    comp = [(c[np.ix_(ri, ci)], x, y) for c, (ri, ci, x, y) in zip(cells, comp)]
    for cell, (cc, x, y) in zip(cells, comp):                      # one layer at a time
        got = _assemble(lib, cc[None], x[None], y[None], hu, hv)[0]
        for a, b in zip(got, O.li_conv_integrated(cell, hu, hv)):
            assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()
    # layers of one compressed shape with their own edges, in one launch sequence
    shp = comp[0][0].shape
    batch = [comp[0]] + [(rng.standard_normal(shp) + 3 + 0.1j,
                          np.append(np.sort(rng.random(shp[1] - 1)), 1.0),
                          np.append(np.sort(rng.random(shp[0] - 1)), 1.0)) for _ in range(2)]
    got = _assemble(lib, np.stack([b[0] for b in batch]), np.stack([b[1] for b in batch]),
                    np.stack([b[2] for b in batch]), hu, hv)
    for g, (cc, x, y) in zip(got, batch):
        want = O.li_conv(cc, hu, hv, su=O.segment_series(*O.segment_bounds(x), hu),
                         sv=O.segment_series(*O.segment_bounds(y), hv))
        for a, b in zip(g, want):
            assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()
