"""The C ABI library loads on a CPU-only host and exports every symbol its header declares;
the host-only entry points behave (no GPU calls here)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'wavebit_gb300.h')


def _declared():
    text = open(HEADER).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(wb_[a-z_0-9]+)\s*\(', text)))


@pytest.fixture(scope='module')
def lib():
    from wavebit_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        import __graft_entry__ as g
        g.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 10
    for name in names:
        assert hasattr(lib, name), name


def test_abi_version(lib):
    assert lib.wb_version() == 202


def test_binding_table_covers_the_header():
    from wavebit_gb300 import _lib
    assert set(_declared()) == set(_lib.SIGNATURES)


def test_index_tables_are_bit_exact(lib):
    from oracle import rcwa_oracle as O
    for hu, hv in ((0, 0), (3, 1), (7, 7), (12, 5)):
        nu, nv = 2 * hu + 1, 2 * hv + 1
        lu, lv = np.zeros(nu, np.int32), np.zeros(nv, np.int32)
        tu, tv = np.zeros(nu * nu, np.int32), np.zeros(nv * nv, np.int32)
        assert lib.wb_build_indices(hu, hv, lu.ctypes.data, lv.ctypes.data, tu.ctypes.data, tv.ctypes.data) == 0
        assert np.array_equal(lu, O.order_labels(hu)) and np.array_equal(lv, O.order_labels(hv))
        assert np.array_equal(tu, O.toeplitz_positions(hu)) and np.array_equal(tv, O.toeplitz_positions(hv))


def test_invalid_orders_are_refused_with_a_message(lib):
    from wavebit_gb300 import _lib
    rc = lib.wb_build_indices(-1, 2, None, None, None, None)
    assert rc == _lib.WB_E_INVALID
    assert 'orders' in _lib.last_error()


def test_order_windows_end_where_the_kernels_on_chip_buffers_do(lib):
    from wavebit_gb300 import _lib
    for hu, hv in ((0, 43), (28, 28), (1614, 0)):
        assert lib.wb_build_indices(hu, hv, None, None, None, None) == _lib.WB_E_INVALID, (hu, hv)
        assert 'hv <= 42' in _lib.last_error()
        assert lib.wb_workspace_bytes(hu, hv, 1, 1, 0) == 0
    for hu, hv in ((27, 27), (1613, 0), (18, 42)):
        assert lib.wb_workspace_bytes(hu, hv, 1, 1, 0) > 0, (hu, hv)


def test_create_without_a_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    from wavebit_gb300 import _lib
    h = ctypes.c_void_p()
    rc = lib.wb_create(0, 0, ctypes.byref(h))
    assert rc == _lib.WB_E_CUDA and not h.value
    assert 'device' in _lib.last_error().lower()


def test_workspace_estimate_grows_with_the_chunk(lib):
    a = lib.wb_solve_workspace_bytes(7, 7, 4, 16)
    b = lib.wb_solve_workspace_bytes(7, 7, 4, 32)
    assert 0 < a < b
    assert lib.wb_solve_workspace_bytes(-1, 7, 4, 16) == 0


def test_workspace_estimate_per_form(lib):
    """The FP64 form matches wb_solve_workspace_bytes; the mixed forms need more (FP32 copies,
    group slots, refinement vectors); bad precisions give 0."""
    from wavebit_gb300 import _lib
    fp64 = lib.wb_workspace_bytes(7, 7, 4, 16, _lib.PRECISION['double'])
    assert fp64 == lib.wb_solve_workspace_bytes(7, 7, 4, 16)
    for name in ('mixed', 'mixed_fp32', 'mixed_df64_eig'):
        assert lib.wb_workspace_bytes(7, 7, 4, 16, _lib.PRECISION[name]) > fp64, name
    assert lib.wb_workspace_bytes(7, 7, 4, 16, 99) == 0 and lib.wb_workspace_bytes(7, 7, 4, 16, -1) == 0


def test_smm_solve_refuses_bad_arguments_before_any_device_work(lib):
    """wb_smm_solve checks pointers, sizes and the precision on the host (no GPU calls): NULL
    arguments, empty batches and forms other than FP64 / MIXED are WB_E_INVALID."""
    from wavebit_gb300 import _lib
    fake = ctypes.create_string_buffer(64)             # a non-NULL address, never dereferenced here
    p = ctypes.addressof(fake)
    args = lambda B, prec, h=p: (h, B, 2, 1, 1) + (p,) * 15 + (prec, None)
    assert lib.wb_smm_solve(*args(4, 0, None)) == _lib.WB_E_INVALID
    assert 'NULL' in _lib.last_error()
    assert lib.wb_smm_solve(*args(0, 0)) == _lib.WB_E_INVALID
    assert lib.wb_smm_solve(*args(4, _lib.PRECISION['mixed_df64'])) == _lib.WB_E_INVALID
    assert 'precision' in _lib.last_error()


def test_scattering_matrix_refuses_bad_arguments_before_any_device_work(lib):
    """wb_scattering_matrix checks pointers and sizes on the host: NULL arguments, empty batches
    and bad orders are WB_E_INVALID with a message."""
    from wavebit_gb300 import _lib
    fake = ctypes.create_string_buffer(64)
    p = ctypes.addressof(fake)
    args = lambda B, hu=1, h=p, out=p: (h, B, 2, hu, 1) + (p,) * 10 + (out, p, p, p, p, None)
    assert lib.wb_scattering_matrix(*args(4, h=None)) == _lib.WB_E_INVALID
    assert 'NULL' in _lib.last_error()
    assert lib.wb_scattering_matrix(*args(4, out=None)) == _lib.WB_E_INVALID
    assert lib.wb_scattering_matrix(*args(0)) == _lib.WB_E_INVALID
    assert lib.wb_scattering_matrix(*args(4, hu=-1)) == _lib.WB_E_INVALID
    assert 'wb_scattering_matrix' in _lib.last_error()


def test_reverse_passes_refuse_bad_arguments_before_any_device_work(lib):
    """The wb_*_vjp entry points check pointers and sizes on the host: NULL required arguments,
    empty batches and bad orders are WB_E_INVALID with a message naming the entry point; the
    optional cotangents may be NULL."""
    from wavebit_gb300 import _lib
    fake = ctypes.create_string_buffer(64)
    p = ctypes.addressof(fake)
    smm = lambda B, h=p, out=p: (h, B, 2, 1, 1) + (p,) * 11 + (None, None, out, p, p, p, p, None)
    assert lib.wb_smm_solve_vjp(*smm(2, h=None)) == _lib.WB_E_INVALID
    assert 'NULL' in _lib.last_error()
    assert lib.wb_smm_solve_vjp(*smm(2, out=None)) == _lib.WB_E_INVALID
    assert lib.wb_smm_solve_vjp(*smm(0)) == _lib.WB_E_INVALID
    assert 'wb_smm_solve_vjp' in _lib.last_error()
    modes = lambda P, hu=1, conv=p: (p, P, hu, 1, 2, conv) + (p,) * 7 + (None,) * 4 + (p, None, None)
    assert lib.wb_layer_modes_vjp(*modes(3, conv=None)) == _lib.WB_E_INVALID
    assert lib.wb_layer_modes_vjp(*modes(0)) == _lib.WB_E_INVALID
    assert lib.wb_layer_modes_vjp(*modes(3, hu=-2)) == _lib.WB_E_INVALID
    assert 'wb_layer_modes_vjp' in _lib.last_error()
    asm = lambda L, hv=1, g=p: (p, p, L, 8, 8, 1, hv, p, p, None, None, None, g, None, None)
    assert lib.wb_assemble_li_vjp(*asm(2, g=None)) == _lib.WB_E_INVALID
    assert lib.wb_assemble_li_vjp(*asm(0)) == _lib.WB_E_INVALID
    assert lib.wb_assemble_li_vjp(*asm(2, hv=43)) == _lib.WB_E_INVALID
    assert 'wb_assemble_li_vjp' in _lib.last_error()


def test_header_is_plain_c_and_a_c_program_links(lib, tmp_path):
    """The boundary is a C ABI: the public header compiles as strict C99 (no C++ or torch types)
    and a C program links libwbgpu.so and calls its host-only entry points."""
    import shutil
    import subprocess
    from wavebit_gb300 import _lib
    gcc = shutil.which('gcc')
    if gcc is None:
        pytest.skip('gcc is not available')
    src = tmp_path / 'main.c'
    src.write_text('''
#include <stdio.h>
#include "wavebit_gb300.h"
int main(void) {
  int32_t lu[5], lv[3], tu[25], tv[9];
  int rc = wb_build_indices(2, 1, lu, lv, tu, tv);
  printf("%d %d %d %d %zu\\n", wb_version(), rc, lu[0], tv[8], wb_workspace_bytes(2, 1, 1, 1, WB_PRECISION_FP64));
  return rc;
}
''')
    exe = tmp_path / 'main'
    libdir = os.path.dirname(_lib.LIB_PATH)
    cc = subprocess.run([gcc, '-std=c99', '-Wall', '-Wextra', '-Werror', '-pedantic', '-I', os.path.join(ROOT, 'include'),
                         '-o', str(exe), str(src), '-L', libdir, '-lwbgpu', f'-Wl,-rpath,{libdir}'],
                        capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
    version, rc, first, last, ws = run.stdout.split()
    assert (int(version), int(rc), int(first), int(last)) == (202, 0, -2, 2) and int(ws) > 0
