"""ctypes binding of libwbgpu.so (the C ABI in include/wavebit_gb300.h).

The library is built in-tree by ``wavebit_gb300/csrc/build.py`` (``__graft_entry__.build()``
runs it). There is no CPU fallback: if the library is missing, every entry point raises.
"""
import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, 'libwbgpu.so')

WB_OK = 0
WB_E_INVALID, WB_E_NOMEM, WB_E_SINGULAR, WB_E_NOCONV, WB_E_NONFINITE, WB_E_CUDA = 1, 2, 3, 4, 5, 6
WB_ST_SINGULAR, WB_ST_NOCONV, WB_ST_NONFINITE, WB_ST_GRAZING = 1, 2, 4, 8
WB_TUNE_QR_THREADS, WB_TUNE_HRD_THREADS, WB_TUNE_LU_THREADS, WB_TUNE_TENSOR_CORES, WB_TUNE_HRD_BLOCKED = 0, 1, 2, 3, 4
PRECISION = {'double': 0, 'fp64': 0, 'mixed': 1, 'mixed_fp32': 2, 'mixed_df64': 3, 'mixed_df64_eig': 4}

_c = ctypes
_vp, _i, _sz, _ll = _c.c_void_p, _c.c_int, _c.c_size_t, _c.c_longlong

# name: (restype, argtypes)
SIGNATURES = {
    'wb_version': (_i, []),
    'wb_last_error': (_i, [_c.c_char_p, _sz]),
    'wb_create': (_i, [_i, _sz, _c.POINTER(_vp)]),
    'wb_destroy': (_i, [_vp]),
    'wb_reserve': (_i, [_vp, _sz]),
    'wb_build_indices': (_i, [_i, _i, _vp, _vp, _vp, _vp]),
    'wb_assemble_li': (_i, [_vp, _vp, _i, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    'wb_assemble_li_integrated': (_i, [_vp, _vp, _i, _i, _i, _vp, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    'wb_layer_modes': (_i, [_vp, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
    'wb_solve_batch': (_i, [_vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                            _vp, _vp, _vp, _vp, _i, _vp]),
    'wb_scattering_matrix': (_i, [_vp, _i, _i, _i, _i] + [_vp] * 16),
    'wb_smm_solve': (_i, [_vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                          _vp, _vp, _vp, _vp, _i, _vp]),
    'wb_etm_solve': (_i, [_vp, _i, _i, _i, _i] + [_vp] * 16),
    'wb_layer_amplitudes': (_i, [_vp, _i, _i, _i, _i] + [_vp] * 11 + [_i] + [_vp] * 7),
    'wb_solve_host': (_i, [_vp, _i, _i, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                           _vp, _vp, _vp, _vp, _i]),
    'wb_solve_workspace_bytes': (_sz, [_i, _i, _i, _i]),
    'wb_workspace_bytes': (_sz, [_i, _i, _i, _i, _i]),
    'wb_kernel_launches': (_ll, [_vp]),
    'wb_set_tuning': (_i, [_i, _i]),
    'wb_get_tuning': (_i, [_i]),
    'wb_profile_qr': (_i, [_i]),
    'wb_tensor_core_errors': (_ll, []),
    'wb_profile_qr_read': (_i, [_i, _vp, _vp, _vp]),
    'wb_assemble_li_noalloc': (_i, [_vp, _i, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    'wb_smm_solve_vjp': (_i, [_vp, _i, _i, _i, _i] + [_vp] * 19),
    'wb_layer_modes_vjp': (_i, [_vp, _i, _i, _i, _i] + [_vp] * 15),
    'wb_assemble_li_vjp': (_i, [_vp, _vp, _i, _i, _i, _i, _i] + [_vp] * 8),
    'wb_assemble_li_noalloc_limit': (_sz, []),
}

_lib = None
_lock = threading.Lock()


class WavebitError(RuntimeError):
    """A failure reported by libwbgpu.so; ``code`` is the WB_E_* value."""

    def __init__(self, code, message):
        super().__init__(f'[WB_E {code}] {message}')
        self.code = code


def load():
    """Load libwbgpu.so and bind every entry point the public header declares."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f'{LIB_PATH} is missing: build it first (python -c "import __graft_entry__ as g; g.build()"). '
                'wavebit_gb300 has no CPU fallback.')
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(1024)
    load().wb_last_error(buf, len(buf))
    return buf.value.decode(errors='replace')


def check(rc):
    if rc != WB_OK:
        raise WavebitError(rc, last_error())
    return rc


def ptr(t):
    """Device (or host) address of a torch tensor / numpy array, or None."""
    if t is None:
        return None
    if hasattr(t, 'data_ptr'):
        return t.data_ptr()
    return t.ctypes.data


class Handle:
    """Owns one ``wb_handle``: a device and its scratch arena."""

    def __init__(self, device=0, hbm_budget=0):
        self.lib = load()
        h = ctypes.c_void_p()
        check(self.lib.wb_create(int(device), int(hbm_budget), ctypes.byref(h)))
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            self.lib.wb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def launches(self):
        return int(self.lib.wb_kernel_launches(self.h))


_handles = {}


def handle(device=0, hbm_budget=0):
    """The process-wide handle of ``device`` (created on first use)."""
    key = int(device)
    if key not in _handles:
        _handles[key] = Handle(key, hbm_budget)
    return _handles[key]
