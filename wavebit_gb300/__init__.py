"""wavebit_gb300: Wavebit's RCWA raster layer path on GB300 (sm_103a) CUDA kernels.

``engine`` is the torch-facing functional layer over libwbgpu.so (include/wavebit_gb300.h).
"""
__version__ = '0.2.1'

from . import _lib  # noqa: F401
from . import engine  # noqa: F401
from . import rcwa  # noqa: F401

__all__ = ['engine', 'rcwa', '__version__']
