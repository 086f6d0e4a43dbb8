"""NumPy as an Array-API namespace (NumPy 2.x exports the standard names itself)."""
from numpy import *  # noqa: F401,F403
from numpy import linalg, fft  # noqa: F401
import numpy as _np

bool = _np.bool_  # noqa: A001
__array_api_version__ = '2023.12'
