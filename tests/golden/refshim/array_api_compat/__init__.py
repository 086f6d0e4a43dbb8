"""Minimal stand-in for the ``array_api_compat`` package, written from the Array-API standard.

Test infrastructure only: it lets the reference package be imported in a container where the
real ``array_api_compat`` is not installed, so that golden fixtures can be generated from the
reference's own NumPy and PyTorch paths. ``array_namespace`` maps NumPy arrays and Python scalars
to the NumPy namespace (NumPy 2.x already implements the standard names the reference uses) and
torch tensors to the torch one (``array_api_compat.torch``, the standard's names mapped onto
torch).
"""
import numpy as _np

from . import numpy as _numpy_ns


def array_namespace(*xs, **_kw):
    for x in xs:
        if x is None or isinstance(x, (bool, int, float, complex)):
            continue
        if isinstance(x, (_np.ndarray, _np.generic)):
            continue
        mod = type(x).__module__
        if mod.startswith('torch'):
            from . import torch as _torch_ns
            return _torch_ns
        raise TypeError(f'unsupported array type {type(x)!r}')
    return _numpy_ns


def to_device(x, device, /, **_kw):
    if type(x).__module__.startswith('torch'):
        return x.to(device)
    if device is None or str(device) == 'cpu':
        return x
    raise ValueError(f'numpy arrays live on the cpu, not {device!r}')


def device(x, /):
    return x.device if type(x).__module__.startswith('torch') else 'cpu'


def is_numpy_array(x):
    return isinstance(x, _np.ndarray)


def is_torch_array(x):
    return type(x).__module__.startswith('torch')


def is_jax_array(x):
    return False
