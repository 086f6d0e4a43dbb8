"""PyTorch as an Array-API namespace: test infrastructure only, so that the reference's torch
backend (its differentiable path) runs in a container without the third-party package. Written
from the Array-API standard: the standard's names and keyword forms, mapped onto torch; every
other name falls through to torch itself."""
import builtins as _b
import sys as _sys
import types as _types

import torch as _t

__array_api_version__ = '2023.12'

bool = _t.bool  # noqa: A001
float32, float64, complex64, complex128 = _t.float32, _t.float64, _t.complex64, _t.complex128
int32, int64, int8, uint8 = _t.int32, _t.int64, _t.int8, _t.uint8
nan, inf, pi, e = float('nan'), float('inf'), 3.141592653589793, 2.718281828459045


def _dt(dtype):
    return dtype


def asarray(obj, dtype=None, device=None, copy=None, requires_grad=None):
    if isinstance(obj, _t.Tensor):
        out = obj
        if dtype is not None and out.dtype != dtype:
            out = out.to(dtype)
        if device is not None:
            out = out.to(device)
        if copy:
            out = out.clone()
    else:
        if dtype is None:
            import numpy as _np
            if isinstance(obj, (_b.bool, int, float, complex)) or isinstance(obj, (list, tuple)):
                a = _np.asarray(obj)
                if a.dtype.kind == 'f':
                    a = a.astype(_np.float64)
                elif a.dtype.kind == 'c':
                    a = a.astype(_np.complex128)
                obj = a
            out = _t.as_tensor(obj, device=device)
        else:
            out = _t.as_tensor(obj, dtype=dtype, device=device)
    if requires_grad is not None and requires_grad and not out.requires_grad:
        out = out.detach().requires_grad_(True)
    return out


def astype(x, dtype, copy=True, device=None):
    out = x.to(dtype)
    return out.to(device) if device is not None else out


def _fdefault(kw):
    if kw.get('dtype') is None:
        kw['dtype'] = _t.float64
    return kw


def zeros(shape, dtype=None, device=None):
    return _t.zeros(shape, **_fdefault(dict(dtype=dtype, device=device)))


def ones(shape, dtype=None, device=None):
    return _t.ones(shape, **_fdefault(dict(dtype=dtype, device=device)))


def full(shape, fill_value, dtype=None, device=None):
    if dtype is None:
        dtype = _t.complex128 if isinstance(fill_value, complex) else (_t.float64 if isinstance(fill_value, float) else None)
    return _t.full(shape if isinstance(shape, tuple) else (shape,) if isinstance(shape, int) else tuple(shape),
                   fill_value, dtype=dtype, device=device)


def empty(shape, dtype=None, device=None):
    return _t.empty(shape, **_fdefault(dict(dtype=dtype, device=device)))


def eye(n_rows, n_cols=None, k=0, dtype=None, device=None):
    dtype = dtype or _t.float64
    if k == 0:
        return _t.eye(n_rows, n_cols if n_cols is not None else n_rows, dtype=dtype, device=device)
    m = n_cols if n_cols is not None else n_rows
    return _t.diag(_t.ones(min(n_rows, m - k) if k >= 0 else min(n_rows + k, m), dtype=dtype, device=device), k)[:n_rows, :m]


def zeros_like(x, dtype=None, device=None):
    return _t.zeros_like(x, dtype=dtype, device=device)


def ones_like(x, dtype=None, device=None):
    return _t.ones_like(x, dtype=dtype, device=device)


def full_like(x, fill_value, dtype=None, device=None):
    return _t.full_like(x, fill_value, dtype=dtype, device=device)


def arange(start, stop=None, step=1, dtype=None, device=None):
    if stop is None:
        start, stop = 0, start
    if dtype is None and builtins_any_float(start, stop, step):
        dtype = _t.float64
    return _t.arange(start, stop, step, dtype=dtype, device=device)


def builtins_any_float(*vals):
    return _b.any(isinstance(v, float) for v in vals)


def linspace(start, stop, num, dtype=None, device=None, endpoint=True):
    dtype = dtype or (_t.complex128 if isinstance(start, complex) or isinstance(stop, complex) else _t.float64)
    if endpoint:
        return _t.linspace(start, stop, num, dtype=dtype, device=device)
    return _t.linspace(start, stop, num + 1, dtype=dtype, device=device)[:-1]


def _axis(axis):
    return tuple(axis) if isinstance(axis, list) else axis


def sum(x, axis=None, dtype=None, keepdims=False):
    if axis is None:
        out = _t.sum(x, dtype=dtype)
        return out.reshape((1,) * x.ndim) if keepdims else out
    return _t.sum(x, dim=_axis(axis), keepdim=keepdims, dtype=dtype)


def prod(x, axis=None, dtype=None, keepdims=False):
    if axis is None:
        return _t.prod(x, dtype=dtype)
    return _t.prod(x, dim=axis, keepdim=keepdims, dtype=dtype)


def _red(fn, x, axis, keepdims):
    if axis is None:
        out = fn(x)
        return out.reshape((1,) * x.ndim) if keepdims else out
    if isinstance(axis, (tuple, list)):
        out = x
        for a in sorted((a % x.ndim for a in axis), reverse=True):
            out = fn(out, dim=a, keepdim=keepdims)
            out = out[0] if isinstance(out, tuple) else out
        return out
    out = fn(x, dim=axis, keepdim=keepdims)
    return out[0] if isinstance(out, tuple) else out


def max(x, axis=None, keepdims=False):  # noqa: A001
    return _red(_t.amax if axis is not None else _t.max, x, axis, keepdims)


def min(x, axis=None, keepdims=False):  # noqa: A001
    return _red(_t.amin if axis is not None else _t.min, x, axis, keepdims)


def mean(x, axis=None, keepdims=False):
    return _t.mean(x) if axis is None else _t.mean(x, dim=_axis(axis), keepdim=keepdims)


def any(x, axis=None, keepdims=False):  # noqa: A001
    x = _t.as_tensor(x)
    return _t.any(x) if axis is None else _t.any(x, dim=axis, keepdim=keepdims)


def all(x, axis=None, keepdims=False):  # noqa: A001
    x = _t.as_tensor(x)
    return _t.all(x) if axis is None else _t.all(x, dim=axis, keepdim=keepdims)


def argmax(x, axis=None, keepdims=False):
    return _t.argmax(x, dim=axis, keepdim=keepdims)


def argmin(x, axis=None, keepdims=False):
    return _t.argmin(x, dim=axis, keepdim=keepdims)


def argsort(x, axis=-1, descending=False, stable=True):
    return _t.argsort(x, dim=axis, descending=descending, stable=stable)


def sort(x, axis=-1, descending=False, stable=True):
    return _t.sort(x, dim=axis, descending=descending, stable=stable).values


def cumulative_sum(x, axis=None, dtype=None, include_initial=False):
    out = _t.cumsum(x, dim=0 if axis is None else axis, dtype=dtype)
    if include_initial:
        z = _t.zeros_like(out.narrow(0 if axis is None else axis, 0, 1))
        out = _t.cat([z, out], dim=0 if axis is None else axis)
    return out


def cumsum(x, axis=None, dtype=None):
    return _t.cumsum(x, dim=0 if axis is None else axis, dtype=dtype)


def concat(arrays, axis=0):
    return _t.cat(list(arrays), dim=axis)


def stack(arrays, axis=0):
    return _t.stack(list(arrays), dim=axis)


def permute_dims(x, axes):
    return x.permute(*axes)


def matrix_transpose(x):
    return x.transpose(-1, -2)


def reshape(x, shape, copy=None):
    return _t.reshape(x, tuple(shape))


def expand_dims(x, axis=0):
    return _t.unsqueeze(x, axis)


def squeeze(x, axis):
    return _t.squeeze(x, axis)


def flip(x, axis=None):
    return _t.flip(x, dims=tuple(range(x.ndim)) if axis is None else (axis if isinstance(axis, tuple) else (axis,)))


def roll(x, shift, axis=None):
    if axis is None:
        return _t.roll(x, shift)
    return _t.roll(x, shift, dims=axis)


def take(x, indices, axis=None):
    indices = _t.as_tensor(indices, device=x.device)
    if axis is None:
        return x.reshape(-1)[indices]
    return _t.index_select(x, axis, indices.reshape(-1)).reshape(
        x.shape[:axis % x.ndim] + indices.shape + x.shape[axis % x.ndim + 1:]) if indices.ndim != 1 else \
        _t.index_select(x, axis, indices)


def repeat(x, repeats, axis=None):
    if axis is None:
        return _t.repeat_interleave(x.reshape(-1), repeats)
    return _t.repeat_interleave(x, repeats, dim=axis)


def broadcast_to(x, shape):
    return _t.broadcast_to(x, tuple(shape))


def broadcast_arrays(*arrays):
    return list(_t.broadcast_tensors(*arrays))


def _as_t(v, like):
    if isinstance(v, _t.Tensor):
        return v
    return _t.as_tensor(v, dtype=like.dtype if isinstance(v, (int, float, complex)) and like is not None and
                        (like.is_complex() or like.is_floating_point()) else None,
                        device=like.device if like is not None else None)


def where(condition, x1, x2):
    like = x1 if isinstance(x1, _t.Tensor) else (x2 if isinstance(x2, _t.Tensor) else None)
    if like is not None:
        dt = _t.result_type(x1, x2) if isinstance(x1, _t.Tensor) and isinstance(x2, _t.Tensor) else like.dtype
        if not isinstance(x1, _t.Tensor):
            x1 = _t.as_tensor(x1, dtype=dt, device=like.device)
        if not isinstance(x2, _t.Tensor):
            x2 = _t.as_tensor(x2, dtype=dt, device=like.device)
        if x1.dtype != x2.dtype:
            rt = _t.promote_types(x1.dtype, x2.dtype)
            x1, x2 = x1.to(rt), x2.to(rt)
    return _t.where(_t.as_tensor(condition), x1, x2)


def result_type(*args):
    ts = [a for a in args if isinstance(a, (_t.Tensor, _t.dtype))]
    out = None
    for a in args:
        d = a if isinstance(a, _t.dtype) else (a.dtype if isinstance(a, _t.Tensor) else None)
        if d is None:
            continue
        out = d if out is None else _t.promote_types(out, d)
    for a in args:
        if isinstance(a, complex) and out is not None and not out.is_complex:
            out = _t.promote_types(out, _t.complex128)
        elif isinstance(a, float) and out is not None and not (out.is_floating_point or out.is_complex):
            out = _t.promote_types(out, _t.float64)
    del ts
    return out


def isdtype(dtype, kind):
    if isinstance(kind, tuple):
        return _b.any(isdtype(dtype, k) for k in kind)
    if isinstance(kind, _t.dtype):
        return dtype == kind
    if kind == 'bool':
        return dtype == _t.bool
    if kind == 'complex floating':
        return dtype.is_complex
    if kind == 'real floating':
        return dtype.is_floating_point
    if kind == 'numeric':
        return dtype != _t.bool
    if kind in ('integral', 'signed integer', 'unsigned integer'):
        return not dtype.is_floating_point and not dtype.is_complex and dtype != _t.bool
    raise ValueError(kind)


def finfo(dtype):
    return _t.finfo(dtype)


def iinfo(dtype):
    return _t.iinfo(dtype)


def real(x):
    return _t.real(x) if x.is_complex() else x


def imag(x):
    return _t.imag(x) if x.is_complex() else _t.zeros_like(x)


def conj(x):
    return _t.conj(x).resolve_conj() if x.is_complex() else x


def atan(x):
    return _t.atan(x)


def asin(x):
    return _t.asin(x)


def atan2(x1, x2):
    return _t.atan2(x1, x2)


def pow(x1, x2):
    return _t.pow(x1, x2)


def nonzero(x):
    return tuple(_t.nonzero(x, as_tuple=True))


def clip(x, min=None, max=None):  # noqa: A002
    return _t.clamp(x, min=min, max=max)


def einsum(spec, *ops):
    return _t.einsum(spec, *ops)


def diag(x, k=0):
    return _t.diag(x, k)


def matmul(a, b):
    return _t.matmul(a, b)


def isfinite(x):
    return _t.isfinite(_t.as_tensor(x))


def maximum(a, b):
    a_t, b_t = isinstance(a, _t.Tensor), isinstance(b, _t.Tensor)
    if a_t and b_t:
        return _t.maximum(a, b)
    return _t.clamp(a, min=b) if a_t else _t.clamp(b, min=a)


def minimum(a, b):
    a_t, b_t = isinstance(a, _t.Tensor), isinstance(b, _t.Tensor)
    if a_t and b_t:
        return _t.minimum(a, b)
    return _t.clamp(a, max=b) if a_t else _t.clamp(b, max=a)


def hypot(a, b):
    return _t.hypot(a, b)


def logical_and(a, b):
    return _t.logical_and(_t.as_tensor(a), _t.as_tensor(b))


def logical_or(a, b):
    return _t.logical_or(_t.as_tensor(a), _t.as_tensor(b))


def logical_not(a):
    return _t.logical_not(_t.as_tensor(a))


def signbit(x):
    return _t.signbit(x)


class _Linalg(_types.ModuleType):
    def __getattr__(self, name):
        return getattr(_t.linalg, name)

    @staticmethod
    def diagonal(x, offset=0):
        return _t.diagonal(x, offset=offset, dim1=-2, dim2=-1)

    @staticmethod
    def matrix_transpose(x):
        return x.transpose(-1, -2)

    @staticmethod
    def vector_norm(x, axis=None, keepdims=False, ord=2):
        return _t.linalg.vector_norm(x, ord=ord, dim=axis, keepdim=keepdims)

    @staticmethod
    def matrix_norm(x, keepdims=False, ord='fro'):
        return _t.linalg.matrix_norm(x, ord=ord, keepdim=keepdims)

    @staticmethod
    def svdvals(x):
        return _t.linalg.svdvals(x)


class _Fft(_types.ModuleType):
    def __getattr__(self, name):
        return getattr(_t.fft, name)

    @staticmethod
    def fft(x, n=None, axis=-1, norm='backward'):
        return _t.fft.fft(x, n=n, dim=axis, norm=norm)

    @staticmethod
    def ifft(x, n=None, axis=-1, norm='backward'):
        return _t.fft.ifft(x, n=n, dim=axis, norm=norm)


linalg = _Linalg('array_api_compat.torch.linalg')
fft = _Fft('array_api_compat.torch.fft')


def __getattr__(name):
    return getattr(_t, name)


_sys.modules[__name__ + '.linalg'] = linalg
_sys.modules[__name__ + '.fft'] = fft
