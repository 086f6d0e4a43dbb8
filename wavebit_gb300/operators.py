"""Explicit convolution operators on the GB300 path (rcwa/operators.py:70-140 of the reference).

``assemble`` builds the Li-rule convolution matrices of a problem's layers on the device without
solving scattering; ``solve`` solves with them. The arrays are torch tensors and may be replaced
(same shapes) to study alternative factorizations, as with the reference's ``operators``.

Conventions follow the reference's public operators: one ``ConvMatrices`` per wavelength with
the five slots ``(epx, epy, epz_i, epxy, epyx)``, each ``(n_layers, N, N)`` in the solver's layer
order (entry face first), about the cell centre (``D C D`` of the kernels' corner-frame matrices,
``D = diag((-1)^(m+n))``, conventions.py:1263-1292). Li's rules do not couple x and y, so
``epxy`` and ``epyx`` are ``None``; ``mu`` is ``None`` (non-magnetic) for every wavelength.
"""
from dataclasses import dataclass, field
from types import MappingProxyType
from typing import NamedTuple

import numpy as np
import torch

from . import engine
from . import rcwa as _rcwa

__all__ = ['ConvMatrices', 'Operators', 'Port', 'ScatteringMatrix', 'assemble', 'solve']

# the scattering-matrix types, which the reference's operators module re-exports (operators.py:14-21)
Port = _rcwa.Port
ScatteringMatrix = _rcwa.ScatteringMatrix


class ConvMatrices(NamedTuple):
    """The five convolution slots of a layer stack (factorization.py:136-162 of the reference)."""
    epx: object
    epy: object
    epz_i: object
    epxy: object = None
    epyx: object = None


@dataclass(frozen=True)
class Operators:
    """One epsilon/mu pair per wavelength; holds no solved fields or scattering matrix."""
    epsilon: tuple
    mu: tuple
    wavelengths: tuple
    numerics: object
    execution: object
    metadata: object = field(default_factory=dict)
    _prepared: object = field(default=None, repr=False)
    _physical_contract: object = field(default=None, repr=False)

    def __post_init__(self):
        object.__setattr__(self, 'epsilon', tuple(self.epsilon))
        object.__setattr__(self, 'mu', tuple(self.mu))
        object.__setattr__(self, 'metadata', MappingProxyType(dict(self.metadata)))


def _frame_signs(hu, hv, device):
    """``(-1)^(m+n)`` over the flattened orders ``i = n*n_u + m``."""
    m = np.arange(-hu, hu + 1)[None, :] + np.arange(-hv, hv + 1)[:, None]
    return torch.as_tensor(np.where(m.reshape(-1) % 2 == 0, 1.0, -1.0), dtype=torch.complex128, device=device)


def _swap_frame(slot, hu, hv):
    """Corner frame <-> centre frame of a stack of (N, N) slots (an involution)."""
    d = _frame_signs(hu, hv, slot.device)
    return d[None, :, None] * slot * d[None, None, :]


def _contract(problem, numerics):
    """The physical inputs the operators were built for: rasters, thicknesses, period, half
    spaces, wavelengths and the order window."""
    r = _rcwa._resolve(problem, numerics)
    rasters, thick, top, bot = r['rasters'], r['thickness'], r['eps_top'], r['eps_bot']
    if _lit_below(r):                      # the scene's own order and half-spaces, whichever side is lit
        rasters, thick, top, bot = rasters[::-1], thick[::-1], bot, top
    return (tuple((e.shape, e.tobytes()) for e in rasters), np.ascontiguousarray(thick).tobytes(), r['period'],
            complex(top), complex(bot), r['wavelengths'].tobytes(), r['orders'])


def _lit_below(r):
    """Lit from below, the resolved layers are the z-mirrored scene's (entry face first); the
    operators keep the scene's own top-first order either way."""
    return r.get('side', 'top') == 'bottom'


def assemble(problem, *, numerics=None, backend='gb300', device='cuda', precision='double'):
    """Build the operators of a concrete problem without solving (operators.py:71-104)."""
    prepared = _rcwa.prepare(problem, numerics=numerics, backend=backend, device=device, precision=precision)
    r = prepared.resolved
    hu, hv = r['orders']
    conv = prepared.conv
    cm = ConvMatrices(*(_swap_frame(conv.slot(k), hu, hv) for k in range(3)))
    if _lit_below(r):
        cm = ConvMatrices(*(a.flip(0) for a in cm[:3]), None, None)
    n_wl = len(r['wavelengths'])
    return Operators(epsilon=(cm,) * n_wl, mu=(None,) * n_wl, wavelengths=tuple(float(w) for w in r['wavelengths']),
                     numerics=numerics, execution={'backend': backend, 'device': device, 'precision': precision},
                     metadata={'fourier_origin': 'cell center (0,0)',
                               'slot_order': ('xx', 'yy', 'inverse_zz', 'xy', 'yx'),
                               'layer_order': 'top layer first',
                               'physical_contract': 'stack and vacuum wavelengths fixed; replace arrays '
                                                    'explicitly for a different constitutive operator'},
                     _prepared=prepared, _physical_contract=_contract(problem, numerics))


def solve(problem, operators):
    """Solve with explicit operators, without rebuilding them (operators.py:107-140)."""
    if not isinstance(operators, Operators) or operators._prepared is None:
        raise _rcwa.ValidationError('Supply Operators returned by assemble (optionally with replaced arrays).',
                                    code='operators.type', path='operators')
    if _contract(problem, operators.numerics) != operators._physical_contract:
        raise _rcwa.IncompatibleProblemError('The physical stack or wavelength differs from the assembled '
                                             'operator contract. Assemble it again.',
                                             code='operators.physical_contract', path='problem')
    prepared = operators._prepared
    r = _rcwa._resolve(problem, operators.numerics)
    n_wl, L = len(r['wavelengths']), len(r['rasters'])
    if len(operators.epsilon) != n_wl or len(operators.mu) != n_wl:
        raise _rcwa.ValidationError('One operator tuple is required per wavelength.',
                                    code='operators.spectral_shape', path='operators')
    if any(m is not None for m in operators.mu):
        raise _rcwa.UnsupportedFeatureError('magnetic operators are outside the GB300 raster path',
                                            path='operators.mu')
    hu, hv = r['orders']
    N = engine.n_orders(hu, hv)
    # one stack of corner-frame slots per distinct ConvMatrices object, shared by its wavelengths
    stacks, which = [], {}
    layer_index = np.zeros((n_wl, L), dtype=np.int32)
    for w, cm in enumerate(operators.epsilon):
        cm = ConvMatrices(*cm)
        if cm.epxy is not None or cm.epyx is not None:
            raise _rcwa.UnsupportedFeatureError('coupled x/y operators are outside the Li-rule raster path',
                                                path=f'operators.epsilon[{w}]')
        key = id(operators.epsilon[w])
        if key not in which:
            slots = []
            for k, a in enumerate(cm[:3]):
                t = torch.as_tensor(a, dtype=torch.complex128, device=prepared.conv.buf.device)
                if tuple(t.shape) != (L, N, N):
                    raise _rcwa.ValidationError(f'slot {k} must be ({L}, {N}, {N})', code='operators.shape',
                                                path=f'operators.epsilon[{w}]')
                slots.append(_swap_frame(t, hu, hv))
            which[key] = len(stacks)
            stacks.append(engine.ConvStack.from_matrices(*slots, hu, hv))
        layer_index[w] = which[key] * L + (np.arange(L)[::-1] if _lit_below(r) else np.arange(L))
    conv = stacks[0] if len(stacks) == 1 else engine.ConvStack(torch.cat([c.buf for c in stacks]), hu, hv)
    res = prepared._solve(r, conv, layer_index, amplitudes=True, scattering=_rcwa._wants_scattering(problem),
                          fields=_rcwa._wants_fields(problem))
    res.diagnostics['explicit_operators'] = True
    return res
