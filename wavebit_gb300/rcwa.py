"""The ``rcwa.check -> prepare -> run`` lifecycle of the reference, as a GB300 backend.

Mirrors ``wavebit.rcwa`` (rcwa/_lifecycle.py:422 ``check``, :737 ``prepare``, :698
``Prepared.run``, :801 ``run``) for raster stacks under Li's fixed nesting, with sampled or
integrated coefficients, the SMM or (as a cross-check) the ETM connecting algorithm, and the
optional outputs ``scattering`` and ``fields``. It accepts the reference's own declaration
objects (``wavebit.rcwa.Problem`` and friends) unchanged, by their attributes, or the small
mirror dataclasses defined here when the reference is not installed. Results come back as torch
tensors on the device with the reference's ``(wavelength, order_v, order_u)`` axes.

Stages A, B and C run in libwbgpu.so; the field amplitudes and the ETM recursion run as torch
linear algebra on the same device, over the library's modes. There is no CPU path.
"""
from dataclasses import dataclass, field
import math
import warnings
from typing import NamedTuple

import numpy as np
import torch

from . import _lib, engine

# ------------------------------------------------------------------------------- errors


@dataclass(frozen=True)
class Issue:
    """One structured finding (errors.py:9-15 of the reference)."""
    code: str
    path: str
    message: str
    expected: object = None
    actual: object = None
    severity: str = 'error'


class WavebitError(Exception):
    """Base error with a machine-readable ``code`` and its ``Issue`` (errors.py:18-66 of the
    reference)."""
    default_code = 'input.invalid'

    def __init__(self, message, *, code=None, path=None):
        self.code = code or self.default_code
        self.path = path
        self.message = message
        self.issue = Issue(code=self.code, path=path or 'problem', message=message)
        super().__init__(f'{path}: {message}' if path else message)


class ValidationError(WavebitError, ValueError):
    default_code = 'input.invalid'


class UnsupportedFeatureError(ValidationError):
    default_code = 'feature.unsupported'


class IncompatibleProblemError(ValidationError):
    """A live problem violates a prepared calculation's reuse contract (errors.py:56-58)."""
    default_code = 'problem.incompatible'


class NumericalError(WavebitError):
    default_code = 'numerical.failure'


class RayleighPointWarning(UserWarning):
    """A layer eigenmode sits numerically on its light line (backend.py:1151 of the reference)."""


class AutoDetuneWarning(UserWarning):
    """The auto-detune ladder moved a wavelength or angle (backend.py:1253 of the reference)."""


# relative step of an auto-detune retry (engine.py:141-147 of the reference)
_AUTO_DETUNE_REL = 1e-12

# ------------------------------------------------------------- declarations (mirror)


#: metres in one length unit (units.py:10)
_LENGTH_METRES = {'m': 1.0, 'mm': 1e-3, 'um': 1e-6, 'nm': 1e-9}


@dataclass(frozen=True)
class Units:
    """The length unit of every length in the problem (units.py:10-26): ``'m'``, ``'mm'``,
    ``'um'`` or ``'nm'``."""
    length: str = 'm'

    def __post_init__(self):
        if not isinstance(self.length, str) or self.length not in _LENGTH_METRES:
            raise ValidationError("length must be 'm', 'mm', 'um', or 'nm'", code='units.length', path='units.length')

    @property
    def length_unit_meters(self):
        return _LENGTH_METRES[self.length]


@dataclass(frozen=True)
class Material:
    epsilon: object = 1.0
    mu: object = None


@dataclass(frozen=True)
class Layer:
    """A raster layer: ``epsilon`` is a ``(ny, nx)`` permittivity raster (rows along v) or a
    scalar for a uniform layer."""
    thickness: object
    epsilon: object = None
    background: object = None
    regions: tuple = ()
    mu: object = None


@dataclass(frozen=True)
class Stack:
    """Bottom-to-top layers between two half spaces (problem.py:414)."""
    layers: tuple = ()
    top: object = field(default_factory=lambda: Material(1.0))
    bottom: object = field(default_factory=lambda: Material(1.0))
    period: object = (1.0, 1.0)
    lattice: object = None


@dataclass(frozen=True)
class PlaneWave:
    side: str = 'top'
    polarization: object = 's'
    amplitude: object = 1.0
    theta: object = None
    phi: object = None
    kx: object = None
    ky: object = None


@dataclass(frozen=True)
class Excitation:
    wavelength: object
    sources: tuple


@dataclass(frozen=True)
class Outputs:
    """What a run keeps beyond R and T (the reference's ``rcwa.Outputs``): ``scattering`` keeps
    the stack's scattering matrix of every wavelength (``Result.scattering``), ``fields`` the
    layers' mode amplitudes that ``Result.field`` samples."""
    fields: bool = False
    scattering: bool = False


@dataclass(frozen=True)
class Problem:
    stack: Stack
    excitation: Excitation
    units: Units = field(default_factory=Units)
    outputs: Outputs = field(default_factory=Outputs)


class Port(NamedTuple):
    """The basis one end of a :class:`ScatteringMatrix` counts (scattering.py:379-425 of the
    reference): the retained orders' in-plane wavevectors over k0 (one per order, ``i = n*n_u +
    m``), the half-space the port opens into, and the channel (``'sp'``: N s amplitudes over N p
    port variables)."""
    kx_over_k0: object
    ky_over_k0: object
    refractive_index: object
    mu: object
    channel: str


def _port_disagreement(a, b, tol=1e-12):
    """Why ports ``a`` and ``b`` are not the same basis, or ``None`` (scattering.py:655-700)."""
    if a.channel != b.channel:
        return f'they count different polarizations: {a.channel!r} against {b.channel!r}'

    def differ(x, y):
        if (x is None) != (y is None):
            return True
        if x is None:
            return False
        xa, ya = np.asarray(x), np.asarray(y)
        return xa.shape != ya.shape or bool(np.max(np.abs(xa - ya)) > tol)

    if differ(a.kx_over_k0, b.kx_over_k0) or differ(a.ky_over_k0, b.ky_over_k0):
        return ('their retained orders are different in-plane wavevectors; for lossless media choose '
                'theta_b = arcsin(sin(theta_a) * n_a / n_b) so that both pieces share k_par')
    if differ(a.refractive_index, b.refractive_index) or differ(a.mu, b.mu):
        return 'they open into different half-spaces; both pieces have to name the same joint medium'
    return None


def redheffer_star(S_a, S_b):
    """``S_a * S_b`` of two block 4-tuples (scattering.py:191-200 of the reference)."""
    a11, a12, a21, a22 = S_a
    b11, b12, b21, b22 = S_b
    I = torch.eye(a11.shape[-1], dtype=a11.dtype, device=a11.device)
    D_i = torch.linalg.inv(I - b11 @ a22)
    F_i = torch.linalg.inv(I - a22 @ b11)
    return (a11 + a12 @ D_i @ b11 @ a21, a12 @ D_i @ b12, b21 @ F_i @ a21, b22 + b21 @ F_i @ a22 @ b12)


class ScatteringMatrix(NamedTuple):
    """The stack's scattering matrix at its two half-space ports (scattering.py:482-605 of the
    reference), torch tensors of side 2N: rows and columns are the N s amplitudes followed by the
    N p port variables (the p wave's magnetic field, so ``S11`` of a unit p column is ``-r_p``),
    every order referenced at the cell centre. ``S11`` reflects back into the incidence medium,
    ``S21`` transmits into the far half-space, ``S12`` / ``S22`` are the same for light arriving
    from the far side."""
    S11: object
    S12: object
    S21: object
    S22: object
    entry_port: Port
    exit_port: Port

    @property
    def blocks(self):
        return (self.S11, self.S12, self.S21, self.S22)

    def cascade(self, beyond):
        """This stack followed by ``beyond`` (the piece the light reaches next), refused when the
        two ports where they meet are not the same basis (scattering.py:552-604)."""
        if not isinstance(beyond, ScatteringMatrix):
            raise TypeError(f'cascade() takes a ScatteringMatrix, got {type(beyond).__name__}')
        why = _port_disagreement(self.exit_port, beyond.entry_port)
        if why is not None:
            raise ValueError(f'cascade() cannot join these two: {why}')
        return ScatteringMatrix(*redheffer_star(self.blocks, beyond.blocks), entry_port=self.entry_port,
                                exit_port=beyond.exit_port)


@dataclass(frozen=True)
class Numerics:
    orders: tuple = (0, 0)
    algorithm: str = 'smm'
    fourier_coefficients: object = None
    factorization: object = None
    li_nesting: object = None
    detuning: object = None
    exceptional_points: str = 'rebuild'
    formulation: str = 'auto'
    half_space_merge_tolerance: float = 0.0

# ------------------------------------------------------------------------ resolution


def _scalar_eps(material, path):
    if material is None:
        return 1.0 + 0j
    if getattr(material, 'mu', None) not in (None, 1, 1.0):
        raise UnsupportedFeatureError('magnetic half-spaces are outside the GB300 raster path',
                                      code='feature.unsupported', path=path)
    eps = getattr(material, 'epsilon', material)
    if callable(eps):
        raise UnsupportedFeatureError('dispersive materials are outside the GB300 raster path',
                                      path=path)
    return complex(np.asarray(eps).reshape(()))


def _numerics_orders(numerics):
    orders = tuple(int(v) for v in getattr(numerics, 'orders', (0, 0)))
    if len(orders) != 2 or min(orders) < 0:
        raise ValidationError('orders must be a pair of nonnegative integers', path='numerics.orders')
    if _lib.load().wb_workspace_bytes(orders[0], orders[1], 1, 1, 0) == 0:
        raise ValidationError(f'orders {orders} exceed the windows the GB300 kernels hold on chip: '
                              '0 <= hv <= 42 and (2hu+1)(2hv+1) <= 3228', path='numerics.orders')
    for name, allowed in (('algorithm', (None, 'smm', 'etm')), ('fourier_coefficients', (None, 'sampled', 'integrated')),
                          ('factorization', (None, 'li')), ('li_nesting', (None, 'fixed'))):
        val = getattr(numerics, name, None)
        val = getattr(val, 'value', val)                # the reference's enums carry the name
        if isinstance(val, str):
            val = val.lower()
        if val not in allowed:
            raise UnsupportedFeatureError(
                f'numerics.{name}={val!r}: the GB300 path implements {", ".join(map(repr, allowed[1:]))} only',
                path=f'numerics.{name}')
    # the layer operator here is the second-order one (Omega^2, solve_2d.py:2377-2418), and a
    # tolerance that snaps nearly equal media into a half-space changes the problem
    form = getattr(getattr(numerics, 'formulation', 'auto'), 'value', getattr(numerics, 'formulation', 'auto'))
    if form not in (None, 'auto', 'second_order'):
        raise UnsupportedFeatureError(f'numerics.formulation={form!r}: the GB300 path solves the second-order '
                                      "layer operator ('auto' or 'second_order')", path='numerics.formulation')
    tol = getattr(numerics, 'half_space_merge_tolerance', 0.0)
    if tol not in (None, 0, 0.0):
        raise UnsupportedFeatureError('numerics.half_space_merge_tolerance: the GB300 path solves the stack as '
                                      'declared (tolerance 0)', path='numerics.half_space_merge_tolerance')
    det = getattr(numerics, 'detuning', None)
    if det is not None and (type(det) not in (float, int) or not math.isfinite(det) or det <= 0):
        raise ValidationError('detuning is None (exact requested problem) or a positive relative step.',
                              code='numerics.detuning', path='numerics.detuning')
    return orders


def _wants_scattering(problem):
    return bool(getattr(getattr(problem, 'outputs', None), 'scattering', False))


def _wants_fields(problem):
    return bool(getattr(getattr(problem, 'outputs', None), 'fields', False))


def _algorithm(numerics):
    """``'smm'`` or ``'etm'`` (the connecting algorithm of ``Numerics``)."""
    val = getattr(numerics, 'algorithm', None)
    val = getattr(val, 'value', val)
    return 'etm' if isinstance(val, str) and val.lower() == 'etm' else 'smm'


def _integrated(numerics):
    """Whether the Li slots take integrated (closed-form segment) coefficients."""
    val = getattr(numerics, 'fourier_coefficients', None)
    val = getattr(val, 'value', val)
    return isinstance(val, str) and val.lower() == 'integrated'


def _resolve(problem, numerics):
    """Problem -> flat arrays in kernel order (entry layer first)."""
    length = getattr(getattr(problem, 'units', None), 'length', 'm')
    if not isinstance(length, str) or length not in _LENGTH_METRES:
        raise ValidationError("length must be 'm', 'mm', 'um', or 'nm'", code='units.length', path='units.length')
    stack = problem.stack
    if getattr(stack, 'lattice', None) is not None:
        raise UnsupportedFeatureError('oblique lattices are outside the GB300 raster path',
                                      path='stack.lattice')
    period = tuple(float(p) for p in stack.period)
    if len(period) == 1:
        period = (period[0], period[0])
    layers = tuple(stack.layers)
    rasters, thick = [], []
    for i, layer in enumerate(layers):
        if getattr(layer, 'regions', ()):
            raise UnsupportedFeatureError('region (shape) layers are outside the GB300 raster path',
                                          path=f'stack.layers[{i}]')
        if hasattr(layer, 'layers') or not hasattr(layer, 'epsilon'):
            # a profiled layer is sliced by height, its material may grade with height
            raise UnsupportedFeatureError('profiled (height-dependent) layers are outside the GB300 raster path',
                                          path=f'stack.layers[{i}]')
        if getattr(layer, 'mu', None) is not None:
            raise UnsupportedFeatureError('magnetic layers are outside the GB300 raster path',
                                          path=f'stack.layers[{i}].mu')
        eps = layer.epsilon
        if eps is None:
            eps = _scalar_eps(layer.background, f'stack.layers[{i}].background')
        eps = np.asarray(eps.detach().cpu().numpy() if hasattr(eps, 'detach') else eps, dtype=np.complex128)
        if eps.ndim == 0:
            eps = eps.reshape(1, 1)
        if eps.ndim == 1:
            eps = eps.reshape(1, -1)
        if eps.ndim != 2 or not np.all(np.isfinite(eps)):
            raise ValidationError('a layer raster must be a finite 2D array', path=f'stack.layers[{i}].epsilon')
        d = float(np.asarray(layer.thickness.detach().cpu() if hasattr(layer.thickness, 'detach') else layer.thickness))
        if not (d >= 0 and math.isfinite(d)):
            raise ValidationError('thickness must be finite and >= 0', path=f'stack.layers[{i}].thickness')
        rasters.append(eps)
        thick.append(d)
    # public order is bottom to top; kernels take the entry face (top) first
    rasters, thick = rasters[::-1], thick[::-1]
    eps_top = _scalar_eps(stack.top, 'stack.top')
    eps_bot = _scalar_eps(stack.bottom, 'stack.bottom')
    sources = tuple(problem.excitation.sources)
    side = getattr(sources[0], 'side', 'top') if len(sources) == 1 else 'top'
    if side not in ('top', 'bottom'):
        raise ValidationError("side must be 'top' or 'bottom'.", code='source.side', path='source.side')
    if side == 'bottom':
        # lit from below: exactly the z-mirrored scene lit from above (the reference's
        # incidence_side contract): the public bottom-first layers are the entry face first and the
        # half-spaces trade places; results are mapped back to the scene's frame afterwards
        rasters, thick = rasters[::-1], thick[::-1]
        eps_top, eps_bot = eps_bot, eps_top
    bare = not layers
    if bare:
        # the bare interface between the half-spaces, solved as the reference solves it: through
        # one zero-thickness layer of the top medium (results.py:180-189)
        rasters, thick = [np.full((1, 1), eps_top, dtype=np.complex128)], [0.0]
    if eps_top.imag != 0 or eps_top.real <= 0:
        raise UnsupportedFeatureError('the lit half-space must be lossless with Re(eps) > 0',
                                      path='stack.top' if side == 'top' else 'stack.bottom')
    exc = problem.excitation
    wl = np.atleast_1d(np.asarray(exc.wavelength, dtype=np.float64)).reshape(-1)
    if not (wl.size and np.all(np.isfinite(wl)) and np.all(wl > 0)):
        raise ValidationError('wavelengths must be finite and positive', path='excitation.wavelength')
    sources = tuple(exc.sources)
    if len(sources) != 1:
        raise UnsupportedFeatureError('one PlaneWave source per problem on the GB300 path',
                                      path='excitation.sources')
    src = sources[0]
    # a coherent order set, a beam or a dipole reads like a plane wave by its angle fields but is
    # another illumination; it is refused by what defines it, never solved as its central wave
    for marker, kind in (('weights', 'incident orders'), ('waist', 'a Gaussian beam'), ('moment', 'a dipole')):
        if hasattr(src, marker):
            raise UnsupportedFeatureError(f'{kind} as a source is outside the GB300 path (one plane wave per problem)',
                                          path='excitation.sources[0]')
    direct = getattr(src, 'kx', None) is not None or getattr(src, 'ky', None) is not None
    if direct:
        thetas, phi = _direct_incidence(src, wl, eps_top)
        theta = float(thetas[0])
    else:
        theta = float(np.real(0.0 if src.theta is None else src.theta))
        phi = float(np.real(0.0 if src.phi is None else src.phi))
        if not abs(theta) < math.pi / 2:
            raise ValidationError('theta must be a real angle below pi/2', path='excitation.sources[0].theta')
        if not math.isfinite(phi):
            raise ValidationError('phi must be a finite angle', path='excitation.sources[0].phi')
        thetas = np.full(wl.shape[0], theta)
    pol = src.polarization
    if isinstance(pol, str):
        if pol not in ('s', 'p'):
            raise ValidationError("polarization must be 's', 'p' or an (s, p) pair",
                                  path='excitation.sources[0].polarization')
        a_s, a_p = (complex(1.0, 0.0), complex(math.cos(math.pi / 2))) if pol == 's' else (0j, 1 + 0j)
    else:
        a_s, a_p = (complex(v) for v in pol)
        nrm = math.sqrt(abs(a_s) ** 2 + abs(a_p) ** 2)
        if not (nrm > 0 and math.isfinite(nrm)):
            raise ValidationError('an (s, p) polarization pair must be finite and not both zero',
                                  path='excitation.sources[0].polarization')
        a_s, a_p = a_s / nrm, a_p / nrm
    if _wants_scattering(problem) and _algorithm(numerics) == 'etm':
        raise UnsupportedFeatureError('Scattering matrices require algorithm="smm".',
                                      code='rcwa.scattering_algorithm', path='outputs.scattering')
    amplitude = complex(np.asarray(getattr(src, 'amplitude', 1.0)).reshape(()))
    if not np.isfinite(amplitude):
        raise ValidationError('the source amplitude must be finite', path='excitation.sources[0].amplitude')
    orders = _numerics_orders(_numerics_or_default(numerics))
    return dict(rasters=rasters, thickness=np.array(thick), period=period, eps_top=eps_top,
                eps_bot=eps_bot, wavelengths=wl, theta=theta, thetas=thetas, phi=phi, pol=(a_s, a_p), orders=orders,
                amplitude=amplitude, bare_interface=bare, length=length, side=side)


def _direct_incidence(src, wl, eps_inc):
    """``PlaneWave(kx=, ky=)``: physical wavenumbers (rad per length unit), taken as given at every
    wavelength (engine.py:2750-2758): ``k_par / k0 = (kx, ky) * wavelength / (2 pi)``. The
    kernels take that wavevector as the polar angle in the lit medium of index ``n`` and the
    azimuth, ``sin(theta) = |k_par| / (k0 n)`` (one angle per wavelength) and
    ``phi = atan2(ky, kx)`` (0 at normal incidence, where the s/p frame takes ``phi = 0``, as
    the reference's frame azimuth does for a direct wavevector)."""
    if getattr(src, 'theta', None) is not None or getattr(src, 'phi', None) is not None:
        raise ValidationError('Use theta/phi or kx/ky, not both.', code='source.direction_ambiguous', path='source')
    k = []
    for name in ('kx', 'ky'):
        v = getattr(src, name, None)
        v = 0.0 if v is None else complex(np.asarray(v).reshape(()))
        if not (np.isfinite(v) and v.imag == 0):
            raise ValidationError(f'{name} must be a finite real wavenumber', path=f'excitation.sources[0].{name}')
        k.append(v.real)
    kpar = math.hypot(*k) * wl / (2 * math.pi)
    n = math.sqrt(eps_inc.real)
    if np.any(kpar >= n):
        raise UnsupportedFeatureError('an incident wavevector at or past the lit medium\'s light line (evanescent '
                                      'incidence) is outside the GB300 raster path', path='excitation.sources[0]')
    return np.arcsin(kpar / n), (math.atan2(k[1], k[0]) if k[0] or k[1] else 0.0)


def _numerics_or_default(numerics):
    return Numerics() if numerics is None else numerics

# -------------------------------------------------------------------------- lifecycle


@dataclass
class CheckReport:
    issues: tuple = ()
    estimates: dict = field(default_factory=dict)
    resolved: dict = field(default_factory=dict)


def _issue(error, path='problem'):
    """The Issue a refusal reports (_lifecycle.py:63-69 of the reference)."""
    if isinstance(error, WavebitError):
        return error.issue
    if isinstance(error, NotImplementedError):
        return UnsupportedFeatureError(str(error), code='rcwa.unsupported', path=path).issue
    return ValidationError(str(error), code='rcwa.invalid', path=path).issue


def check(problem, *, numerics=None, backend='gb300', device='cuda', precision='double'):
    """Admission without a solve (_lifecycle.py:422-457): the report keys plus GB300 estimates, or
    -- as in the reference -- a report whose ``issues`` hold the refusal instead of raising it."""
    try:
        return _check(problem, numerics, backend, device, precision)
    except (ValidationError, TypeError, ValueError, NotImplementedError) as error:
        return CheckReport(issues=(_issue(error),))


def _check(problem, numerics, backend, device, precision):
    r = _resolve(problem, numerics)
    hu, hv = r['orders']
    N = engine.n_orders(hu, hv)
    L = len(r['rasters'])
    chunk = max(1, min(len(r['wavelengths']), 128))
    ws = int(_lib.load().wb_workspace_bytes(hu, hv, L, chunk, _lib.PRECISION.get(precision, 0)))
    n_wl = len(r['wavelengths'])
    est = {'retained_spatial_modes': N,
           'one_dense_material_matrix_bytes': 16 * N * N,
           'one_first_order_matrix_bytes': 16 * (2 * N) ** 2,
           # what Outputs keeps resident on the device after the run
           'retained_field_bytes': 16 * n_wl * L * (2 * (2 * N) ** 2 + 4 * N) if _wants_fields(problem) else 0,
           'retained_scattering_bytes': 16 * n_wl * 4 * (2 * N) ** 2 if _wants_scattering(problem) else 0,
           'device_workspace_bytes': ws,
           'device_chunk': chunk}
    if torch.cuda.is_available():
        free, total = torch.cuda.mem_get_info()
        est['device_free_bytes'] = int(free)
        est['admissible'] = ws <= free
    resolved = {'order_window': ((0, hu), (0, hv)), 'wavelength_count': len(r['wavelengths']),
                'layer_count': L, 'fourier_coefficients': 'integrated' if _integrated(numerics) else 'sampled',
                'factorization': 'li',
                'algorithm': _algorithm(numerics), 'solve_path': '2d', 'backend': backend, 'device': device,
                'precision': precision, 'retained_fields': _wants_fields(problem),
                'retained_scattering': _wants_scattering(problem),
                'length_units': getattr(getattr(problem, 'units', None), 'length', None)}
    return CheckReport(issues=(), estimates=est, resolved=resolved)


def _incident_scaled(ratio, reference):
    field_ = (reference or {}).get('incident_field')
    return None if ratio is None or field_ is None else ratio * field_


class DiffractionOrder(NamedTuple):
    """One order of :class:`DiffractionOrders` (contracts.py:149-175): each array with the
    wavelength axis only (``k_parallel`` and ``amplitude_ratio_xyz`` with their trailing axis)."""
    wavelengths: tuple
    order_u: int
    order_v: int
    efficiency: object = None
    amplitude_ratio_s: object = None
    amplitude_ratio_p: object = None
    power: object = None
    amplitude_ratio_xyz: object = None
    k_parallel: object = None
    k_normal: object = None
    reference: dict = None
    metadata: dict = None

    field_s = property(lambda self: _incident_scaled(self.amplitude_ratio_s, self.reference))
    field_p = property(lambda self: _incident_scaled(self.amplitude_ratio_p, self.reference))
    field_xyz = property(lambda self: _incident_scaled(self.amplitude_ratio_xyz, self.reference))


class DiffractionOrders(NamedTuple):
    """One port's diffraction orders (results.py:373-392, contracts.py:288-345 of the reference),
    arrays ``(wavelength, order_v, order_u)``: ``efficiency``; the Fresnel amplitude ratios of each
    order's s and p waves and of its Cartesian E (``amplitude_ratio_xyz``, trailing xyz axis),
    referenced at the port's plane and the cell centre; ``power``, each order's outgoing power
    in W; ``k_parallel`` (trailing (kx, ky) axis) and ``k_normal``, the order's wavevector in
    rad per length unit, ``k_normal`` signed along z (negative for a wave leaving through the
    bottom). ``reference`` names the port, its plane, medium, cell measure and the incident
    normalisation with their units; ``metadata`` the run's flags. The amplitude-derived arrays
    are None when the run did not keep amplitudes."""
    wavelengths: tuple
    orders_u: object
    orders_v: object
    efficiency: object
    amplitude_ratio_s: object = None
    amplitude_ratio_p: object = None
    power: object = None
    amplitude_ratio_xyz: object = None
    k_parallel: object = None
    k_normal: object = None
    reference: dict = None
    metadata: dict = None

    field_s = property(lambda self: _incident_scaled(self.amplitude_ratio_s, self.reference))
    field_p = property(lambda self: _incident_scaled(self.amplitude_ratio_p, self.reference))
    field_xyz = property(lambda self: _incident_scaled(self.amplitude_ratio_xyz, self.reference))

    #: entries of ``reference`` / ``metadata`` that carry a wavelength axis (contracts.py:216-219)
    _PER_WAVELENGTH = ('plane', 'epsilon', 'mu', 'cell_measure', 'incident_power', 'power_defined',
                       'efficiency_defined')

    def at_wavelength_index(self, index):
        """These orders at the wavelength in position ``index``, as a length-1 wavelength axis
        (contracts.py:269-285): every array and every per-wavelength reference entry sliced."""
        i = int(index)
        if not 0 <= i < len(self.wavelengths):
            raise IndexError(i)
        cut = lambda a: None if a is None else a[i:i + 1]
        maps = []
        for mapping in (self.reference, self.metadata):
            m = dict(mapping or {})
            for key in self._PER_WAVELENGTH:
                v = m.get(key)
                if v is not None and not isinstance(v, str) and len(v) == len(self.wavelengths):
                    m[key] = v[i:i + 1]
            maps.append(m)
        return self._replace(wavelengths=tuple(self.wavelengths)[i:i + 1], efficiency=cut(self.efficiency),
                             amplitude_ratio_s=cut(self.amplitude_ratio_s), amplitude_ratio_p=cut(self.amplitude_ratio_p),
                             power=cut(self.power), amplitude_ratio_xyz=cut(self.amplitude_ratio_xyz),
                             k_parallel=cut(self.k_parallel), k_normal=cut(self.k_normal),
                             reference=maps[0], metadata=maps[1])

    def order(self, m, n=0):
        """Order ``(m, n)`` as one :class:`DiffractionOrder` (contracts.py:259-267); KeyError when
        the order is not retained."""
        labels_u, labels_v = [int(v) for v in self.orders_u], [int(v) for v in self.orders_v]
        if int(m) not in labels_u or int(n) not in labels_v:
            raise KeyError((m, n))
        i, j = labels_u.index(int(m)), labels_v.index(int(n))
        pick = lambda a: None if a is None else a[:, j, i]
        return DiffractionOrder(self.wavelengths, int(m), int(n), pick(self.efficiency), pick(self.amplitude_ratio_s),
                                pick(self.amplitude_ratio_p), pick(self.power), pick(self.amplitude_ratio_xyz),
                                pick(self.k_parallel), pick(self.k_normal), self.reference, self.metadata)


def _diffraction_orders(R, T, amplitudes, wavelengths, hu, hv, ports=None):
    """``outputs['reflected']`` and ``outputs['transmitted']`` of the given polarization. The
    kernels' amplitudes (B, 3, 4, N: column, (r_s, r_p, t_s, t_p), order) are about the cell
    corner; order (m, n) about the centre is ``(-1)^(m+n)`` times it. ``ports`` (the solves'
    effective wavelengths and angles, the media, the cell, the source and the length unit) adds
    the wavevectors, the Cartesian ratios and the powers (results.py:292-420)."""
    from . import fields as F
    ou, ov = np.arange(-hu, hu + 1), np.arange(-hv, hv + 1)
    nu, nv = 2 * hu + 1, 2 * hv + 1
    ratios = [None] * 4
    if amplitudes is not None:
        m = ou[None, :] + ov[:, None]
        sign = torch.as_tensor(np.where(m % 2 == 0, 1.0, -1.0), dtype=torch.complex128, device=amplitudes.device)
        B = amplitudes.shape[0]
        ratios = [amplitudes[:, 0, k].reshape(B, nv, nu) * sign for k in range(4)]
    if ports is None:
        return (DiffractionOrders(wavelengths, ou, ov, R, ratios[0], ratios[1]),
                DiffractionOrders(wavelengths, ou, ov, T, ratios[2], ratios[3]))
    p = ports
    dev = R.device
    wl = np.asarray(p['wavelengths'], dtype=np.float64)
    B = wl.shape[0]
    kx, ky, c, s, kzt, kzb = F.order_table(wl, p['thetas'], p['phi'], p['period'], p['eps_top'], p['eps_bot'],
                                           hu, hv, dev)
    k0 = torch.as_tensor(2 * math.pi / wl, device=dev)[:, None]
    k_par = (torch.stack([kx, ky], -1) * k0[..., None]).to(torch.complex128).reshape(B, nv, nu, 2)
    area = abs(p['period'][0] * p['period'][1]) * _LENGTH_METRES[p['length']] ** 2
    amp = complex(p['amplitude'])
    xyz, power, incident = [None, None], [None, None], None
    if amplitudes is not None:
        flat = [r.reshape(B, -1) for r in ratios]
        n_top, n_bot = np.sqrt(complex(p['eps_top'])), np.sqrt(complex(p['eps_bot']))
        inc, refl, trn = F.order_waves(kx, ky, c, s, kzt, kzb, n_top, n_bot, flat, p['pol'])
        xyz = [w[..., :3].reshape(B, nv, nu, 3) for w in (refl, trn)]
        power = [F.wave_power(w, sg, area, amp).reshape(B, nv, nu) for w, sg in ((refl, 1.0), (trn, -1.0))]
        incident = F.wave_power(inc, -1.0, area, amp).sum(-1)
    defined = torch.ones(B, dtype=torch.bool, device=dev)
    metadata = {'power_defined': defined, 'efficiency_defined': defined, 'propagation': 'continuum',
                'polarization_frame': "each order's outgoing s/p frame", 'time_convention': 'exp(-i*omega*t)'}
    # lit from below, the solve ran on the z-mirrored scene: its reflected wave leaves through
    # the scene's bottom, its transmitted one through the top, and E_z changes sign
    lit, far = ('bottom', 'top') if p.get('side', 'top') == 'bottom' else ('top', 'bottom')
    if lit == 'bottom' and xyz[0] is not None:
        flip = torch.as_tensor([1.0, 1.0, -1.0], dtype=torch.complex128, device=dev)
        xyz = [a * flip for a in xyz]
    planes, normals = {'top': float(p['top_plane']), 'bottom': 0.0}, {'top': 1.0, 'bottom': -1.0}
    out = []
    for k, (wave, port, kz, eps) in enumerate((('reflected', lit, kzt, p['eps_top']),
                                               ('transmitted', far, kzb, p['eps_bot']))):
        sign, plane = normals[port], planes[port]
        reference = {'port': port, 'wave': wave, 'plane': (plane,) * B, 'length_units': p['length'],
                     'lateral_origin': (0.0, 0.0), 'outward_normal': (0.0, 0.0, sign), 'incident_port': lit,
                     'incident_field': amp, 'incident_field_units': 'V/m', 'incident_power': incident,
                     'incident_power_units': 'W', 'cell_measure': (area,) * B, 'cell_measure_units': 'm^2',
                     'invariant_axes': (), 'epsilon': (complex(eps),) * B, 'mu': (1.0,) * B,
                     'amplitude_ratio_units': '1', 'power_units': 'W', 'wavevector_units': 'rad/' + p['length']}
        out.append(DiffractionOrders(tuple(float(v) for v in wl), ou, ov, R if k == 0 else T, ratios[2 * k],
                                     ratios[2 * k + 1], power[k], xyz[k], k_par,
                                     (sign * k0 * kz).reshape(B, nv, nu), reference, metadata))
    return tuple(out)


class Result:
    """R and T with the reference's ``(wavelength, order_v, order_u)`` axes, on the device.

    ``outputs`` holds the reference's ``'reflected'`` / ``'transmitted'`` diffraction orders of
    the given polarization, and the per-polarization efficiencies of the three incidence columns
    (``'incident'``, ``'s_inc'``, ``'p_inc'``)."""

    def __init__(self, R, T, R_sp, T_sp, status, wavelengths, diagnostics, amplitudes=None, scattering=None,
                 field_states=None, field_geometry=None, orders=None, ports=None, provenance=None):
        self.R, self.T = R, T
        self.outputs = {'incident': {'R': R, 'T': T},
                        's_inc': {'R': R_sp[0], 'T': T_sp[0]},
                        'p_inc': {'R': R_sp[1], 'T': T_sp[1]}}
        if orders is not None:
            self.outputs['reflected'], self.outputs['transmitted'] = _diffraction_orders(
                R, T, amplitudes, wavelengths, *orders, ports=ports)
        if torch.is_tensor(R) and torch.is_tensor(T):
            # real in-plane wavevectors and a lossless superstrate: the net flux into the stack is
            # the incident one less the reflected orders' (results.py:375-380)
            sr, st_ = R.sum(dim=(-2, -1)), T.sum(dim=(-2, -1))
            self.outputs['power_entering'] = 1.0 - sr
            self.outputs['absorption'] = 1.0 - sr - st_
            finite = bool(torch.isfinite(R).all()) and bool(torch.isfinite(T).all())
        else:
            finite = None
        # finiteness is numerical validity, not a statement of convergence in the orders
        self.validity = {'checks': {'numerical_finite': finite},
                         'convergence': {'status': 'not assessed', 'requires': 'independent refinement study'}}
        self.status = status
        self.wavelengths = wavelengths
        self.diagnostics = diagnostics
        self.provenance = dict(provenance or {})
        self.amplitudes = amplitudes
        self._scattering = scattering
        self._field_states = field_states
        self._field_geometry = field_geometry

    def field(self, *, x, y, z, reconstruction='plain'):
        """Collocated complex phasors at explicit points or counts (results.py:148-229 of the
        reference): values ``(wavelength, z, y, x, 6)`` for ``(Ex, Ey, Ez, Hx, Hy, Hz)``, E in
        V/m and H in A/m; ``x``, ``y`` from the cell centre, ``z`` upward from the stack's bottom
        face (a face belongs to the layer above it). ``reconstruction`` is ``'plain'`` (the modes'
        Fourier sums) or ``'lalanne'`` (``E_x``, ``E_y`` of patterned layers from the displacement
        series line by line, field_result.py:610-650)."""
        from . import fields as F
        if not self._field_states:
            raise UnsupportedFeatureError('This result did not retain field reconstruction state. Request '
                                          'Outputs(fields=True).', code='outputs.unavailable', path='outputs.fields')
        if reconstruction in ('split', 'splitw'):
            raise UnsupportedFeatureError(f'reconstruction={reconstruction!r} is outside the GB300 raster path; '
                                          "use 'plain' or 'lalanne'", code='field.reconstruction',
                                          path='reconstruction')
        if reconstruction not in ('plain', 'lalanne'):
            raise ValidationError(f"reconstruction must be 'plain', 'lalanne', 'split' or 'splitw', not "
                                  f'{reconstruction!r}.', code='field.reconstruction', path='reconstruction')
        thickness, period, amplitude = self._field_geometry[:3]
        if len(self._field_geometry) > 3 and self._field_geometry[3]:
            raise ValidationError('This stack has no layers, so field() has nothing to sample: it reconstructs '
                                  'inside finite layers only, and here z = 0 is the interface between the two '
                                  'half-spaces. Add a layer to sample inside it.', code='field.coordinates', path='z')
        lit_below = self._lit_side() == 'bottom'
        try:
            xs = F.axis_points(x, period[0], 'x')
            ys = F.axis_points(y, period[1], 'y')
            # heights and face ownership in the scene's frame; lit from below the state is that
            # of the z-mirrored scene, whose layer p is the scene's (L-1-p), depth measured upward
            scene = thickness[::-1] if lit_below else thickness
            zs, owner, depth = F.height_points(z, scene)
        except ValueError as e:
            raise ValidationError(str(e), code='field.coordinates', path='x/y/z') from e
        if lit_below:
            depth = np.asarray(scene, dtype=np.float64)[owner] - depth
            owner = len(scene) - 1 - owner
        orders = self._field_geometry[4] if len(self._field_geometry) > 4 else None
        values = torch.stack([F.synthesize(st, owner, depth, xs, ys, amplitude, reconstruction, period, orders)
                              for st in self._field_states])
        if lit_below:
            values = values * F.z_mirror(values.device)
        return F.FieldSamples(coordinates={'x': xs, 'y': ys, 'z': zs, 'wavelength': self.wavelengths},
                              values=values, components=F.COMPONENTS, sampling='collocated Cartesian phasor',
                              metadata={'axis_order': ('wavelength', 'z', 'y', 'x', 'component'),
                                        'time_convention': 'exp(-i*omega*t)', 'reconstruction': reconstruction})

    def boundary_fields(self, *, side, x, y, part='total'):
        """Collocated phasors of the half-spaces' waves on the top or bottom face (results.py:231-265
        of the reference): ``part`` ``'incoming'``, ``'outgoing'`` or ``'total'``; values
        ``(wavelength, y, x, 6)``, E in V/m and H in A/m; ``x``, ``y`` from the cell centre."""
        from . import fields as F
        if not self._field_states:
            raise UnsupportedFeatureError('This result did not retain field reconstruction state. Request '
                                          'Outputs(fields=True).', code='outputs.unavailable', path='outputs.fields')
        for name, value, allowed in (('side', side, ('top', 'bottom')),
                                     ('part', part, ('incoming', 'outgoing', 'total'))):
            if not isinstance(value, str) or value not in allowed:
                raise ValidationError(f'{name} is one of {", ".join(map(repr, allowed))}; got {value!r}.',
                                      code=f'field.{name}', path=name)
        period, amplitude = self._field_geometry[1], self._field_geometry[2]
        try:
            xs = F.axis_points(x, period[0], 'x')
            ys = F.axis_points(y, period[1], 'y')
        except ValueError as e:
            raise ValidationError(str(e), code='field.coordinates', path='x/y') from e
        lit_below = self._lit_side() == 'bottom'
        face = {'top': 'bottom', 'bottom': 'top'}[side] if lit_below else side
        values = torch.stack([F.expand_boundary(st, face, part, xs, ys, amplitude) for st in self._field_states])
        if lit_below:
            values = values * F.z_mirror(values.device)
        return F.FieldSamples(coordinates={'x': xs, 'y': ys, 'wavelength': self.wavelengths}, values=values,
                              components=F.COMPONENTS, sampling='collocated boundary phasor',
                              metadata={'side': side, 'part': part, 'axis_order': ('wavelength', 'y', 'x', 'component')})

    @property
    def scattering(self):
        """One :class:`ScatteringMatrix` per wavelength (results.py:137-141 of the reference)."""
        if self._scattering is None:
            raise UnsupportedFeatureError('Request Outputs(scattering=True) with the SMM algorithm before running.',
                                          code='outputs.unavailable', path='outputs.scattering')
        return self._scattering

    @property
    def absorption(self):
        return 1.0 - self.R.sum(dim=(-2, -1)) - self.T.sum(dim=(-2, -1))

    def _lit_side(self):
        g = self._field_geometry
        return g[5] if g is not None and len(g) > 5 else 'top'

    @property
    def reflection(self):
        """``outputs['reflected']`` (results.py:128-130)."""
        return self.outputs['reflected']

    @property
    def transmission(self):
        """``outputs['transmitted']`` (results.py:132-134)."""
        return self.outputs['transmitted']


class Prepared:
    """Stage A done once and kept on the device (_lifecycle.py:698-733 ``Prepared.run``)."""

    def __init__(self, problem, numerics, precision, handle):
        self.problem = problem
        self.numerics = numerics
        self.precision = precision
        self.handle = handle
        r = _resolve(problem, numerics)
        self.resolved = r
        hu, hv = r['orders']
        self.integrated = _integrated(numerics)
        self.conv = _assemble_layers(r['rasters'], hu, hv, handle, self.integrated)

    @staticmethod
    def _layout(problem, r):
        """What a preparation fixes (_adapt.py:633-640 of the reference): the layer count and
        raster shapes, the number of wavelengths and sources, and the requested outputs; the
        values in them stay live. Shapes are read in the scene's own layer order, whichever side
        the source lights."""
        rasters = r['rasters'][::-1] if r.get('side', 'top') == 'bottom' else r['rasters']
        return ((len(rasters), tuple(e.shape for e in rasters)),
                (len(r['wavelengths']), len(tuple(problem.excitation.sources))),
                (_wants_fields(problem), _wants_scattering(problem)))

    def validate(self, problem):
        """Whether a concrete problem can reuse this preparation (_lifecycle.py:678-698 of the
        reference): its check report, or a report whose ``issues`` say why not."""
        try:
            r = _resolve(problem, self.numerics)
            self._check_layout(problem, r)
        except (ValidationError, TypeError, ValueError, NotImplementedError) as error:
            return CheckReport(issues=(_issue(error),))
        return check(problem, numerics=self.numerics, precision=self.precision)

    def _check_layout(self, problem, r):
        old = self._layout(self.problem, self.resolved)
        new = self._layout(problem, r)
        if new != old:
            path = ('stack.layers' if new[0] != old[0] else 'excitation' if new[1] != old[1] else 'outputs')
            raise IncompatibleProblemError('The problem declaration layout changed. Prepare it again (layer/source '
                                           'counts, raster shapes, outputs and spectral shape are structural).',
                                           code='prepared.structure', path=path)

    def run(self, problem=None, *, amplitudes=True):
        """Solve ``problem`` (or the prepared one) on the kept convolution matrices
        (_lifecycle.py:698-733). ``amplitudes`` keeps the kernels' Fresnel amplitudes, which the
        amplitude ratios, Cartesian ratios and per-order powers of ``outputs['reflected']`` and
        ``outputs['transmitted']`` read; the reference always answers them (``answers='amplitude'``)."""
        r = self.resolved if problem is None else _resolve(problem, self.numerics)
        if problem is not None:
            self._check_layout(problem, r)
        conv = self.conv
        if problem is not None and not _same_rasters(r['rasters'], self.resolved['rasters']):
            conv = _assemble_layers(r['rasters'], *r['orders'], self.handle, self.integrated)
        L = len(r['rasters'])
        asked = self.problem if problem is None else problem
        layer_index = np.tile(np.arange(L), (len(r['wavelengths']), 1))
        if _algorithm(self.numerics) == 'etm':
            return self._solve_etm(r, conv, layer_index, _wants_fields(asked))
        return self._solve(r, conv, layer_index, amplitudes, _wants_scattering(asked), _wants_fields(asked))

    def _batch(self, r, conv, layer_index, idx, wl, theta, precision, amplitudes):
        """One wb_solve_batch over the wavelengths ``idx`` (with their own, possibly detuned,
        wavelength and theta)."""
        k = len(idx)
        inp = engine.BatchInputs(np.asarray(layer_index)[idx], np.tile(r['thickness'], (k, 1)), wl[idx],
                                 np.tile(r['period'], (k, 1)), theta[idx], np.full(k, r['phi']),
                                 np.full(k, r['eps_top']), np.full(k, r['eps_bot']), np.tile(r['pol'], (k, 1)))
        return engine.solve_batch(conv, inp, precision=precision, amplitudes=amplitudes, handle=self.handle)

    def _rebuild_grazing(self, r, conv, layer_index, idx, wl, theta, amplitudes, merge):
        """The solves ``idx`` the kernels flagged grazing (a layer eigenvalue zero to round-off),
        again: FP64 modes from the kernels, every flagged layer's cluster re-derived on the host
        (``graze.rebuild_grazing_cluster``, solve_2d.py:118-222 and :2463-2488 of the
        reference), then stage C on the device from the repaired modes. A numerically defective
        cluster raises NumericalError('rcwa.singular') with the reference's remedy. Returns the
        solves whose flag was cleared."""
        from . import graze
        from .adjoint import ports
        hu, hv = conv.hu, conv.hv
        li = np.asarray(layer_index)[idx]
        k, L = li.shape
        kxs, kys = [], []
        for b in idx:
            pv = ports(float(wl[b]), tuple(r['period']), float(theta[b]), float(r['phi']), r['eps_top'], r['eps_bot'],
                       hu, hv, 'cpu')
            for _ in range(L):
                kxs.append(pv['kx'].numpy()); kys.append(pv['ky'].numpy())
        kxs, kys = np.array(kxs), np.array(kys)
        w, q, W, V, _ = engine.layer_modes(conv, li.reshape(-1), kxs, kys, precision='double', handle=self.handle)
        wh, qh, Wh, Vh = (t.cpu().numpy().copy() for t in (w, q, W, V))
        slots = [conv.slot(s_).cpu().numpy() for s_ in range(3)]
        still = np.zeros(k, dtype=bool)
        for p in range(k * L):
            if not graze.grazing(wh[p]):
                continue
            lay = int(li.reshape(-1)[p])
            omega_l, omega_r = graze.layer_factors(kxs[p], kys[p], slots[0][lay], slots[1][lay], slots[2][lay])
            try:
                out = graze.rebuild_grazing_cluster(wh[p], Wh[p], Vh[p], qh[p], omega_l, omega_r)
            except FloatingPointError as exc:
                raise NumericalError(str(exc), code='rcwa.singular') from None
            if out is None:
                still[p // L] = True                  # structure not understood: the flag stays
                continue
            Wh[p], Vh[p], qh[p] = out
        dev = W.device
        inp = engine.BatchInputs(li, np.tile(r['thickness'], (k, 1)), wl[idx], np.tile(r['period'], (k, 1)),
                                 theta[idx], np.full(k, r['phi']), np.full(k, r['eps_top']), np.full(k, r['eps_bot']),
                                 np.tile(r['pol'], (k, 1)))
        res = list(engine.smm_solve(torch.as_tensor(Wh, device=dev), torch.as_tensor(Vh, device=dev),
                                    torch.as_tensor(qh, device=dev), inp, hu, hv, precision='double',
                                    amplitudes=amplitudes, handle=self.handle))
        stt = res[2]
        stt &= ~_lib.WB_ST_GRAZING
        stt[torch.as_tensor(np.nonzero(still)[0], device=stt.device)] |= _lib.WB_ST_GRAZING
        merge(idx, res)
        return tuple(int(b) for b, s_ in zip(idx, still) if not s_)

    def _solve(self, r, conv, layer_index, amplitudes=False, scattering=False, fields=False):
        """Solve every wavelength of ``r`` with the layers ``layer_index[b]`` of ``conv``; with
        ``scattering`` also keep the stack's scattering matrix of each (at the same, possibly
        detuned, wavelength and angle)."""
        B = len(r['wavelengths'])
        wl = np.asarray(r['wavelengths'], dtype=np.float64).copy()
        th = np.asarray(r['thetas'], dtype=np.float64).copy()
        out = list(self._batch(r, conv, layer_index, np.arange(B), wl, th, self.precision, amplitudes))
        R, T, status = out[:3]

        def merge(idx, res):
            t = torch.as_tensor(idx, device=R.device)
            R[t], T[t], status[t] = res[0], res[1], res[2]
            if amplitudes:
                out[3][t] = res[3]

        st = status.cpu().numpy()
        fallback = np.nonzero(st & ~_lib.WB_ST_GRAZING)[0] if self.precision == 'mixed' else np.zeros(0, int)
        if fallback.size:
            # solves the mixed form could not finish (a near-degenerate group too large for its
            # Newton step, say) are solved again with the double-float eigen-solve
            merge(fallback, self._batch(r, conv, layer_index, fallback, wl, th, 'mixed_df64_eig', amplitudes))
            st = status.cpu().numpy()
        moved = self._detune(r, conv, layer_index, wl, th, st, merge, amplitudes)
        st = status.cpu().numpy()
        flagged = np.nonzero(st & _lib.WB_ST_GRAZING)[0]
        rebuilt = ()
        if flagged.size:
            # correct or loud at a grazing order: the layer's cluster is re-derived from the
            # first-order problem, or the solve is refused as numerically defective
            rebuilt = self._rebuild_grazing(r, conv, layer_index, flagged, wl, th, amplitudes, merge)
            st = status.cpu().numpy()
        grazing = np.nonzero(st & _lib.WB_ST_GRAZING)[0]
        if grazing.size:
            warnings.warn(f'a layer mode sits on its cutoff at {grazing.size} wavelength(s) and its cluster could not '
                          'be re-derived, so those results may be inaccurate. rcwa.Numerics(detuning=1e-12) retries '
                          'them slightly detuned.', RayleighPointWarning, stacklevel=3)
        bad = st & ~_lib.WB_ST_GRAZING
        if np.any(bad & _lib.WB_ST_SINGULAR):
            raise NumericalError('a factorization met an exact zero pivot', code='rcwa.singular')
        if np.any(bad & (_lib.WB_ST_NONFINITE | _lib.WB_ST_NOCONV)):
            raise NumericalError('the solve produced non-finite results', code='rcwa.nonfinite')
        diag = {'solve_path': ('2d',) * B, 'effective_wavelengths': tuple(float(v) for v in wl),
                'effective_theta': tuple(float(v) for v in th),
                'grazing': tuple(bool(s & _lib.WB_ST_GRAZING) for s in st),
                'status': st, 'precision': self.precision,
                'fallback_solves': tuple(int(i) for i in fallback), 'detuned': moved,
                'grazing_rebuilt': tuple(int(i) for i in rebuilt),
                **_defined_flags(B, R.device, self.numerics)}
        S = self._scattering(r, conv, np.asarray(layer_index), wl, th) if scattering else None
        states = self._field_states(r, conv, np.asarray(layer_index), wl, th) if fields else None
        return Result(R[:, 0], T[:, 0], (R[:, 1], R[:, 2]), (T[:, 1], T[:, 2]), status, tuple(float(v) for v in wl),
                      diag, out[3] if amplitudes else None, S, states,
                      (np.asarray(r['thickness'], dtype=np.float64), r['period'], r.get('amplitude', 1.0),
                       r.get('bare_interface', False), tuple(r['orders']), r.get('side', 'top')), orders=r['orders'],
                      ports=_ports_context(r, wl, th), provenance=_provenance(r, self.numerics, self.precision))

    def _solve_etm(self, r, conv, layer_index, fields=False):
        """``Numerics(algorithm='etm')``: the ETM recursion (``wb_etm_solve``) over the FP64 modes
        of every (wavelength, layer) pair, a cross-check of the cascade on the same modes. Fields,
        when asked for, are read off the cascade's state as with the SMM."""
        hu, hv = r['orders']
        B, L = layer_index.shape
        n = 2 * engine.n_orders(hu, hv)
        wl = np.asarray(r['wavelengths'], dtype=np.float64).copy()
        th = np.asarray(r['thetas'], dtype=np.float64).copy()
        parts = []
        for idx, pvs, q, W, V in self._mode_chunks(r, conv, layer_index, wl, th, (2 * L + 4) * n * n * 16):
            k = len(idx)
            inp = engine.BatchInputs(layer_index[idx], np.tile(r['thickness'], (k, 1)), wl[idx],
                                     np.tile(r['period'], (k, 1)), th[idx], np.full(k, r['phi']),
                                     np.full(k, r['eps_top']), np.full(k, r['eps_bot']), np.tile(r['pol'], (k, 1)),
                                     device=W.device)
            parts.append(engine.etm_solve(W, V, q, inp, hu, hv, amplitudes=True, handle=self.handle))
        R, T, stt, amps = (torch.cat([p_[j] for p_ in parts]) for j in range(4))
        st = stt.cpu().numpy()
        if np.any(st & _lib.WB_ST_SINGULAR):
            raise NumericalError('an ETM factorization met an exact zero pivot', code='rcwa.singular')
        if np.any(st) or not (bool(torch.isfinite(R).all()) and bool(torch.isfinite(T).all())):
            raise NumericalError('the ETM solve produced non-finite results', code='rcwa.nonfinite')
        st = np.zeros(B, dtype=np.int32)
        diag = {'solve_path': ('2d',) * B, 'algorithm': 'etm', 'effective_wavelengths': tuple(float(v) for v in wl),
                'effective_theta': tuple(float(v) for v in th),
                'grazing': (False,) * B, 'status': st, 'precision': 'double', 'fallback_solves': (), 'detuned': {},
                **_defined_flags(B, R.device, self.numerics)}
        states = self._field_states(r, conv, layer_index, wl, th) if fields else None
        return Result(R[:, 0], T[:, 0], (R[:, 1], R[:, 2]), (T[:, 1], T[:, 2]),
                      torch.as_tensor(st, device=R.device), tuple(float(v) for v in wl), diag, amps, None, states,
                      (np.asarray(r['thickness'], dtype=np.float64), r['period'], r.get('amplitude', 1.0),
                       r.get('bare_interface', False), tuple(r['orders']), r.get('side', 'top')), orders=r['orders'],
                      ports=_ports_context(r, wl, th), provenance=_provenance(r, self.numerics, 'double'))

    def _mode_chunks(self, r, conv, layer_index, wl, th, per_wl_bytes, budget=2 << 30):
        """FP64 modes of every (wavelength, layer) pair (wb_layer_modes), a chunk of wavelengths
        at a time: yields ``(idx, pvs, q, W, V)`` with W, V Cartesian in natural orientation."""
        from .adjoint import ports
        hu, hv = r['orders']
        B, L = layer_index.shape
        dev = conv.buf.device
        chunk = max(1, int(budget // per_wl_bytes))
        for lo in range(0, B, chunk):
            idx = np.arange(lo, min(B, lo + chunk))
            pvs = [ports(float(wl[b]), r['period'], float(th[b]), r['phi'], r['eps_top'], r['eps_bot'], hu, hv, dev)
                   for b in idx]
            kx = torch.stack([p['kx'] for p in pvs]).repeat_interleave(L, 0)
            ky = torch.stack([p['ky'] for p in pvs]).repeat_interleave(L, 0)
            _, q, W, V, st = engine.layer_modes(conv, layer_index[idx].reshape(-1), kx, ky, precision='double',
                                                handle=self.handle)
            bad = st.cpu().numpy() & ~_lib.WB_ST_GRAZING
            if np.any(bad & _lib.WB_ST_SINGULAR):
                raise NumericalError('a layer factorization met an exact zero pivot', code='rcwa.singular')
            if np.any(bad):
                raise NumericalError('the layer eigen-solve did not converge', code='rcwa.nonfinite')
            yield idx, pvs, q, W, V

    def _field_states(self, r, conv, layer_index, wl, th):
        """Per wavelength, every layer's modes and the incident column's ``(+, -)`` amplitudes
        (Outputs(fields=True)), computed on the device from FP64 modes; the states stay resident
        (2 (2N)^2 complex per layer and wavelength) for ``Result.field``."""
        from . import fields as F
        hu, hv = r['orders']
        B, L = layer_index.shape
        n = 2 * engine.n_orders(hu, hv)
        states = []
        for idx, pvs, q, W, V in self._mode_chunks(r, conv, layer_index, wl, th, (6 * L + 2) * n * n * 16):
            k = len(idx)
            inp = engine.BatchInputs(layer_index[idx], np.tile(r['thickness'], (k, 1)), wl[idx],
                                     np.tile(r['period'], (k, 1)), th[idx], np.full(k, r['phi']),
                                     np.full(k, r['eps_top']), np.full(k, r['eps_bot']), np.tile(r['pol'], (k, 1)),
                                     device=W.device)
            C = torch.stack([F.incident_column(pv, r['pol']) for pv in pvs])
            plus, mtop, mbot, cref, ctrn, st = engine.layer_amplitudes(W, V, q, inp, hu, hv, C, handle=self.handle)
            if np.any(st.cpu().numpy() & _lib.WB_ST_SINGULAR):
                raise NumericalError('a layer factorization met an exact zero pivot', code='rcwa.singular')
            for i, b in enumerate(idx):
                modes = [(W[i * L + l], V[i * L + l], q[i * L + l]) for l in range(L)]
                epz = [conv.slot(2)[int(layer_index[b][l])] for l in range(L)]
                rasters = [r['rasters'][int(layer_index[b][l])] for l in range(L)]
                states.append(F.build_state(modes, epz, r['thickness'], wl[b], pvs[i], r['pol'], hu, hv, rasters,
                                            faces=(plus[i], mtop[i], mbot[i], cref[i], ctrn[i])))
        return tuple(states)

    def _scattering(self, r, conv, layer_index, wl, th):
        """The stack's scattering matrix per wavelength (Outputs(scattering=True)): the FP64 modes
        of every (wavelength, layer) pair, then wb_scattering_matrix, a chunk of wavelengths at a
        time so that about 2 GiB of modes and blocks are held at once."""
        hu, hv = r['orders']
        B, L = layer_index.shape
        n = 2 * engine.n_orders(hu, hv)
        n_top, n_bot = complex(np.sqrt(complex(r['eps_top']))), complex(np.sqrt(complex(r['eps_bot'])))
        out = []
        for idx, pvs, q, W, V in self._mode_chunks(r, conv, layer_index, wl, th, (2 * L + 4) * n * n * 16):
            k = len(idx)
            inp = engine.BatchInputs(layer_index[idx], np.tile(r['thickness'], (k, 1)), wl[idx],
                                     np.tile(r['period'], (k, 1)), th[idx], np.full(k, r['phi']),
                                     np.full(k, r['eps_top']), np.full(k, r['eps_bot']), np.tile(r['pol'], (k, 1)))
            S11, S12, S21, S22, st = engine.scattering_matrix(W, V, q, inp, hu, hv, handle=self.handle)
            bad = st.cpu().numpy() & ~_lib.WB_ST_GRAZING
            if np.any(bad & _lib.WB_ST_SINGULAR):
                raise NumericalError('a factorization of the scattering matrix met an exact zero pivot',
                                     code='rcwa.singular')
            if np.any(bad):
                raise NumericalError('the scattering matrix is not finite', code='rcwa.nonfinite')
            for i, b in enumerate(idx):
                kxo, kyo = pvs[i]['kx'].cpu().numpy(), pvs[i]['ky'].cpu().numpy()
                out.append(ScatteringMatrix(S11[i], S12[i], S21[i], S22[i],
                                            entry_port=Port(kxo, kyo, n_top, 1.0, 'sp'),
                                            exit_port=Port(kxo, kyo, n_bot, 1.0, 'sp')))
        return tuple(out)

    def _detune(self, r, conv, layer_index, wl, th, st, merge, amplitudes):
        """The reference's auto-detune ladder (engine.py:6382-6480), opt-in through
        ``Numerics(detuning=step)``, a positive relative step: wavelengths with a grazing layer mode or a failed
        solve are solved again at wavelength * (1 + step), then, where the condition stays and
        theta != 0, with theta * (1 + step) as well. A rung that fails keeps the previous values;
        the detuned values are kept (``wl``, ``th`` updated in place). Returns {index: knobs}."""
        det = getattr(_numerics_or_default(self.numerics), 'detuning', None)
        if not det:
            return {}
        step = float(det)
        remaining = np.nonzero(st != 0)[0]
        moved = {}
        knobs = ['wavelength'] + (['theta'] if np.any(np.asarray(r['thetas']) != 0.0) else [])
        for knob in knobs:
            if not remaining.size:
                break
            arr = wl if knob == 'wavelength' else th
            saved = arr[remaining].copy()
            arr[remaining] = saved * (1 + step)
            res = self._batch(r, conv, layer_index, remaining, wl, th, self.precision, amplitudes)
            s2 = res[2].cpu().numpy()
            ok = (s2 & ~_lib.WB_ST_GRAZING) == 0           # the rung solved (grazing or not)
            arr[remaining[~ok]] = saved[~ok]                # a failed rung keeps the previous values
            if ok.any():
                sel = np.nonzero(ok)[0]
                merge(remaining[sel], tuple(x[torch.as_tensor(sel, device=x.device)] if x is not None else None
                                           for x in res))
                for i in remaining[sel]:
                    moved.setdefault(int(i), []).append(knob)
            remaining = remaining[~ok | ((s2 & _lib.WB_ST_GRAZING) != 0)]
        if moved:
            warnings.warn(f'auto_detune: {len(moved)} wavelength(s) had a mode on its cutoff or a failed solve; '
                          f're-solved with {", ".join(sorted({k for v in moved.values() for k in v}))} * (1 + {step:g}). '
                          'The results keep those values (Result.diagnostics["effective_wavelengths"]).',
                          AutoDetuneWarning, stacklevel=4)
        return {i: tuple(v) for i, v in moved.items()}


def _defined_flags(B, device, numerics):
    """The diagnostics' power and efficiency flags (results.py:474-478): on this path (real
    in-plane wavevectors from a lossless superstrate) every solve has both."""
    ones = torch.ones(B, dtype=torch.bool, device=device)
    return {'port_power_defined': ones, 'efficiency_defined': ones,
            'detuning_relative_step': getattr(_numerics_or_default(numerics), 'detuning', None),
            'half_space_merge': None}


def _provenance(r, numerics, precision):
    """What produced a result (results.py:479-484): solver, versions, units, numerics, frames."""
    from . import __version__
    try:
        library = int(_lib.load().wb_version())
    except ImportError:               # no library: nothing ran on the device, only the version is unknown
        library = None
    return {'solver': 'rcwa', 'backend': 'gb300', 'code_version': __version__,
            'library_version': library, 'length_units': r.get('length', 'm'),
            'units': Units(r.get('length', 'm')), 'numerics': numerics, 'precision': precision,
            'coordinate_frame': '+z up; bottom interface z=0; layers bottom-to-top',
            'time_convention': 'exp(-i*omega*t)', 'source_normalization': 'electric amplitude V/m',
            'requested_wavelengths': tuple(float(v) for v in r['wavelengths'])}


def _ports_context(r, wl, th):
    """What the diffraction-order readings need beside R, T and the amplitudes: the solves'
    effective wavelengths and angles, the media, the cell, the source and the length unit."""
    return dict(wavelengths=np.asarray(wl, dtype=np.float64), thetas=np.asarray(th, dtype=np.float64),
                phi=float(r['phi']), period=tuple(r['period']), eps_top=r['eps_top'], eps_bot=r['eps_bot'],
                pol=r['pol'], amplitude=r.get('amplitude', 1.0), length=r.get('length', 'm'),
                top_plane=float(np.sum(r['thickness'])), side=r.get('side', 'top'))


def _same_rasters(a, b):
    return len(a) == len(b) and all(x.shape == y.shape and np.array_equal(x, y) for x, y in zip(a, b))


def compression(cell):
    """A raster reduced to one pixel per block of equal neighbours, with the right edges of the
    column and row blocks on the unit cell: ``(cell, x_edges, y_edges)``
    (compression_indices, factorization.py:3005-3045). A column block ends where any row
    changes between neighbouring columns; a row block where the column-reduced rows change."""
    cell = np.asarray(cell)
    ny, nx = cell.shape
    cols = np.append(np.nonzero((cell[:, 1:] != cell[:, :-1]).any(axis=0))[0], nx - 1)
    reduced = cell[:, cols]
    rows = np.append(np.nonzero((reduced[1:] != reduced[:-1]).any(axis=1))[0], ny - 1)
    return (reduced[rows], (cols.astype(np.float64) + 1.0) / nx, (rows.astype(np.float64) + 1.0) / ny)


def _assemble_layers(rasters, hu, hv, handle, integrated=False):
    """Stage A for every layer; consecutive layers of one shape are assembled together. With
    ``integrated`` each raster is compressed first (on the host, once per prepare) and shapes
    are those of the compressed cells."""
    if integrated:
        comp = [compression(e) for e in rasters]
        cells = [c[0] for c in comp]
    else:
        cells = rasters
    bufs = []
    i = 0
    while i < len(cells):
        j = i
        while j < len(cells) and cells[j].shape == cells[i].shape:
            j += 1
        eps = torch.as_tensor(np.stack(cells[i:j]), device='cuda')
        edges = (np.stack([c[1] for c in comp[i:j]]), np.stack([c[2] for c in comp[i:j]])) if integrated else None
        bufs.append(engine.assemble(eps, hu, hv, handle=handle, edges=edges).buf)
        i = j
    return engine.ConvStack(torch.cat(bufs, dim=0), hu, hv)


def prepare(problem, *, numerics=None, backend='gb300', device='cuda', precision='double'):
    """Resolve and assemble once (_lifecycle.py:737-797)."""
    if backend not in ('gb300', 'cuda'):
        raise ValidationError(f'backend {backend!r}: this package is the gb300 backend', path='backend')
    if precision not in ('double', 'mixed'):
        raise ValidationError("precision must be 'double' or 'mixed'", path='precision')
    dev = torch.device(device)
    if dev.type != 'cuda':
        raise ValidationError('the GB300 backend runs on a CUDA device only; there is no CPU path',
                              path='device')
    handle = _lib.handle(dev.index or 0)
    return Prepared(problem, numerics, precision, handle)


def sample_structure(problem, *, layer=0, samples=512, wavelength_index=0, quantity='epsilon', component=None):
    """One layer's relative permittivity as the solve reads it, without a solve
    (_structure.py:19-100 of the reference): a raster layer keeps its own resolution, axes
    ``(y, x)``, row zero the negative-y edge; ``layer`` counts from the bottom. Region and
    profiled layers, permeability and tensor components are outside the raster path."""
    layers = tuple(problem.stack.layers)
    if type(layer) is not int or not 0 <= layer < len(layers):
        raise ValidationError('layer must index a finite layer from zero.', code='structure.layer', path='layer')
    if type(samples) is not int or samples < 1:
        raise ValidationError('samples must be a positive integer.', code='structure.samples', path='samples')
    if quantity not in ('epsilon', 'mu'):
        raise ValidationError("quantity must be 'epsilon' or 'mu'.", code='structure.quantity', path='quantity')
    wl = np.atleast_1d(np.asarray(problem.excitation.wavelength, dtype=np.float64)).reshape(-1)
    if type(wavelength_index) is not int or not 0 <= wavelength_index < len(wl):
        raise ValidationError('wavelength_index must index the excitation spectrum from zero.',
                              code='structure.wavelength', path='wavelength_index')
    if quantity == 'mu' or component is not None:
        raise UnsupportedFeatureError('permeability and tensor components are outside the GB300 raster path',
                                      path='quantity' if quantity == 'mu' else 'component')
    selected = layers[layer]
    if getattr(selected, 'regions', ()):
        raise UnsupportedFeatureError('region (shape) layers are outside the GB300 raster path',
                                      path=f'stack.layers[{layer}]')
    eps = selected.epsilon
    if eps is None:
        eps = _scalar_eps(selected.background, f'stack.layers[{layer}].background')
    eps = np.array(eps.detach().cpu().numpy() if hasattr(eps, 'detach') else eps, dtype=np.complex128)
    return eps.reshape(1, 1) if eps.ndim == 0 else eps.reshape(1, -1) if eps.ndim == 1 else eps


def run(problem, *, numerics=None, backend='gb300', device='cuda', precision='double', amplitudes=True):
    """``prepare(...).run()`` (_lifecycle.py:801-803)."""
    return prepare(problem, numerics=numerics, backend=backend, device=device,
                   precision=precision).run(amplitudes=amplitudes)


from . import operators  # noqa: E402  (rcwa.operators.assemble / solve, as in the reference)
