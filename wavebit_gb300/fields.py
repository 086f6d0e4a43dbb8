"""Field reconstruction inside the stack (``Outputs(fields=True)``, ``Result.field``).

The reference keeps, per wavelength, every layer's ``(+, -)`` mode amplitudes of the incident
column, read off the S-matrix cascade (rcwa/_engine/scattering.py:236-350), and sums the
collocated phasors from them on request (rcwa/results.py:148-229,
rcwa/_engine/field_result.py:332-700, rcwa/_engine/fields.py:630-790). Here the modes are the
stage-B kernels' (wb_layer_modes, FP64); the amplitudes come from the cascade kernels' own
recursion (``wb_layer_amplitudes``, :func:`wavebit_gb300.engine.layer_amplitudes`) and the
synthesis is batched matrix products on the device that holds the modes.
:func:`layer_amplitudes` restates the same recursion in torch (the adjoint's
:func:`wavebit_gb300.adjoint.cascade_forward`), for modes held on the host.

Conventions (the reference's): ``x`` and ``y`` are measured from the cell centre, ``z`` upward
from the stack's bottom face, a face belongs to the layer above it; values are
``(wavelength, z, y, x, 6)`` for ``(Ex, Ey, Ez, Hx, Hy, Hz)``, E in V/m for a source of
``amplitude`` V/m and H in A/m, time convention ``exp(-i omega t)``.
"""
import math
from typing import NamedTuple

import numpy as np
import torch

from .adjoint import cascade_forward

#: free-space impedance 1 / (epsilon0 c0) (units.py:7-9 of the reference)
Z0 = 1.0 / (8.8541878188e-12 * 299792458.0)
#: a mode's ``-`` amplitude is read off the layer's top face below this ``|k0 q d|``
#: (scattering.py:225-232, modal_gradient.two_face)
TOP_FACE = 1.0
#: (Ex, Ey, Ez, Hx, Hy, Hz) parity between the propagation frame (z into the stack from the
#: lit face) and the public frame (z up from the bottom): E is polar, H axial (fields.py:114-118)
MIRROR = (1.0, 1.0, -1.0, -1.0, -1.0, 1.0)
COMPONENTS = ('Ex', 'Ey', 'Ez', 'Hx', 'Hy', 'Hz')


class LayerState(NamedTuple):
    """One layer of one wavelength: Cartesian modes (natural orientation), roots, thickness,
    the inverse-zz convolution slot (cell corner), the incident column's amplitudes and the
    layer's raster ``(ny, nx)`` (for Lalanne's rule; ``None`` when not kept)."""
    W: torch.Tensor
    V: torch.Tensor
    q: torch.Tensor
    d: float
    epz_i: torch.Tensor
    plus: torch.Tensor
    minus: torch.Tensor
    raster: object = None


class FieldState(NamedTuple):
    """What one wavelength keeps for :meth:`Result.field` and :meth:`Result.boundary_fields`;
    layers entry (top) face first; ``boundary`` maps each face to its (incoming, outgoing)
    six-component spectra (N, 6)."""
    k0: float
    kx: torch.Tensor          # (N,) per-order kx / k0
    ky: torch.Tensor
    odd: torch.Tensor         # (N,) True where (-1)^(m+n) = -1 (corner -> centre sign)
    layers: tuple
    boundary: dict = None


class FieldSamples(NamedTuple):
    """Collocated phasors and the points they were taken at (results.py:214-229)."""
    coordinates: dict
    values: torch.Tensor
    components: tuple
    sampling: str
    metadata: dict


def z_mirror(device):
    """The six components' signs under z -> -z: E is a polar vector (E_z turns), H an axial
    one (H_x and H_y turn). A scene lit from below is solved as its mirror image lit from above,
    and its fields are that solve's, mirrored back."""
    return torch.as_tensor([1, 1, -1, -1, -1, 1], dtype=torch.complex128, device=device)


def sp_rotate(W, V, c, s):
    """The s/p rotation of a layer's Cartesian modes (solve_2d.py:2584-2616), as the kernels'
    sp_rotate_kernel and :func:`wavebit_gb300.adjoint.solve_and_grad` apply it."""
    N = c.shape[0]
    W1, W2, V1, V2 = W[:N], W[N:], V[:N], V[N:]
    bw = torch.cat([c[:, None] * W2 - s[:, None] * W1, c[:, None] * W1 + s[:, None] * W2], 0)
    bv = torch.cat([c[:, None] * V1 + s[:, None] * V2, c[:, None] * V2 - s[:, None] * V1], 0)
    return bw, bv


def layer_faces(modes, thickness, k0, pv, C):
    """Every layer's ``(plus, minus_top, minus_bottom)`` for the incidence columns ``C`` (n, k),
    and the reflected and transmitted columns: the torch restatement of ``wb_layer_amplitudes``
    (scattering.py:270-350). ``modes`` is a list of ``(W, V, q)`` (Cartesian, entry face first),
    ``pv`` the port vectors of :func:`wavebit_gb300.adjoint.ports`.

    With ``g``, ``h = R g`` the gap amplitudes above a layer and ``bW``, ``bV`` its rotated modes,
    the layer's amplitudes at that face are ``(b1 + b2)/2`` down and ``(b1 - b2)/2`` up,
    ``b1 = bW^-1 wg (g + h)``, ``b2 = bV^-1 vg (g - h)``; ``minus_bottom`` is the same up-going
    half from the gap below the layer, with the same layer's ``bW``, ``bV``."""
    bW, bV, Xs = [], [], []
    for (W, V, q), d in zip(modes, thickness):
        bw, bv = sp_rotate(W, V, pv['c'], pv['s'])
        bW.append(bw); bV.append(bv)
        Xs.append(torch.exp(-k0 * float(d) * q))
    cref, ctrn, sv = cascade_forward(bW, bV, Xs, pv, C)
    wg, vg = pv['wg'][:, None], pv['vg'][:, None]
    faces = []
    for l in range(len(modes)):
        b1, b2 = sv['td'][l]['b1'], sv['td'][l]['b2']
        gn = sv['g'][l + 1]
        hn = sv['Rk'][l + 1] @ gn
        minus_bottom = 0.5 * (torch.linalg.solve(bW[l], wg * (gn + hn)) - torch.linalg.solve(bV[l], vg * (gn - hn)))
        faces.append((0.5 * (b1 + b2), 0.5 * (b1 - b2), minus_bottom))
    return faces, cref, ctrn


def layer_amplitudes(modes, thickness, k0, pv, C):
    """Every layer's ``(+, -)`` amplitudes and the reflected and transmitted columns, by the torch
    recursion (:func:`layer_faces` and :func:`face_amplitudes`)."""
    faces, cref, ctrn = layer_faces(modes, thickness, k0, pv, C)
    return face_amplitudes(faces, [q for _, _, q in modes], thickness, k0), cref, ctrn


def face_amplitudes(faces, qs, thickness, k0):
    """Each layer's ``(+, -)`` amplitudes from its ``(plus, minus_top, minus_bottom)``: the ``-``
    amplitude is read at the bottom face, except for a mode with ``|k0 q d| < 1``, whose two
    amplitudes nearly cancel in the field and which takes its top-face value carried down by
    ``exp(k0 q d)`` (scattering.py:225-232, modal_gradient.two_face)."""
    out = []
    for (plus, minus_top, minus_bottom), q, d in zip(faces, qs, thickness):
        kd = k0 * float(d)
        keep = (torch.abs(q * kd) < TOP_FACE)[:, None]
        carried = torch.exp(torch.where(keep[:, 0], kd * q, torch.zeros_like(q)))[:, None] * minus_top
        out.append((plus, torch.where(keep, carried, minus_bottom)))
    return out


def order_waves(kx, ky, c, s, kzt, kzb, n_top, n_bot, ratios, pol):
    """Per order, the incoming wave and the reflected and transmitted ones, six components each
    ``(E, k x E)`` (field_result.py:700-800, ordinary_spectra): every order's s and p waves in the
    Cartesian basis ``e_s = (-s, c, 0)``, ``e_p = (-kz c, -kz s, d rho) / n``, ``H = k x e``
    (``k = (kx, ky, d kz)``, ``d = -1`` down, ``+1`` up, ``rho = kx c + ky s``) of the half-space it
    lives in, weighted by the Fresnel ratios ``(r_s, r_p, t_s, t_p)`` about the cell centre (the
    reflected p one with the opposite sign to that basis). Every argument but the two indices
    and ``pol`` may carry leading batch axes; returns three ``(..., N, 6)`` tensors."""
    C = torch.complex128
    gx, gy, c, s = (t.to(C) for t in (kx, ky, c, s))
    zero = torch.zeros_like(gx)
    rho = gx * c + gy * s

    def cross(a, b):
        a0, a1, a2 = a.unbind(-1)
        b0, b1, b2 = b.unbind(-1)
        return torch.stack([a1 * b2 - a2 * b1, a2 * b0 - a0 * b2, a0 * b1 - a1 * b0], -1)

    def basis(n, kz, d):
        es = torch.stack([-s, c, zero], -1)
        ep = torch.stack([-kz * c / n, -kz * s / n, d * rho / n], -1)
        k = torch.stack([gx, gy, d * kz], -1)
        return torch.cat([es, cross(k, es)], -1), torch.cat([ep, cross(k, ep)], -1)

    inc_s, inc_p = basis(complex(n_top), kzt, -1.0)
    ref_s, ref_p = basis(complex(n_top), kzt, 1.0)
    trn_s, trn_p = basis(complex(n_bot), kzb, -1.0)
    r_s, r_p, t_s, t_p = ratios
    N = gx.shape[-1]
    delta = torch.zeros(N, dtype=C, device=gx.device)
    delta[N // 2] = 1.0
    incoming = delta[:, None] * (complex(pol[0]) * inc_s + complex(pol[1]) * inc_p)
    reflected = r_s[..., None] * ref_s - r_p[..., None] * ref_p
    transmitted = t_s[..., None] * trn_s + t_p[..., None] * trn_p
    return incoming, reflected, transmitted


def order_table(wavelengths, thetas, phi, period, eps_top, eps_bot, hu, hv, device):
    """Every retained order's normalised in-plane wavevector ``(kx, ky)``, its s/p frame angle
    ``(c, s) = (cos, sin)`` and its normal component ``kz`` in the superstrate and the substrate,
    each ``(B, N)`` over ``B`` solves: what the ports kernel forms per solve
    (conventions.py:1118-1147, solve_2d.py:76-98), for all solves at once."""
    import math
    C = torch.complex128
    wl = torch.as_tensor(np.asarray(wavelengths, dtype=np.float64), device=device)[:, None]
    th = torch.as_tensor(np.asarray(thetas, dtype=np.float64), device=device)[:, None]
    nu = 2 * hu + 1
    N = nu * (2 * hv + 1)
    index = math.sqrt(float(np.real(eps_top)))
    kix = index * torch.sin(th) * math.cos(phi)
    kiy = index * torch.sin(th) * math.sin(phi)
    u = (torch.arange(N, device=device) % nu - hu).double()
    v = (torch.arange(N, device=device) // nu - hv).double()
    kx = kix + u * (wl / period[0])
    ky = kiy + v * (wl / period[1])
    one = torch.ones_like(kx)
    spec = math.atan(math.sin(phi) / math.cos(phi)) + (math.pi if math.cos(phi) < 0 else 0.0)
    vphi = torch.where(kx == 0,
                       torch.where(ky == 0, spec * one, torch.where(ky < 0, -math.pi / 2 * one, math.pi / 2 * one)
                                   - kx / torch.where(ky == 0, one, ky)),
                       torch.atan(ky / torch.where(kx == 0, one, kx)) + math.pi * (kx < 0).double())
    kpar = (kx * kx + ky * ky).to(C)

    def kz(eps):
        z = torch.sqrt(complex(eps) - kpar)
        return torch.where((z.real + z.imag) < 0, -z, z)
    return kx, ky, torch.cos(vphi), torch.sin(vphi), kz(eps_top), kz(eps_bot)


def wave_power(waves, sign, area, amplitude):
    """The time-averaged power of each wave through a face of ``area`` (m^2), counted along
    ``sign`` times +z: ``sign/2 Re(E_x conj(Z0 H_y) - E_y conj(Z0 H_x)) / Z0 * area * |amplitude|^2``
    (results.py:279-282)."""
    return (sign * 0.5 / Z0 * (waves[..., 0] * waves[..., 4].conj() - waves[..., 1] * waves[..., 3].conj()).real
            * area * abs(amplitude) ** 2)


def boundary_spectra(pv, cref, ctrn, pol, odd):
    """Each face's (incoming, outgoing) six-component spectra of the incident column, (N, 6) per
    order (field_result.py:700-800, ordinary_spectra / ordinary_state): on the lit (top) face the
    incident wave and the reflected orders, on the far face nothing and the transmitted orders.
    Every order's s and p waves take the Cartesian basis ``e_s = (-s, c, 0)``,
    ``e_p = (-kz c, -kz s, d rho) / n``, ``H = k x e`` (k = (kx, ky, d kz), d = -1 down, +1 up,
    rho = kx c + ky s) of the half-space it lives in; the coefficients are the Fresnel amplitude
    ratios about the cell centre (the reflected p one with the opposite sign to that basis)."""
    N = pv['kx'].shape[0]
    C = torch.complex128
    n_top, n_bot = complex(pv['nt']), complex(pv['nb'])
    sign = torch.where(odd, -1.0, 1.0).to(C)
    ratios = (cref[:N, 0] * sign, (-cref[N:, 0]) / (-1j * n_top) * sign,
              ctrn[:N, 0] * sign, ctrn[N:, 0] / (-1j * n_bot) * sign)
    incoming, reflected, transmitted = order_waves(pv['kx'], pv['ky'], pv['c'], pv['s'], pv['kzt'], pv['kzb'],
                                                   n_top, n_bot, ratios, pol)
    return {'top': (incoming, reflected), 'bottom': (torch.zeros_like(transmitted), transmitted)}


def expand_boundary(state, side, part, x, y, amplitude):
    """``(ny, nx, 6)`` phasors of one face's waves at the centre-origin points (field_result.py:109-122)."""
    incoming, outgoing = state.boundary[side]
    coef = incoming if part == 'incoming' else outgoing if part == 'outgoing' else incoming + outgoing
    dev = state.kx.device
    xs = torch.as_tensor(x, dtype=torch.float64, device=dev)
    ys = torch.as_tensor(y, dtype=torch.float64, device=dev)
    arg = state.k0 * (xs[None, :, None] * state.kx[None, None, :] + ys[:, None, None] * state.ky[None, None, :])
    out = torch.exp(1j * arg) @ coef                                    # (ny, nx, 6)
    scale = torch.as_tensor([1, 1, 1, 1 / Z0, 1 / Z0, 1 / Z0], dtype=torch.complex128, device=dev)
    return complex(amplitude) * out * scale


def layer_coefficients(layer, k0, kx, ky, depth):
    """Per-order ``(Sx, Sy, -Sz, i Ux, i Uy, -i Uz)`` of the incident column at ``depth`` (nz,)
    below the layer's top face, in the propagation frame (fields.py:630-790, ``U = i H``):
    ``Sx, Sy = W (a+ + a-)``, ``Ux, Uy = V (a- - a+)`` with ``a+ = exp(-k0 q z) c+`` and
    ``a- = exp(k0 q (z - d)) c-``; ``Sz = i epz_i (Kx Uy - Ky Ux)``, ``Uz = i (Kx Sy - Ky Sx)``."""
    N = kx.shape[0]
    z = depth[:, None]
    q = layer.q[None, :]
    ap = torch.exp(-k0 * q * z) * layer.plus[None, :]
    am = torch.exp(k0 * q * (z - layer.d)) * layer.minus[None, :]
    S = (ap + am) @ layer.W.T                                # (nz, n): Sx | Sy
    U = (am - ap) @ layer.V.T                                #           Ux | Uy
    Sx, Sy, Ux, Uy = S[:, :N], S[:, N:], U[:, :N], U[:, N:]
    Sz = 1j * (kx[None, :] * Uy - ky[None, :] * Ux) @ layer.epz_i.T
    Uz = 1j * (kx[None, :] * Sy - ky[None, :] * Sx)
    return torch.stack([Sx, Sy, -Sz, 1j * Ux, 1j * Uy, -1j * Uz], dim=-1)   # (nz, N, 6)


# ------------------------------------------------------------------ Lalanne's rule (2D)

def staircase_series(lines, h):
    """Orders ``-2h..2h`` of each line (rows of ``lines``) as an exact staircase over equal pixels
    about the cell corner -- the series stage A's series_kernel evaluates (factorization.py:
    289-440): the DFT of ``(a - a0)/n`` at ``k mod n``, times ``sinc(k/n) exp(-i pi k/n)``, plus
    ``a0`` at order 0."""
    lines = np.asarray(lines, dtype=np.complex128)
    n = lines.shape[-1]
    k = np.arange(-2 * h, 2 * h + 1)
    a0 = lines[:, :1]
    spec = np.fft.fft((lines - a0) / n, axis=-1) if n > 1 else np.zeros_like(lines)
    t = k / n
    with np.errstate(invalid='ignore', divide='ignore'):
        sinc = np.where(k == 0, 1.0, np.sin(np.pi * t) / (np.pi * t))
    out = spec[:, k % n] * (sinc * np.exp(-1j * np.pi * t))[None, :]
    out[:, 2 * h] += a0[:, 0]
    return out


def line_rules(lines, h):
    """Li's inverse rule ``[T(1/a)]^-1`` of each line, ``(m, 2h+1, 2h+1)``, ``T[r, c] = c_{r-c}``
    (factorization.py:570-592): it takes the Fourier coefficients of the field normal to the
    line's walls to those of its displacement."""
    c = staircase_series(1.0 / np.asarray(lines, dtype=np.complex128), h)
    r = np.arange(2 * h + 1)
    return np.linalg.inv(c[:, r[:, None] - r[None, :] + 2 * h])


def sample_pixels(corner_points, period, n_pixels):
    """The raster pixel under each sample (corner-origin coordinates), periodically; a sample
    on a wall belongs to the pixel on its positive side (lalanne.py:298-318)."""
    frac = np.asarray(corner_points, dtype=np.float64) / float(period)
    return np.floor(frac * n_pixels + 1e-9).astype(int) % n_pixels


def lalanne_pair(coef, raster, hu, hv, k0, kx_u, ky_v, x, y, period, phase, odd):
    """``E_x`` and ``E_y`` ``(nz, ny, nx)`` of a patterned layer by Lalanne's rule
    (fields.py:1068-1110, field_result.py:610-650 of the reference): in the kernels' corner frame
    (the centre sign of ``coef`` undone), the ``E_x`` series is summed over the y orders, turned
    into the ``D_x`` series by the inverse rule of the raster row under each y sample, summed over
    x and divided by ``eps`` at the sample; ``E_y`` likewise along the columns; ``phase`` puts the
    incident wave's phase at the cell centre back."""
    dev = coef.device
    nu, nv = 2 * hu + 1, 2 * hv + 1
    ny, nx = raster.shape
    xc = np.asarray(x, dtype=np.float64) + 0.5 * period[0]
    yc = np.asarray(y, dtype=np.float64) + 0.5 * period[1]
    cols = sample_pixels(xc, period[0], nx)
    rows = sample_pixels(yc, period[1], ny)
    ops_x = torch.as_tensor(line_rules(raster[rows], hu), device=dev)              # (n_y, nu, nu)
    ops_y = torch.as_tensor(line_rules(raster[:, cols].T, hv), device=dev)         # (n_x, nv, nv)
    eps = torch.as_tensor(raster[np.ix_(rows, cols)], device=dev)                 # (n_y, n_x)
    kernel = torch.where(odd[None, :, None], -coef, coef)
    gx = kernel[..., 0].reshape(-1, nv, nu)
    gy = kernel[..., 1].reshape(-1, nv, nu)
    px = torch.exp(1j * k0 * torch.as_tensor(xc, device=dev)[:, None] * kx_u[None, :])   # (n_x, nu)
    py = torch.exp(1j * k0 * torch.as_tensor(yc, device=dev)[:, None] * ky_v[None, :])   # (n_y, nv)
    ex_rows = torch.einsum('jv,zvu->zju', py, gx)
    dx = torch.einsum('jab,zjb->zja', ops_x, ex_rows)
    ex = torch.einsum('zju,iu->zji', dx, px) / eps
    ey_cols = torch.einsum('zvu,iu->ziv', gy, px)
    dy = torch.einsum('iab,zib->zia', ops_y, ey_cols)
    ey = torch.einsum('ziv,jv->zji', dy, py) / eps
    return ex * phase, ey * phase


def heights(thickness_top_first, z):
    """Public heights -> ``(owner, depth)``: the layer (entry face first) holding each height and
    the depth below that layer's top face. Heights run upward from the bottom face; a face
    belongs to the layer above it; the outer faces are inside (field_result.py:375-398)."""
    ds = np.asarray(thickness_top_first, dtype=np.float64)[::-1]       # bottom layer first
    L = ds.shape[0]
    edges = np.concatenate([[0.0], np.cumsum(ds)])
    z = np.asarray(z, dtype=np.float64).reshape(-1)
    if not np.all(np.isfinite(z)):
        raise ValueError('z must hold finite heights')
    if z.size and (z.min() < 0.0 or z.max() > edges[-1]):
        raise ValueError(f'z coordinates must lie inside the stack, 0 to {edges[-1]:g} measured upward from '
                         f'its bottom; got {z.min():g} to {z.max():g}')
    j = np.minimum((z[:, None] >= edges[None, 1:]).sum(axis=1), L - 1)
    return L - 1 - j, ds[j] - (z - edges[j])


def synthesize(state, owner, depth, x, y, amplitude, reconstruction='plain', period=None, orders=None):
    """``(nz, ny, nx, 6)`` phasors of one wavelength at the heights ``(owner, depth)`` and the
    centre-origin points ``x`` (nx,), ``y`` (ny,) (field_result.py:109-122, 640-690).
    ``reconstruction='lalanne'`` rebuilds ``E_x`` and ``E_y`` in patterned layers by Lalanne's rule
    (needs the ``period`` and the ``orders`` ``(hu, hv)``)."""
    dev = state.kx.device
    nz, N = owner.shape[0], state.kx.shape[0]
    coef = torch.zeros((nz, N, 6), dtype=torch.complex128, device=dev)
    for p, layer in enumerate(state.layers):
        sel = np.flatnonzero(owner == p)
        if sel.size:
            idx = torch.as_tensor(sel, device=dev)
            d = torch.as_tensor(depth[sel], dtype=torch.float64, device=dev)
            coef[idx] = layer_coefficients(layer, state.k0, state.kx, state.ky, d)
    coef = coef * torch.as_tensor(MIRROR, dtype=torch.complex128, device=dev)
    coef = torch.where(state.odd[None, :, None], -coef, coef)
    xs = torch.as_tensor(x, dtype=torch.float64, device=dev)
    ys = torch.as_tensor(y, dtype=torch.float64, device=dev)
    arg = state.k0 * (xs[None, :, None] * state.kx[None, None, :] + ys[:, None, None] * state.ky[None, None, :])
    phase = torch.exp(1j * arg).reshape(-1, N)                         # (ny*nx, N)
    out = torch.einsum('po,zoc->zpc', phase, coef).reshape(nz, ys.shape[0], xs.shape[0], 6)
    if reconstruction == 'lalanne':
        hu, hv = orders
        nu = 2 * hu + 1
        kx_u, ky_v = state.kx[:nu], state.ky[::nu]
        spec = N // 2
        centre_phase = torch.exp(-1j * state.k0 * (state.kx[spec] * 0.5 * period[0] + state.ky[spec] * 0.5 * period[1]))
        for p, layer in enumerate(state.layers):
            r = layer.raster
            sel = np.flatnonzero(owner == p)
            if r is None or not sel.size or np.all(r == r.flat[0]):
                continue                          # a uniform layer keeps the Fourier sum
            idx = torch.as_tensor(sel, device=dev)
            ex, ey = lalanne_pair(coef[idx], r, hu, hv, state.k0, kx_u, ky_v, x, y, period, centre_phase, state.odd)
            out[idx, :, :, 0], out[idx, :, :, 1] = ex, ey
    scale = torch.as_tensor([1, 1, 1, 1 / Z0, 1 / Z0, 1 / Z0], dtype=torch.complex128, device=dev)
    return complex(amplitude) * out * scale


def explicit_coordinates(spec, name):
    """A nonempty one-dimensional array of finite real coordinates (numbers, or a torch tensor on
    any device), as float64 on the host; anything else is refused, a complex value with a
    nonzero imaginary part included (results.py:47-69)."""
    if hasattr(spec, 'detach'):
        spec = spec.detach().cpu().numpy()
    try:
        arr = np.asarray(spec)
        usable = (arr.dtype.kind in 'biufc' and arr.ndim == 1 and arr.size > 0
                  and bool(np.all(np.isfinite(arr))) and not np.any(np.imag(arr)))
    except (TypeError, ValueError):
        usable = False
    if not usable:
        raise ValueError(f'{name} must be a positive integer count or a nonempty one-dimensional array of '
                         'finite real coordinates')
    return np.real(arr).astype(np.float64)


def axis_points(spec, extent, name):
    """A count spans ``[-extent/2, extent/2]`` inclusive; explicit coordinates are taken as
    given (field_result.py:85-106)."""
    if isinstance(spec, (int, np.integer)) and not isinstance(spec, bool):
        if spec < 1:
            raise ValueError(f'{name} must be a positive integer count')
        return np.linspace(-0.5, 0.5, int(spec)) * extent
    return explicit_coordinates(spec, name)


def height_points(spec, thickness_top_first):
    """Heights for a ``z`` request: explicit heights as given, with owners by face rule; a
    count gives every layer its own ``count`` heights from its bottom face to its top face, so
    an internal face appears twice, the lower layer's first (field_result.py:375-398)."""
    if isinstance(spec, (int, np.integer)) and not isinstance(spec, bool):
        if spec < 1:
            raise ValueError('z must be a positive integer count')
        ds = np.asarray(thickness_top_first, dtype=np.float64)[::-1]
        L = ds.shape[0]
        edges = np.concatenate([[0.0], np.cumsum(ds)])
        frac = np.linspace(0.0, 1.0, int(spec))
        z = np.concatenate([edges[j] + frac * ds[j] for j in range(L)])
        j = np.repeat(np.arange(L), int(spec))
        return z, L - 1 - j, ds[j] - (z - edges[j])
    z = explicit_coordinates(spec, 'z')
    owner, depth = heights(thickness_top_first, z)
    return z, owner, depth


def order_parity(hu, hv, device):
    """``(-1)^(m+n) = -1`` over the flattened orders ``i = n*n_u + m``: the sign between a
    coefficient about the cell corner and the same about its centre (field_result.py:672-679)."""
    m = np.arange(-hu, hu + 1)[None, :] + np.arange(-hv, hv + 1)[:, None]
    return torch.as_tensor(m.reshape(-1) % 2 == 1, device=device)


def incident_column(pv, pol):
    """The incident column ``(2N, 1)`` in the superstrate's port variables: ``a_s`` on the
    specular order's s entry, ``-i n_top a_p`` on its p entry."""
    N = pv['kx'].shape[0]
    C = torch.zeros((2 * N, 1), dtype=torch.complex128, device=pv['kx'].device)
    C[N // 2, 0] = complex(pol[0])
    C[N + N // 2, 0] = -1j * complex(pv['nt']) * complex(pol[1])
    return C


def build_state(modes, epz_i, thickness, wavelength, pv, pol, hu, hv, rasters=None, faces=None):
    """The :class:`FieldState` of one wavelength from its layers' ``(W, V, q)`` (Cartesian,
    entry face first), their corner-frame ``epz_i`` slots and the port vectors ``pv``; ``pol``
    is the source's ``(a_s, a_p)``. ``faces``: the incident column's amplitudes as
    ``wb_layer_amplitudes`` returns them for this solve, ``(plus, minus_top, minus_bottom)`` each
    (L, 2N, 1) and ``(cref, ctrn)`` each (2N, 1); without it the torch recursion computes them."""
    dev = pv['kx'].device
    k0 = 2 * math.pi / float(wavelength)
    if faces is None:
        amps, cref, ctrn = layer_amplitudes(modes, thickness, k0, pv, incident_column(pv, pol))
    else:
        ptop, mtop, mbot, cref, ctrn = faces
        amps = face_amplitudes([(ptop[l], mtop[l], mbot[l]) for l in range(len(modes))],
                               [q for _, _, q in modes], thickness, k0)
    rasters = rasters if rasters is not None else [None] * len(modes)
    layers = tuple(LayerState(W, V, q, float(d), e, plus[:, 0], minus[:, 0], r)
                   for (W, V, q), d, e, (plus, minus), r in zip(modes, thickness, epz_i, amps, rasters))
    odd = order_parity(hu, hv, dev)
    return FieldState(k0, pv['kx'], pv['ky'], odd, layers, boundary_spectra(pv, cref, ctrn, pol, odd))
