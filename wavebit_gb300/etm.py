"""The ETM connecting algorithm (``Numerics(algorithm='etm')``): the reference's enhanced
transmittance-matrix recursion (rcwa/_engine/solve_2d.py:2619-2843, the final matching of
rcwa/_engine/solve_1d.py:1389-1520) over the stage-B kernels' FP64 modes, as a cross-check of
the S-matrix cascade on the same modes. Batched torch linear algebra on the device that holds
the modes.

From the substrate up, per layer with rotated modes ``W``, ``V`` and ``X = exp(-k0 d q)``::

    a = (W^-1 F + V^-1 G) / 2,   b = (W^-1 F - V^-1 G) / 2
    Y = X b a^-1 X,   F = W (I + Y),   G = V (I - Y),   T = T a^-1 X

seeded with the substrate's ``F``, ``G`` and ``T = I``; one block solve of the superstrate's
boundary equations then gives ``R_s``, ``R_p`` and ``T_1``, and ``(T_s, T_p) = T T_1``. Real
in-plane wavevectors and passive layers, where the ETM's mode labels are ``mode_q``'s
(conventions.py:252-300) and every layer takes the plain form of ``_run_ab``; a finite gain
film too, whose answer does not depend on how its modes are labelled.
"""
import math

import torch

from .fields import sp_rotate

HALF_PI = math.pi / 2


def _diag(v):
    return torch.diag_embed(v)


def etm_solve(modes, thickness, k0, pv, pol, n_u, n_v, amplitudes=False):
    """Per-order efficiencies ``(R, T)``, each ``(3, n_v, n_u)`` for the given polarization,
    pure s and pure p, of one wavelength. ``modes``: ``(W, V, q)`` per layer, Cartesian, entry
    face first; ``pv``: the port vectors of :func:`wavebit_gb300.adjoint.ports`; ``pol``:
    ``(a_s, a_p)``. With ``amplitudes`` also the Fresnel amplitudes ``(3, 4, N)`` in the
    efficiency kernel's layout (column; r_s, r_p, t_s, t_p; order, about the cell corner): the
    final matching's p unknowns are ``-i n`` times the Fresnel p ratios."""
    kzt, kzb = pv['kzt'], pv['kzb']
    et, eb = complex(pv['et']), complex(pv['eb'])
    n_top = complex(pv['nt'])
    N = kzt.shape[0]
    dev, C = kzt.device, torch.complex128
    I = torch.eye(N, dtype=C, device=dev)
    O = torch.zeros((N, N), dtype=C, device=dev)
    I2 = torch.eye(2 * N, dtype=C, device=dev)
    F = torch.cat([torch.cat([I, O], 1), torch.cat([O, -1j * _diag(kzb) / eb], 1)], 0)
    G = torch.cat([torch.cat([-1j * _diag(kzb), O], 1), torch.cat([O, I], 1)], 0)
    T = I2
    for (W, V, q), d in reversed(list(zip(modes, thickness))):
        bW, bV = sp_rotate(W, V, pv['c'], pv['s'])
        WiF = torch.linalg.solve(bW, F)
        ViG = torch.linalg.solve(bV, G)
        a, b = 0.5 * (WiF + ViG), 0.5 * (WiF - ViG)
        a_i = torch.linalg.inv(a)
        X = torch.exp(-k0 * float(d) * q)
        Y = X[:, None] * (b @ a_i) * X[None, :]
        F, G = bW @ (I2 + Y), bV @ (I2 - Y)
        T = (T @ a_i) * X[None, :]
    kz_inc = kzt[N // 2]
    Kt = _diag(kzt)
    final_A = torch.cat([
        torch.cat([I, O, -F[:N, :N], -F[:N, N:]], 1),
        torch.cat([O, 1j * Kt / et, -F[N:, :N], -F[N:, N:]], 1),
        torch.cat([1j * Kt, O, -G[:N, :N], -G[:N, N:]], 1),
        torch.cat([O, I, -G[N:, :N], -G[N:, N:]], 1)], 0)
    e_p = n_top * kz_inc / et

    def column(a_s, a_p):
        col = torch.zeros(4 * N, dtype=C, device=dev)
        col[N // 2] = -a_s
        col[N + N // 2] = a_p * e_p
        col[2 * N + N // 2] = 1j * a_s * kz_inc
        col[3 * N + N // 2] = 1j * n_top * a_p
        return col

    pure_s = (complex(math.sin(HALF_PI)), complex(math.cos(HALF_PI)))
    pure_p = (complex(math.sin(0.0)), complex(math.cos(0.0)))
    cols = torch.stack([column(*pol), column(*pure_s), column(*pure_p)], 1)
    x = torch.linalg.solve(final_A, cols)
    Rs, Rp = x[:N], x[N:2 * N]
    Tt = T @ x[2 * N:]
    Ts, Tp = Tt[:N], Tt[N:]
    s_power = kz_inc.real
    p_power = abs(n_top) ** 2 * (kz_inc / et).real
    a_s, a_p = pol
    denom = torch.stack([abs(a_s) ** 2 * s_power + abs(a_p) ** 2 * p_power, s_power, p_power])[:, None]

    def power(amp, adm):
        return (amp * amp.conj()).real.T * adm.real[None, :]

    R = (power(Rs, kzt) + power(Rp, kzt / et)) / denom
    Tr = (power(Ts, kzb) + power(Tp, kzb / eb)) / denom
    if not amplitudes:
        return R.reshape(3, n_v, n_u), Tr.reshape(3, n_v, n_u)
    n_bot = complex(pv['nb'])
    amps = torch.stack([Rs, Rp / (-1j * n_top), Ts, Tp / (-1j * n_bot)]).permute(2, 0, 1)
    return R.reshape(3, n_v, n_u), Tr.reshape(3, n_v, n_u), amps
