"""Torch-facing functional layer over libwbgpu.so: stage A, stage B and whole batched solves.

Every function takes and returns CUDA tensors and runs on the current torch stream. Matrices
handed to or returned by the library are column-major; the helpers here present them in the
natural (row, column) orientation NumPy and the reference use.
"""
import numpy as np
import torch

from . import _lib


def n_orders(hu, hv):
    return (2 * hu + 1) * (2 * hv + 1)


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _c128(x, device):
    if isinstance(x, (list, tuple)):
        x = np.asarray(x, dtype=np.complex128)
    return torch.as_tensor(x, dtype=torch.complex128, device=device).contiguous()


def _f64(x, device):
    if isinstance(x, (list, tuple)):
        x = np.asarray(x, dtype=np.float64)
    return torch.as_tensor(x, dtype=torch.float64, device=device).contiguous()


class ConvStack:
    """Convolution matrices of a set of layers in the library layout ``(L, 3, N, N)``:
    slots ``epx, epy, epz_i``, each N x N column-major (rows ``i = n * n_u + m``)."""

    def __init__(self, buf, hu, hv, status=None):
        self.buf = buf
        self.hu, self.hv = hu, hv
        self.status = status

    @property
    def n_layers(self):
        return self.buf.shape[0]

    def slot(self, k):
        """``(L, N, N)`` view of slot k in natural orientation."""
        return self.buf[:, k].transpose(-1, -2)

    @property
    def epx(self):
        return self.slot(0)

    @property
    def epy(self):
        return self.slot(1)

    @property
    def epz_i(self):
        return self.slot(2)

    @classmethod
    def from_matrices(cls, epx, epy, epz_i, hu, hv):
        """Wrap natural-orientation ``(L, N, N)`` slots (e.g. the reference's corner frame)."""
        buf = torch.stack([epx, epy, epz_i], dim=1).transpose(-1, -2).contiguous()
        return cls(buf.to(torch.complex128), hu, hv)


def assemble(eps, hu, hv, handle=None, edges=None):
    """Stage A: Li-rule convolution matrices of ``eps`` (L, ny, nx) (wb_assemble_li).

    ``edges = (x_edges (L, nx), y_edges (L, ny))`` makes ``eps`` compressed cells with those
    block edges on the unit cell and the coefficients integrated (wb_assemble_li_integrated)."""
    L, ny, nx = (int(v) for v in eps.shape)
    if edges is not None:
        x_edges, y_edges = (np.asarray(e, dtype=np.float64) for e in edges)
        if x_edges.shape != (L, nx) or y_edges.shape != (L, ny):
            raise ValueError(f'edges must be ({L}, {nx}) and ({L}, {ny})')
        for e in (x_edges, y_edges):
            if not (np.all(np.diff(e, axis=1) > 0) and np.all(e[:, 0] > 0) and np.all(e[:, -1] == 1.0)):
                raise ValueError('block edges must increase from above 0 to exactly 1 along each row')
    eps = _c128(eps, 'cuda')
    N = n_orders(hu, hv)
    h = handle or _lib.handle(eps.device.index or 0)
    planes = torch.empty((3, L, N, N), dtype=torch.complex128, device=eps.device)
    status = torch.zeros(1, dtype=torch.int32, device=eps.device)
    if edges is None:
        _lib.check(h.lib.wb_assemble_li(h.h, eps.data_ptr(), L, ny, nx, hu, hv, planes[0].data_ptr(),
                                        planes[1].data_ptr(), planes[2].data_ptr(), status.data_ptr(),
                                        _stream()))
    else:
        xe, ye = _f64(x_edges, eps.device), _f64(y_edges, eps.device)
        _lib.check(h.lib.wb_assemble_li_integrated(h.h, eps.data_ptr(), L, ny, nx, xe.data_ptr(), ye.data_ptr(),
                                                   hu, hv, planes[0].data_ptr(), planes[1].data_ptr(),
                                                   planes[2].data_ptr(), status.data_ptr(), _stream()))
    return ConvStack(planes.transpose(0, 1).contiguous(), hu, hv, status)


def layer_modes(conv, pair_layer, kx, ky, precision='double', handle=None):
    """Stage B for ``P`` pairs: ``(w, q, W, V, status)`` with W, V in natural orientation."""
    dev = conv.buf.device
    hu, hv = conv.hu, conv.hv
    N = n_orders(hu, hv)
    n = 2 * N
    if not (torch.is_tensor(pair_layer) and pair_layer.is_cuda):
        pl = np.asarray(pair_layer.cpu() if torch.is_tensor(pair_layer) else pair_layer)
        if pl.size and (int(pl.min()) < 0 or int(pl.max()) >= conv.n_layers):
            raise ValueError(f'pair_layer spans {int(pl.min())}..{int(pl.max())}; the convolution stack holds '
                             f'{conv.n_layers} layers')
    pair_layer = torch.as_tensor(pair_layer, dtype=torch.int32, device=dev).contiguous()
    P = pair_layer.shape[0]
    kx = _f64(kx, dev).reshape(P, N)
    ky = _f64(ky, dev).reshape(P, N)
    w = torch.empty((P, n), dtype=torch.complex128, device=dev)
    q = torch.empty_like(w)
    W = torch.empty((P, n, n), dtype=torch.complex128, device=dev)
    V = torch.empty_like(W)
    status = torch.zeros(P, dtype=torch.int32, device=dev)
    h = handle or _lib.handle(dev.index or 0)
    _lib.check(h.lib.wb_layer_modes(h.h, P, hu, hv, conv.buf.data_ptr(), pair_layer.data_ptr(),
                                    kx.data_ptr(), ky.data_ptr(), w.data_ptr(), q.data_ptr(),
                                    W.data_ptr(), V.data_ptr(), status.data_ptr(),
                                    _lib.PRECISION[precision], _stream()))
    return w, q, W.transpose(-1, -2), V.transpose(-1, -2), status


class BatchInputs:
    """Per-solve parameters of one batch, as contiguous device tensors."""

    def __init__(self, layer_index, thickness, wavelength, period, theta, phi, eps_top, eps_bot, pol,
                 device='cuda'):
        # the range of the indices, read on the host while they are host data: the kernels index
        # the convolution stack with them, so solve_batch refuses a batch that would read past it
        if torch.is_tensor(layer_index) and layer_index.is_cuda:
            self.index_range = None
        else:
            li = np.asarray(layer_index.cpu() if torch.is_tensor(layer_index) else layer_index)
            self.index_range = (int(li.min()), int(li.max())) if li.size else None
        self.layer_index = torch.as_tensor(layer_index, dtype=torch.int32, device=device).contiguous()
        B, L = self.layer_index.shape
        self.B, self.L = B, L
        self.thickness = _f64(thickness, device).reshape(B, L)
        self.wavelength = _f64(wavelength, device).reshape(B)
        self.period = _f64(period, device).reshape(B, 2)
        self.theta = _f64(theta, device).reshape(B)
        self.phi = _f64(phi, device).reshape(B)
        self.eps_top = _c128(eps_top, device).reshape(B)
        self.eps_bot = _c128(eps_bot, device).reshape(B)
        self.pol = _c128(pol, device).reshape(B, 2)


def solve_batch(conv, inp, precision='double', amplitudes=False, handle=None, out=None):
    """Stages B and C for a batch (wb_solve_batch). Returns ``(R, T, status[, amps])`` with R, T
    of shape ``(B, 3, n_v, n_u)`` for [given polarization, pure s, pure p]."""
    dev = conv.buf.device
    hu, hv = conv.hu, conv.hv
    N = n_orders(hu, hv)
    B, L = inp.B, inp.L
    rng = getattr(inp, 'index_range', None)
    if rng is not None and (rng[0] < 0 or rng[1] >= conv.n_layers):
        raise ValueError(f'layer_index spans {rng[0]}..{rng[1]}; the convolution stack holds {conv.n_layers} layers')
    if out is None:
        R = torch.empty((B, 3, N), dtype=torch.float64, device=dev)
        T = torch.empty_like(R)
        status = torch.zeros(B, dtype=torch.int32, device=dev)
        amps = torch.empty((B, 3, 4, N), dtype=torch.complex128, device=dev) if amplitudes else None
    else:
        R, T, status, amps = out
    h = handle or _lib.handle(dev.index or 0)
    _lib.check(h.lib.wb_solve_batch(
        h.h, B, L, hu, hv, conv.buf.data_ptr(), inp.layer_index.data_ptr(), inp.thickness.data_ptr(),
        inp.wavelength.data_ptr(), inp.period.data_ptr(), inp.theta.data_ptr(), inp.phi.data_ptr(),
        inp.eps_top.data_ptr(), inp.eps_bot.data_ptr(), inp.pol.data_ptr(), R.data_ptr(),
        T.data_ptr(), amps.data_ptr() if amps is not None else None, status.data_ptr(),
        _lib.PRECISION[precision], _stream()))
    nu, nv = 2 * hu + 1, 2 * hv + 1
    res = (R.view(B, 3, nv, nu), T.view(B, 3, nv, nu), status)
    return res + ((amps,) if amplitudes else ())


def _check_modes(W, V, q, inp, hu, hv):
    """The kernels read B*L pairs of (2N, 2N) modes and (2N,) roots: refuse anything smaller."""
    n = 2 * n_orders(hu, hv)
    P = inp.B * inp.L
    if tuple(W.shape) != (P, n, n) or tuple(V.shape) != (P, n, n) or tuple(q.shape) != (P, n):
        raise ValueError(f'modes must be W, V ({P}, {n}, {n}) and q ({P}, {n}) for {inp.B} solves of {inp.L} '
                         f'layers at orders ({hu}, {hv}); got {tuple(W.shape)}, {tuple(V.shape)}, {tuple(q.shape)}')


def smm_solve(W, V, q, inp, hu, hv, precision='double', amplitudes=False, handle=None):
    """Stage C from given modes (wb_smm_solve). ``W, V`` (B*L, n, n) and ``q`` (B*L, n) in the
    natural orientation :func:`layer_modes` returns, pair ``p = b*L + l``; ``inp`` the batch's
    per-solve parameters (its ``layer_index`` is not used). Returns ``(R, T, status[, amps])``."""
    _check_modes(W, V, q, inp, hu, hv)
    dev = W.device
    N = n_orders(hu, hv)
    B, L = inp.B, inp.L
    Wc = W.transpose(-1, -2).contiguous()          # back to the column-major buffers of the ABI
    Vc = V.transpose(-1, -2).contiguous()
    qc = q.contiguous()
    R = torch.empty((B, 3, N), dtype=torch.float64, device=dev)
    T = torch.empty_like(R)
    status = torch.zeros(B, dtype=torch.int32, device=dev)
    amps = torch.empty((B, 3, 4, N), dtype=torch.complex128, device=dev) if amplitudes else None
    h = handle or _lib.handle(dev.index or 0)
    _lib.check(h.lib.wb_smm_solve(
        h.h, B, L, hu, hv, Wc.data_ptr(), Vc.data_ptr(), qc.data_ptr(), inp.thickness.data_ptr(),
        inp.wavelength.data_ptr(), inp.period.data_ptr(), inp.theta.data_ptr(), inp.phi.data_ptr(),
        inp.eps_top.data_ptr(), inp.eps_bot.data_ptr(), inp.pol.data_ptr(), R.data_ptr(), T.data_ptr(),
        amps.data_ptr() if amps is not None else None, status.data_ptr(), _lib.PRECISION[precision], _stream()))
    nu, nv = 2 * hu + 1, 2 * hv + 1
    res = (R.view(B, 3, nv, nu), T.view(B, 3, nv, nu), status)
    return res + ((amps,) if amplitudes else ())


def smm_solve_vjp(W, V, q, inp, hu, hv, g_R=None, g_T=None, handle=None):
    """Reverse of :func:`smm_solve` in the FP64 form (wb_smm_solve_vjp): from the cotangents of
    R and T (``(B, 3, N)`` or ``(B, 3, n_v, n_u)``, either may be None) the cotangents
    ``(g_W, g_V, g_q, g_thickness)`` of W, V (B*L, n, n, natural orientation), q (B*L, n) and the
    thicknesses (B, L). The cascade is recomputed on the device with its intermediates."""
    _check_modes(W, V, q, inp, hu, hv)
    dev = W.device
    N = n_orders(hu, hv)
    n = 2 * N
    B, L = inp.B, inp.L
    Wc = W.transpose(-1, -2).contiguous()
    Vc = V.transpose(-1, -2).contiguous()
    qc = q.contiguous()
    gR = None if g_R is None else _f64(g_R, dev).reshape(B, 3, N).contiguous()
    gT = None if g_T is None else _f64(g_T, dev).reshape(B, 3, N).contiguous()
    gW = torch.empty((B * L, n, n), dtype=torch.complex128, device=dev)
    gV = torch.empty_like(gW)
    gq = torch.empty((B * L, n), dtype=torch.complex128, device=dev)
    gth = torch.empty((B, L), dtype=torch.float64, device=dev)
    status = torch.zeros(B, dtype=torch.int32, device=dev)
    h = handle or _lib.handle(dev.index or 0)
    _lib.check(h.lib.wb_smm_solve_vjp(
        h.h, B, L, hu, hv, Wc.data_ptr(), Vc.data_ptr(), qc.data_ptr(), inp.thickness.data_ptr(),
        inp.wavelength.data_ptr(), inp.period.data_ptr(), inp.theta.data_ptr(), inp.phi.data_ptr(),
        inp.eps_top.data_ptr(), inp.eps_bot.data_ptr(), inp.pol.data_ptr(),
        gR.data_ptr() if gR is not None else None, gT.data_ptr() if gT is not None else None,
        gW.data_ptr(), gV.data_ptr(), gq.data_ptr(), gth.data_ptr(), status.data_ptr(), _stream()))
    return gW.transpose(-1, -2), gV.transpose(-1, -2), gq, gth, status


def layer_modes_vjp(conv, pair_layer, kx, ky, w, q, W, V, g_w=None, g_q=None, g_W=None, g_V=None, handle=None):
    """Reverse of :func:`layer_modes` (wb_layer_modes_vjp): the slot cotangents, summed over the
    pairs that read each layer, as a :class:`ConvStack` (``.slot(k)`` in natural orientation),
    and the per-pair status. W, V, g_W, g_V in natural orientation."""
    dev = conv.buf.device
    hu, hv = conv.hu, conv.hv
    N = n_orders(hu, hv)
    n = 2 * N
    pair_layer = torch.as_tensor(pair_layer, dtype=torch.int32, device=dev).contiguous()
    P = pair_layer.shape[0]
    pl = pair_layer.cpu().numpy()
    if P and (int(pl.min()) < 0 or int(pl.max()) >= conv.n_layers):
        raise ValueError(f'pair_layer spans {int(pl.min())}..{int(pl.max())}; the convolution stack holds '
                         f'{conv.n_layers} layers')
    kx = _f64(kx, dev).reshape(P, N)
    ky = _f64(ky, dev).reshape(P, N)
    wc, qc = w.contiguous(), q.contiguous()
    Wc = W.transpose(-1, -2).contiguous()
    Vc = V.transpose(-1, -2).contiguous()
    col = lambda t: None if t is None else t.transpose(-1, -2).contiguous()  # noqa: E731
    gWc, gVc = col(g_W), col(g_V)
    gwc = None if g_w is None else g_w.contiguous()
    gqc = None if g_q is None else g_q.contiguous()
    for t, shape in ((Wc, (P, n, n)), (Vc, (P, n, n)), (wc, (P, n)), (qc, (P, n)), (gWc, (P, n, n)),
                     (gVc, (P, n, n)), (gwc, (P, n)), (gqc, (P, n))):
        if t is not None and tuple(t.shape) != shape:
            raise ValueError(f'expected {shape}, got {tuple(t.shape)}')
    g = torch.empty((conv.n_layers, 3, N, N), dtype=torch.complex128, device=dev)
    status = torch.zeros(P, dtype=torch.int32, device=dev)
    ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    h = handle or _lib.handle(dev.index or 0)
    _lib.check(h.lib.wb_layer_modes_vjp(
        h.h, P, hu, hv, conv.n_layers, conv.buf.data_ptr(), pair_layer.data_ptr(), kx.data_ptr(), ky.data_ptr(),
        wc.data_ptr(), qc.data_ptr(), Wc.data_ptr(), Vc.data_ptr(), ptr(gwc), ptr(gqc), ptr(gWc), ptr(gVc),
        g.data_ptr(), status.data_ptr(), _stream()))
    return ConvStack(g, hu, hv), status


def assemble_vjp(eps, conv, g_conv, handle=None):
    """Reverse of :func:`assemble` with sampled coefficients (wb_assemble_li_vjp): the cotangent
    of the rasters ``eps`` (L, ny, nx) from the slot cotangents ``g_conv`` (a :class:`ConvStack`),
    given the forward's slots ``conv``. Returns a complex (L, ny, nx) tensor (for a real raster,
    its real part is the gradient)."""
    eps = _c128(eps, 'cuda')
    L, ny, nx = (int(v) for v in eps.shape)
    hu, hv = conv.hu, conv.hv
    epx = conv.buf[:, 0].contiguous()
    epz = conv.buf[:, 2].contiguous()
    g = [g_conv.buf[:, k].contiguous() for k in range(3)]
    g_eps = torch.empty((L, ny, nx), dtype=torch.complex128, device=eps.device)
    status = torch.zeros(1, dtype=torch.int32, device=eps.device)
    h = handle or _lib.handle(eps.device.index or 0)
    _lib.check(h.lib.wb_assemble_li_vjp(h.h, eps.data_ptr(), L, ny, nx, hu, hv, epx.data_ptr(), epz.data_ptr(),
                                        g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(), g_eps.data_ptr(),
                                        status.data_ptr(), _stream()))
    return g_eps


def etm_solve(W, V, q, inp, hu, hv, amplitudes=False, handle=None):
    """The ETM connecting algorithm from given modes (wb_etm_solve, FP64). ``W, V, q`` and
    ``inp`` as for :func:`smm_solve`. Returns ``(R, T, status[, amps])`` in its layout."""
    _check_modes(W, V, q, inp, hu, hv)
    dev = W.device
    N = n_orders(hu, hv)
    B, L = inp.B, inp.L
    Wc = W.transpose(-1, -2).contiguous()
    Vc = V.transpose(-1, -2).contiguous()
    qc = q.contiguous()
    R = torch.empty((B, 3, N), dtype=torch.float64, device=dev)
    T = torch.empty_like(R)
    status = torch.zeros(B, dtype=torch.int32, device=dev)
    amps = torch.empty((B, 3, 4, N), dtype=torch.complex128, device=dev) if amplitudes else None
    h = handle or _lib.handle(dev.index or 0)
    _lib.check(h.lib.wb_etm_solve(
        h.h, B, L, hu, hv, Wc.data_ptr(), Vc.data_ptr(), qc.data_ptr(), inp.thickness.data_ptr(),
        inp.wavelength.data_ptr(), inp.period.data_ptr(), inp.theta.data_ptr(), inp.phi.data_ptr(),
        inp.eps_top.data_ptr(), inp.eps_bot.data_ptr(), inp.pol.data_ptr(), R.data_ptr(), T.data_ptr(),
        amps.data_ptr() if amps is not None else None, status.data_ptr(), _stream()))
    nu, nv = 2 * hu + 1, 2 * hv + 1
    res = (R.view(B, 3, nv, nu), T.view(B, 3, nv, nu), status)
    return res + ((amps,) if amplitudes else ())


def layer_amplitudes(W, V, q, inp, hu, hv, C, handle=None):
    """Every layer's mode amplitudes for the incidence columns ``C`` (B, 2N, k) from given modes
    (wb_layer_amplitudes, FP64). ``W, V, q`` and ``inp`` as for :func:`smm_solve`. Returns
    ``(plus, minus_top, minus_bottom, cref, ctrn, status)``: the first three (B, L, 2N, k), the
    reflected and transmitted columns (B, 2N, k), in natural orientation."""
    _check_modes(W, V, q, inp, hu, hv)
    dev = W.device
    n = 2 * n_orders(hu, hv)
    B, L = inp.B, inp.L
    if C.dim() != 3 or C.shape[0] != B or C.shape[1] != n:
        raise ValueError(f'incidence columns of shape {tuple(C.shape)}, expected ({B}, {n}, k)')
    k = C.shape[2]
    Wc = W.transpose(-1, -2).contiguous()
    Vc = V.transpose(-1, -2).contiguous()
    qc = q.contiguous()
    Cc = C.to(device=dev, dtype=torch.complex128).transpose(-1, -2).contiguous()
    out = torch.empty((3, B, L, k, n), dtype=torch.complex128, device=dev)
    ends = torch.empty((2, B, k, n), dtype=torch.complex128, device=dev)
    status = torch.zeros(B, dtype=torch.int32, device=dev)
    h = handle or _lib.handle(dev.index or 0)
    _lib.check(h.lib.wb_layer_amplitudes(
        h.h, B, L, hu, hv, Wc.data_ptr(), Vc.data_ptr(), qc.data_ptr(), inp.thickness.data_ptr(),
        inp.wavelength.data_ptr(), inp.period.data_ptr(), inp.theta.data_ptr(), inp.phi.data_ptr(),
        inp.eps_top.data_ptr(), inp.eps_bot.data_ptr(), Cc.data_ptr(), k, out[0].data_ptr(), out[1].data_ptr(),
        out[2].data_ptr(), ends[0].data_ptr(), ends[1].data_ptr(), status.data_ptr(), _stream()))
    out = out.transpose(-1, -2)
    ends = ends.transpose(-1, -2)
    return out[0], out[1], out[2], ends[0], ends[1], status


def scattering_matrix(W, V, q, inp, hu, hv, handle=None):
    """The stack's scattering matrix at its half-space ports from given modes
    (wb_scattering_matrix). ``W, V, q`` and ``inp`` as for :func:`smm_solve`. Returns
    ``(S11, S12, S21, S22, status)``: each block ``(B, 2N, 2N)`` in natural orientation, s
    amplitudes then p port variables, about the cell centre."""
    _check_modes(W, V, q, inp, hu, hv)
    dev = W.device
    n = 2 * n_orders(hu, hv)
    B, L = inp.B, inp.L
    Wc = W.transpose(-1, -2).contiguous()
    Vc = V.transpose(-1, -2).contiguous()
    qc = q.contiguous()
    S = torch.empty((4, B, n, n), dtype=torch.complex128, device=dev)
    status = torch.zeros(B, dtype=torch.int32, device=dev)
    h = handle or _lib.handle(dev.index or 0)
    _lib.check(h.lib.wb_scattering_matrix(
        h.h, B, L, hu, hv, Wc.data_ptr(), Vc.data_ptr(), qc.data_ptr(), inp.thickness.data_ptr(),
        inp.wavelength.data_ptr(), inp.period.data_ptr(), inp.theta.data_ptr(), inp.phi.data_ptr(),
        inp.eps_top.data_ptr(), inp.eps_bot.data_ptr(), S[0].data_ptr(), S[1].data_ptr(), S[2].data_ptr(),
        S[3].data_ptr(), status.data_ptr(), _stream()))
    S = S.transpose(-1, -2)
    return S[0], S[1], S[2], S[3], status


def solve_host(eps, layer_index, thickness, wavelength, period, theta, phi, eps_top, eps_bot, pol,
               hu, hv, precision='double', handle=None, out=None):
    """Whole solve from host (NumPy) buffers through ``wb_solve_host``. ``out`` = (R, T, status)
    host arrays of shapes (B, 3, N), (B, 3, N), (B,) to write into (pinned ones make the copies
    asynchronous DMA); fresh arrays otherwise."""
    eps = np.ascontiguousarray(eps, dtype=np.complex128)
    L, ny, nx = eps.shape
    li = np.ascontiguousarray(layer_index, dtype=np.int32)
    B = li.shape[0]
    N = n_orders(hu, hv)
    arrs = dict(th=np.ascontiguousarray(thickness, np.float64).reshape(B, li.shape[1]),
                wl=np.ascontiguousarray(wavelength, np.float64).reshape(B),
                per=np.ascontiguousarray(period, np.float64).reshape(B, 2),
                theta=np.ascontiguousarray(theta, np.float64).reshape(B),
                phi=np.ascontiguousarray(phi, np.float64).reshape(B),
                et=np.ascontiguousarray(eps_top, np.complex128).reshape(B),
                eb=np.ascontiguousarray(eps_bot, np.complex128).reshape(B),
                pol=np.ascontiguousarray(pol, np.complex128).reshape(B, 2))
    if out is None:
        R = np.empty((B, 3, N), np.float64)
        T = np.empty((B, 3, N), np.float64)
        status = np.zeros(B, np.int32)
    else:
        R, T, status = out
        if (R.shape != (B, 3, N) or T.shape != (B, 3, N) or status.shape != (B,) or R.dtype != np.float64
                or T.dtype != np.float64 or status.dtype != np.int32 or not all(a.flags.c_contiguous for a in out)):
            raise ValueError('out must be C-contiguous (B, 3, N) float64, (B, 3, N) float64 and (B,) int32 arrays')
        status[...] = 0
    h = handle or _lib.handle(0)
    _lib.check(h.lib.wb_solve_host(
        h.h, B, li.shape[1], ny, nx, hu, hv, eps.ctypes.data, li.ctypes.data, arrs['th'].ctypes.data,
        arrs['wl'].ctypes.data, arrs['per'].ctypes.data, arrs['theta'].ctypes.data,
        arrs['phi'].ctypes.data, arrs['et'].ctypes.data, arrs['eb'].ctypes.data,
        arrs['pol'].ctypes.data, R.ctypes.data, T.ctypes.data, status.ctypes.data,
        _lib.PRECISION[precision]))
    nu, nv = 2 * hu + 1, 2 * hv + 1
    return R.reshape(B, 3, nv, nu), T.reshape(B, 3, nv, nu), status
