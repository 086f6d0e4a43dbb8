"""Parity of the CUDA path (through the C ABI) against the CPU oracle and the reference fixtures."""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from oracle import rcwa_oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


def _engine():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300 import engine
    return engine


def _rast(rng, ny, nx):
    a = np.ones((ny, nx), complex)
    a[rng.random((ny, nx)) < 0.35] = 12.25
    a[rng.random((ny, nx)) < 0.1] = 4.0 + 0.5j
    return a


@pytest.mark.parametrize('ny,nx,hu,hv', [(16, 16, 2, 2), (12, 20, 3, 1), (1, 4, 10, 0), (33, 17, 4, 5)])
def test_assemble_matches_oracle(ny, nx, hu, hv):
    E = _engine()
    rng = np.random.default_rng(ny * 100 + nx)
    eps = np.stack([_rast(rng, ny, nx), np.full((ny, nx), -20 + 1.5j)])
    conv = E.assemble(torch.as_tensor(eps, device='cuda'), hu, hv)
    torch.cuda.synchronize()
    assert int(conv.status.item()) == 0
    for i in range(eps.shape[0]):
        want = O.li_conv(eps[i], hu, hv)
        for k, w in enumerate(want):
            got = conv.slot(k)[i].cpu().numpy()
            assert np.abs(got - w).max() <= 1e-12 * np.abs(w).max(), (i, k)


@pytest.mark.parametrize('hu,hv', [(2, 2), (3, 3), (5, 4)])
def test_layer_modes_are_eigenpairs(hu, hv):
    """Stage B: Omega^2 W = W diag(w) to round-off, eigenvalues equal LAPACK's as a set, q is
    mode_q(w) and V = Omega_R W / q."""
    E = _engine()
    rng = np.random.default_rng(hu * 10 + hv)
    eps = np.stack([_rast(rng, 20, 20), _rast(rng, 20, 20)])
    conv = E.assemble(torch.as_tensor(eps, device='cuda'), hu, hv)
    kx, ky = O.separable_kxy(700.0, (900.0, 1000.0), O.incident_kxy(0.3, 0.7, 1.0), hu, hv)
    kxg, kyg = O.order_grid(kx, ky)
    P = 2
    w, q, W, V, st = E.layer_modes(conv, [0, 1], np.tile(kxg.real, (P, 1)), np.tile(kyg.real, (P, 1)))
    torch.cuda.synchronize()
    assert not (st.cpu().numpy() & 2).any()
    for p in range(P):
        ex, ey, ez = (s[p].cpu().numpy() for s in (conv.epx, conv.epy, conv.epz_i))
        om2, om_r = O.layer_operator(kxg, kyg, ex, ey, ez)
        wn, Wn, qn, Vn = (t[p].cpu().numpy() for t in (w, W, q, V))
        res = np.linalg.norm(om2 @ Wn - Wn * wn[None, :]) / (np.linalg.norm(om2) * np.linalg.norm(Wn))
        assert res < 1e-13, res
        ref = np.linalg.eigvals(om2)
        # every eigenvalue has a LAPACK twin within round-off
        d = np.abs(wn[:, None] - ref[None, :]).min(axis=1)
        assert d.max() <= 1e-10 * np.abs(ref).max(), d.max()
        assert np.array_equal(qn, O.mode_q(wn)) or np.abs(qn - O.mode_q(wn)).max() < 1e-14 * np.abs(qn).max()
        assert np.abs(om_r @ Wn / qn[None, :] - Vn).max() <= 1e-11 * np.abs(Vn).max()


def _case(d, n):
    return {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(n + '__')}


REF_NAMES = list(np.load(os.path.join(GOLDEN, 'ref_cases.npz'))['names'])


def _solve_case(E, c, pol_pair):
    hu, hv = (int(v) for v in c['orders'])
    st = np.asarray(c['structure'], complex)
    L = st.shape[0]
    conv = E.assemble(torch.as_tensor(st, device='cuda'), hu, hv)
    inp = E.BatchInputs([list(range(L))], [list(c['thickness'])], [float(c['wavelength'])],
                        [list(c['period'])], [float(c['theta'])], [float(c['phi'])],
                        [complex(c['eps_top'])], [complex(c['eps_bot'])], [list(pol_pair)])
    R, T, status = E.solve_batch(conv, inp)
    torch.cuda.synchronize()
    return R[0].cpu().numpy(), T[0].cpu().numpy(), int(status[0].item())


@pytest.mark.parametrize('name', REF_NAMES)
def test_solve_matches_reference_fixtures(name):
    """Per-order R and T within 1e-10 (relative to the largest efficiency) of the reference's
    own rcwa.run, for s and p incidence."""
    E = _engine()
    c = _case(np.load(os.path.join(GOLDEN, 'ref_cases.npz')), name)
    R, T, st = _solve_case(E, c, O.polarization_pair('s'))
    assert st & ~8 == 0, st
    for col, pol in ((1, 's'), (2, 'p')):
        scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
        assert np.abs(R[col] - c[f'R_{pol}']).max() <= 1e-10 * scale, (name, pol)
        assert np.abs(T[col] - c[f'T_{pol}']).max() <= 1e-10 * scale, (name, pol)


def test_solve_host_matches_oracle():
    """The host-buffer entry (wb_solve_host): rasters in, efficiencies out."""
    E = _engine()
    rng = np.random.default_rng(11)
    eps = np.stack([_rast(rng, 16, 16), _rast(rng, 16, 16), np.full((16, 16), 2.25 + 0.1j)])
    B, hu, hv = 5, 3, 3
    wl = np.linspace(500, 900, B)
    li = np.tile(np.arange(3), (B, 1))
    th = np.tile([120.0, 200.0, 60.0], (B, 1))
    R, T, st = E.solve_host(eps, li, th, wl, np.tile([800.0, 900.0], (B, 1)), np.full(B, 0.25),
                            np.full(B, 0.4), np.ones(B), np.full(B, 2.25), np.tile([1.0, 0.0], (B, 1)),
                            hu, hv)
    assert (st & ~8 == 0).all()
    for b in range(B):
        o = O.solve_stack(eps, th[b], wl[b], (800.0, 900.0), hu, hv, 0.25, 0.4, 1.0, 2.25, 's')
        scale = max(np.abs(o['R']).max(), np.abs(o['T']).max())
        assert np.abs(R[b] - o['R']).max() <= 1e-10 * scale
        assert np.abs(T[b] - o['T']).max() <= 1e-10 * scale


@pytest.mark.parametrize('precision,tol', [('mixed', 1e-9), ('mixed_df64', 1e-9), ('mixed_df64_eig', 1e-9),
                                           ('mixed_fp32', 1e-5)])
def test_mixed_precision_within_tolerance(precision, tol):
    """The mixed forms against the FP64 oracle. 'mixed' (FP32 eigen-solve with Newton steps, FP32
    cascade refined against the double-float interface equations), 'mixed_df64' (double-float
    eigen-solve and cascade) and 'mixed_df64_eig' (double-float eigen-solve, refined FP32
    cascade) are held to 1e-9, far inside the 1e-6 target. 'mixed_fp32' (the FP32 cascade with
    no refinement) is held to 1e-5: it does not meet the 1e-6 target on every stack."""
    E = _engine()
    rng = np.random.default_rng(21)
    eps = np.stack([_rast(rng, 24, 24), _rast(rng, 24, 24), np.full((24, 24), -20 + 1.5j)])
    hu = hv = 4
    B = 6
    wl = np.linspace(450, 950, B)
    th = np.array([150.0, 230.0, 50.0])
    conv = E.assemble(torch.as_tensor(eps, device='cuda'), hu, hv)
    inp = E.BatchInputs(np.tile(np.arange(3), (B, 1)), np.tile(th, (B, 1)), wl, np.tile([900.0, 1000.0], (B, 1)),
                        np.full(B, 0.3), np.full(B, 0.2), np.ones(B), np.full(B, 2.25), np.tile([0.6, 0.8], (B, 1)))
    R, T, st = E.solve_batch(conv, inp, precision=precision)
    torch.cuda.synchronize()
    assert (st.cpu().numpy() & ~8 == 0).all()
    worst = 0.0
    for b in range(B):
        o = O.solve_stack(eps, th, wl[b], (900.0, 1000.0), hu, hv, 0.3, 0.2, 1.0, 2.25, (0.6, 0.8))
        worst = max(worst, np.abs(R[b].cpu().numpy() - o['R']).max(), np.abs(T[b].cpu().numpy() - o['T']).max())
    assert worst <= tol, worst


@pytest.mark.parametrize('precision', ['double', 'mixed'])
def test_layer_modes_every_pair_of_a_multi_wave_batch(precision):
    """Pairs that start in later waves of CTAs (six pairs per SM) are eigenpairs like the first
    wave's: a CTA whose warps read a value another thread had already overwritten (the
    Householder alpha in the Hessenberg reduction) broke exactly those pairs."""
    E = _engine()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    rng = np.random.default_rng(11)
    eps = np.stack([_rast(rng, 24, 24) for _ in range(3)])
    hu = hv = 4
    conv = E.assemble(torch.as_tensor(eps, device='cuda'), hu, hv)
    kx, ky = O.separable_kxy(910.0, (1000.0, 1000.0), O.incident_kxy(0.0, 0.0, 1.0), hu, hv)
    kxg, kyg = O.order_grid(kx, ky)
    P = 6 * sms
    layer = [p % 3 for p in range(P)]
    w, q, W, V, st = E.layer_modes(conv, layer, np.tile(kxg.real, (P, 1)), np.tile(kyg.real, (P, 1)),
                                   precision=precision)
    torch.cuda.synchronize()
    assert not (st.cpu().numpy() & 6).any()
    res = torch.zeros(P, dtype=torch.float64, device='cuda')
    for l in range(3):
        om2, _ = O.layer_operator(kxg, kyg, *(s[l].cpu().numpy() for s in (conv.epx, conv.epy, conv.epz_i)))
        A = torch.as_tensor(om2, device='cuda')
        idx = torch.arange(l, P, 3, device='cuda')
        res[idx] = (A[None] @ W[idx] - W[idx] * w[idx][:, None, :]).abs().amax(dim=(1, 2)) / A.abs().max()
    bad = torch.nonzero(res > 1e-11).flatten().cpu().numpy()
    assert bad.size == 0, (bad[:10], float(res.max()))


def test_solve_batch_is_invariant_to_batch_position():
    """A batch of identical solves spanning several CTA waves returns the oracle's answer in every
    slot, bit for bit the same."""
    E = _engine()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    rng = np.random.default_rng(12)
    eps = np.stack([_rast(rng, 24, 24), _rast(rng, 24, 24)])
    hu = hv = 3
    th = np.array([180.0, 260.0])
    B = 3 * sms
    conv = E.assemble(torch.as_tensor(eps, device='cuda'), hu, hv)
    inp = E.BatchInputs([[0, 1]] * B, [th] * B, [905.0] * B, [[1000.0, 1000.0]] * B, [0.1] * B, [0.3] * B,
                        [1.0] * B, [2.25] * B, [[1.0, 0.0]] * B)
    R, T, st = E.solve_batch(conv, inp, precision='double')
    torch.cuda.synchronize()
    assert not (st.cpu().numpy() & ~8).any()
    R, T = R.cpu().numpy(), T.cpu().numpy()
    assert np.array_equal(R, np.broadcast_to(R[:1], R.shape)) and np.array_equal(T, np.broadcast_to(T[:1], T.shape))
    o = O.solve_stack(eps, th, 905.0, (1000.0, 1000.0), hu, hv, 0.1, 0.3, 1.0, 2.25, (1.0, 0.0))
    assert np.abs(R[0] - o['R']).max() <= 1e-10 and np.abs(T[0] - o['T']).max() <= 1e-10


@pytest.mark.parametrize('precision', ['mixed_df64', 'mixed'])
def test_layer_modes_double_float_eigenpairs(precision):
    """The double-float eigen-solve ('mixed_df64') and the FP32 eigen-solve refined by Newton steps
    ('mixed') return FP64-class eigenpairs."""
    E = _engine()
    rng = np.random.default_rng(5)
    eps = np.stack([_rast(rng, 20, 20)])
    hu = hv = 4
    conv = E.assemble(torch.as_tensor(eps, device='cuda'), hu, hv)
    kx, ky = O.separable_kxy(640.0, (900.0, 900.0), O.incident_kxy(0.2, 0.4, 1.0), hu, hv)
    kxg, kyg = O.order_grid(kx, ky)
    w, q, W, V, st = E.layer_modes(conv, [0], kxg.real[None], kyg.real[None], precision=precision)
    torch.cuda.synchronize()
    om2, _ = O.layer_operator(kxg, kyg, *(s[0].cpu().numpy() for s in (conv.epx, conv.epy, conv.epz_i)))
    wn, Wn = w[0].cpu().numpy(), W[0].cpu().numpy()
    res = np.linalg.norm(om2 @ Wn - Wn * wn[None, :]) / (np.linalg.norm(om2) * np.linalg.norm(Wn))
    assert res < 1e-12, res


@pytest.mark.parametrize('precision,tol', [('mixed', 1e-8), ('mixed_df64_eig', 1e-8)])
def test_double_float_form_survives_the_fp32_exponent_range(precision, tol):
    """Requests that once overflowed or underflowed the double-float (FP32-exponent) eigen-solve:
    nearly converged bulges of ~1e-25, metal layers, near-degenerate modes; the same requests
    through the FP32 + Newton eigen-solve. The result must be finite and equal to the FP64 one
    to 1e-8: both forms refine an FP32 cascade whose products run on the tensor cores as split
    TF32 products (a few FP32 ulps; the mixed forms' target is 1e-6)."""
    E = _engine()
    from wavebit_gb300.serving import _stream, _pol_pair
    reqs = _stream(128, 4.0, 5, [(5, 5), (8, 8)], 4)
    for r in (reqs[56], reqs[60], reqs[62], reqs[69]):
        conv = E.assemble(torch.as_tensor(r.eps, device='cuda'), *r.orders)
        L = r.eps.shape[0]
        inp = E.BatchInputs([list(range(L))], [r.thickness], [r.wavelength], [r.period], [r.theta], [r.phi],
                            [r.eps_top], [r.eps_bot], [_pol_pair(r.pol)])
        Rd, Td, sd = E.solve_batch(conv, inp, precision='double')
        Rm, Tm, sm = E.solve_batch(conv, inp, precision=precision)
        torch.cuda.synchronize()
        assert int(sd.item()) & ~8 == 0 and int(sm.item()) & ~8 == 0, (r.id, int(sm.item()))
        assert float((Rd - Rm).abs().max()) <= tol and float((Td - Tm).abs().max()) <= tol, r.id


@pytest.mark.parametrize('precision,tol', [('double', 1e-12), ('mixed', 1e-9)])
def test_smm_solve_from_layer_modes_matches_the_fused_solve(precision, tol):
    """Stage C alone (wb_smm_solve) on the modes of wb_layer_modes gives the fused solve's
    efficiencies: the seam through which eigenpairs kept on the device are reused."""
    E = _engine()
    from wavebit_gb300.adjoint import ports
    rng = np.random.default_rng(31)
    eps = np.stack([_rast(rng, 20, 20), _rast(rng, 20, 20), np.full((20, 20), 2.25 + 0.05j)])
    hu, hv, B, L = 3, 4, 5, 3
    wl = np.linspace(500, 900, B)
    th = np.array([120.0, 240.0, 60.0])
    period = (800.0, 900.0)
    conv = E.assemble(torch.as_tensor(eps, device='cuda'), hu, hv)
    inp = E.BatchInputs(np.tile(np.arange(L), (B, 1)), np.tile(th, (B, 1)), wl, np.tile(period, (B, 1)),
                        np.full(B, 0.3), np.full(B, 0.5), np.ones(B), np.full(B, 2.25), np.tile([0.6, 0.8], (B, 1)))
    R0, T0, st0 = E.solve_batch(conv, inp, precision='double')
    kx, ky = [], []
    for b in range(B):
        pv = ports(float(wl[b]), period, 0.3, 0.5, 1.0, 2.25, hu, hv, 'cpu')
        for _ in range(L):
            kx.append(pv['kx'].numpy()); ky.append(pv['ky'].numpy())
    w, q, W, V, st = E.layer_modes(conv, np.tile(np.arange(L), B), np.array(kx), np.array(ky))
    R, T, st2 = E.smm_solve(W, V, q, inp, hu, hv, precision=precision)
    torch.cuda.synchronize()
    assert not (st2.cpu().numpy() & ~8).any()
    assert float((R - R0).abs().max()) <= tol and float((T - T0).abs().max()) <= tol
