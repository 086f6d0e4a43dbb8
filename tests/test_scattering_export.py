"""The stack's scattering matrix (``Outputs(scattering=True)``): the cascade of published blocks
and its port checks on the CPU; the device export (wb_scattering_matrix) against the reference's
own ``result.scattering`` on a GPU."""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from oracle import rcwa_oracle as O
from wavebit_gb300 import rcwa

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
NAMES = list(np.load(os.path.join(GOLDEN, 'ref_scattering.npz'))['names'])


def _case(name):
    d = np.load(os.path.join(GOLDEN, 'ref_scattering.npz'))
    return {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(name + '__')}


def _oracle_matrix(st, th, wl, period, hu, hv, theta, phi, eps_top, eps_bot):
    """The oracle's published S of a stack with its ports, as torch tensors on the CPU."""
    o = O.solve_stack(st, th, wl, period, hu, hv, theta, phi, eps_top, eps_bot)
    blocks = [torch.as_tensor(b) for b in O.exported_scattering(o['S'], hu, hv)]
    kx, ky = O.order_grid(o['kx'], o['ky'])
    port = lambda eps: rcwa.Port(np.real(kx), np.real(ky), complex(np.sqrt(complex(eps))), 1.0, 'sp')
    return rcwa.ScatteringMatrix(*blocks, entry_port=port(eps_top), exit_port=port(eps_bot))


def _stack(seed=4):
    rng = np.random.default_rng(seed)
    st = np.where(rng.random((4, 10, 12)) < 0.4, 12.25 + 0.2j, 2.1).astype(complex)
    return st, np.array([120., 80., 200., 60.])


def test_cascade_of_two_pieces_is_the_whole_stack():
    """A stack cut in two and joined through any joint medium of the same k_par reproduces the
    joined stack's matrix (scattering.py:552-575): the joint is a basis, not a layer."""
    st, th = _stack()
    hu, hv, wl, per, theta, phi = 2, 1, 640., (700., 650.), 0.35, 0.6
    whole = _oracle_matrix(st, th, wl, per, hu, hv, theta, phi, 1.0, 2.25)
    for joint in (1.0, 2.25):
        # the same transverse wavevector on the far side of the joint
        th_b = float(np.arcsin(np.sin(theta) / np.sqrt(joint)))
        a = _oracle_matrix(st[:2], th[:2], wl, per, hu, hv, theta, phi, 1.0, joint)
        b = _oracle_matrix(st[2:], th[2:], wl, per, hu, hv, th_b, phi, joint, 2.25)
        ab = a.cascade(b)
        for x, y in zip(ab.blocks, whole.blocks):
            assert (x - y).abs().max() <= 1e-12 * max(1.0, float(y.abs().max()))
        assert ab.entry_port is a.entry_port and ab.exit_port is b.exit_port


def test_cascade_refuses_ports_that_do_not_meet():
    st, th = _stack()
    hu, hv, wl, per = 1, 1, 640., (700., 650.)
    a = _oracle_matrix(st[:2], th[:2], wl, per, hu, hv, 0.3, 0.0, 1.0, 1.0)
    th_b = float(np.arcsin(np.sin(0.3) / 1.5))                                     # the same k_par in eps 2.25
    b_index = _oracle_matrix(st[2:], th[2:], wl, per, hu, hv, th_b, 0.0, 2.25, 1.0)  # another joint medium
    b_kpar = _oracle_matrix(st[2:], th[2:], wl, per, hu, hv, 0.2, 0.0, 1.0, 1.0)     # another k_par
    with pytest.raises(ValueError, match='half-spaces'):
        a.cascade(b_index)
    with pytest.raises(ValueError, match='wavevectors'):
        a.cascade(b_kpar)
    with pytest.raises(ValueError, match='polarizations'):
        a.cascade(b_kpar._replace(entry_port=b_kpar.entry_port._replace(channel='te')))
    with pytest.raises(TypeError):
        a.cascade(a.blocks)


def test_the_matrix_is_only_there_when_requested():
    res = rcwa.Result(None, None, (None, None), (None, None), None, (), {})
    with pytest.raises(rcwa.UnsupportedFeatureError) as e:
        res.scattering
    assert e.value.code == 'outputs.unavailable' and e.value.path == 'outputs.scattering'


def test_both_outputs_resolve():
    p = rcwa.Problem(stack=rcwa.Stack(layers=(rcwa.Layer(thickness=10.0, epsilon=2.0),), period=(500., 500.)),
                     excitation=rcwa.Excitation(600.0, (rcwa.PlaneWave(polarization='s', amplitude=3.0),)),
                     outputs=rcwa.Outputs(fields=True, scattering=True))
    r = rcwa._resolve(p, rcwa.Numerics())
    assert r['amplitude'] == 3.0 and rcwa._wants_fields(p) and rcwa._wants_scattering(p)


def _stack_S(structure, thickness, wl, period, hu, hv, kinc, phi, eps_top, eps_bot):
    """The oracle cascade of solve_stack with the incident transverse wavevector given rather than
    derived from theta: the form the device's mirrored stack takes (its k_par fixed by the lit side)."""
    conv = O.to_conv_mat_raster_sampled(np.asarray(structure, complex), hu, hv)
    kx, ky = O.separable_kxy(wl, period, kinc, hu, hv)
    kxg, kyg = O.order_grid(kx, ky)
    N = kxg.shape[0]; k0 = 2 * np.pi / wl
    et, eb = np.complex128(eps_top), np.complex128(eps_bot)
    kpar = kxg ** 2 + kyg ** 2
    kzt, kzb = O.boundary_kz(et, kpar), O.boundary_kz(eb, kpar)
    y = O.gap_waves(kxg, kyg)
    I, Z = np.eye(N, dtype=complex), np.zeros((N, N), complex)
    Wt = np.block([[I, Z], [Z, -1j * np.diag(kzt) / et]]); Vt = np.block([[-1j * np.diag(kzt), Z], [Z, I]])
    Wb = np.block([[I, Z], [Z, -1j * np.diag(kzb) / eb]]); Vb = np.block([[-1j * np.diag(kzb), Z], [Z, I]])
    Wg = np.block([[I, Z], [Z, -1j * np.diag(y)]]); Vg = np.block([[-1j * np.diag(y), Z], [Z, I]])
    vphi = O.order_azimuth(kyg.reshape(ky.shape[0], kx.shape[0]), kxg.reshape(ky.shape[0], kx.shape[0]), phi)
    c, s = np.cos(vphi), np.sin(vphi)
    S = O.s_reflection(Wt, Vt, Wg, Vg)
    for i in range(len(structure)):
        W, V, q, w, _ = O.layer_modes_2d(kxg, kyg, conv[0][i], conv[1][i], conv[2][i])
        bW, bV = O.sp_modes_2d(W, V, c, s, N)
        A, B = O.ab_matrices(bW, bV, Wg, Vg)
        S = O.redheffer_star(S, O.s_layer(A, B, np.diag(np.exp(-k0 * thickness[i] * q))))
    return O.redheffer_star(S, O.s_transmission(Wb, Vb, Wg, Vg))



@pytest.mark.parametrize('name', NAMES)
def test_the_mirrored_stack_gives_the_far_side_blocks(name):
    """The construction wb_scattering_matrix uses for S22 and S12: the stack with its layers in
    reverse order and its half-spaces swapped, at the same transverse wavevector, lit from the
    former substrate -- its S11 and S21 are the stack's S22 and S12 (here against the reference's
    own blocks, complex and evanescent half-spaces included)."""
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    et, eb = complex(c['eps_top']), complex(c['eps_bot'])
    kinc = O.incident_kxy(float(c['theta']), float(c['phi']), et)
    mir = O.exported_scattering(_stack_S(c['structure'][::-1], c['thickness'][::-1], float(c['wavelength']),
                                         tuple(c['period']), hu, hv, kinc, float(c['phi']), eb, et), hu, hv)
    for got, key in ((mir[0], 'S22'), (mir[2], 'S12')):
        want = c[key]
        assert np.abs(got - want).max() <= 1e-12 * max(1.0, np.abs(want).max()), (name, key)


def _problem(c, **kw):
    st, th = np.asarray(c['structure'], complex), np.asarray(c['thickness'], float)
    layers = tuple(rcwa.Layer(thickness=float(t), epsilon=e) for e, t in zip(st[::-1], th[::-1]))
    return rcwa.Problem(units=rcwa.Units('nm'),
                        stack=rcwa.Stack(period=tuple(float(p) for p in c['period']),
                                         top=rcwa.Material(epsilon=complex(c['eps_top'])),
                                         bottom=rcwa.Material(epsilon=complex(c['eps_bot'])), layers=layers),
                        excitation=rcwa.Excitation(wavelength=kw.get('wavelength', float(c['wavelength'])), sources=(
                            rcwa.PlaneWave(polarization='s', theta=float(c['theta']), phi=float(c['phi'])),)),
                        outputs=rcwa.Outputs(scattering=True))


def _cuda():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')


@pytest.mark.gpu
@pytest.mark.parametrize('name', NAMES)
def test_exported_blocks_match_the_reference(name):
    """The four blocks from rcwa.run(..., Outputs(scattering=True)) against the reference's own
    result.scattering, within 1e-10 of max(1, |S|)."""
    _cuda()
    c = _case(name)
    hu, hv = (int(v) for v in c['orders'])
    res = rcwa.run(_problem(c), numerics=rcwa.Numerics(orders=(hu, hv)))
    (sm,) = res.scattering
    for blk, got in zip(('S11', 'S12', 'S21', 'S22'), sm.blocks):
        want = c[blk]
        got = got.cpu().numpy()
        assert np.abs(got - want).max() <= 1e-10 * max(1.0, np.abs(want).max()), (name, blk)
    # the published reading of the s block: S11 on the specular s column is r_s about the centre
    N = (2 * hu + 1) * (2 * hv + 1)
    assert sm.entry_port.channel == 'sp' and sm.S11.shape == (2 * N, 2 * N)


@pytest.mark.gpu
def test_device_pieces_cascade_to_the_device_whole():
    """Two stacks exported on the device and joined by cascade() equal the joined stack's own
    exported matrix; several wavelengths in one run each get their matrix."""
    _cuda()
    st, th = _stack(9)

    def prob(layers_st, layers_th, top, bot, theta):
        layers = tuple(rcwa.Layer(thickness=float(t), epsilon=e) for e, t in zip(layers_st[::-1], layers_th[::-1]))
        return rcwa.Problem(units=rcwa.Units('nm'),
                            stack=rcwa.Stack(period=(700., 650.), top=rcwa.Material(epsilon=top),
                                             bottom=rcwa.Material(epsilon=bot), layers=layers),
                            excitation=rcwa.Excitation(wavelength=(610.0, 655.0, 700.0), sources=(
                                rcwa.PlaneWave(polarization='p', theta=theta, phi=0.6),)),
                            outputs=rcwa.Outputs(scattering=True))
    num = rcwa.Numerics(orders=(2, 2))
    theta = 0.35
    whole = rcwa.run(prob(st, th, 1.0, 2.25, theta), numerics=num).scattering
    th_b = float(np.arcsin(np.sin(theta) / 1.5))
    top = rcwa.run(prob(st[:2], th[:2], 1.0, 2.25, theta), numerics=num).scattering
    bot = rcwa.run(prob(st[2:], th[2:], 2.25, 2.25, th_b), numerics=num).scattering
    assert len(whole) == 3
    for w, a, b in zip(whole, top, bot):
        ab = a.cascade(b)
        for x, y in zip(ab.blocks, w.blocks):
            assert (x - y).abs().max().item() <= 1e-11 * max(1.0, y.abs().max().item())
