"""Pins the CPU oracle against the reference: fixtures made by the reference itself, the
reference's frozen legacy goldens, and RETICOLO's 2D Li-nesting totals."""
import os

import numpy as np
import pytest

from oracle import rcwa_oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


def _ref():
    return np.load(os.path.join(GOLDEN, 'ref_cases.npz'))


def _case(d, n):
    return {k.split('__', 1)[1]: d[k] for k in d.files if k.startswith(n + '__')}


REF_NAMES = list(np.load(os.path.join(GOLDEN, 'ref_cases.npz'))['names'])


@pytest.mark.parametrize('name', REF_NAMES)
def test_oracle_matches_reference_run(name):
    """Per-order R/T of the reference's public rcwa.run, both polarizations."""
    c = _case(_ref(), name)
    hu, hv = (int(v) for v in c['orders'])
    for k, pol in enumerate(('s', 'p')):
        out = O.solve_stack(c['structure'], c['thickness'], float(c['wavelength']),
                            tuple(c['period']), hu, hv, float(c['theta']), float(c['phi']),
                            complex(c['eps_top']), complex(c['eps_bot']), pol)
        R, T = out['R'][0], out['T'][0]
        scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
        assert np.abs(R - c[f'R_{pol}']).max() <= 1e-12 * scale, name
        assert np.abs(T - c[f'T_{pol}']).max() <= 1e-12 * scale, name
        # the pure s/p columns are the same numbers
        assert np.allclose(out['R'][1 + k], c[f'R_{pol}'], rtol=0, atol=1e-12 * scale)


@pytest.mark.parametrize('name', REF_NAMES)
def test_oracle_conv_matrices_match_reference_assemble(name):
    """Stage A slots against ``rcwa.operators.assemble`` (centre frame)."""
    c = _case(_ref(), name)
    if 'epx' not in c:
        pytest.skip('no stored slots for this case')
    hu, hv = (int(v) for v in c['orders'])
    epx, epy, epz_i = O.to_conv_mat_raster_sampled(c['structure'], hu, hv)
    for mine, theirs in ((epx, c['epx']), (epy, c['epy']), (epz_i, c['epz_i'])):
        for i in range(mine.shape[0]):
            got = O.swap_fourier_origin(mine[i], hu, hv)
            assert np.abs(got - theirs[i]).max() <= 1e-12 * np.abs(theirs[i]).max()


LEGACY_NAMES = list(np.load(os.path.join(GOLDEN, 'legacy_cases.npz'))['names'])


@pytest.mark.parametrize('name', LEGACY_NAMES)
def test_oracle_matches_legacy_goldens(name):
    """Frozen efficiencies of the reference's legacy golden file, at its own TOL = 1e-12."""
    d = np.load(os.path.join(GOLDEN, 'legacy_cases.npz'))
    c = _case(d, name)
    hu, hv = (int(v) for v in c['orders'])
    psi = float(c['psi'])
    out = O.solve_stack(np.asarray(c['structure'], complex), c['thickness'],
                        float(c['wavelength']), tuple(c['period']), hu, hv, float(c['theta']),
                        float(c['phi']), complex(c['top']), complex(c['bot']),
                        (np.sin(psi), np.cos(psi)))
    for col, sub in enumerate(('res', 'res_te_inc', 'res_tm_inc')):
        if f'{sub}__de_ri' not in c:
            continue
        want_r = np.asarray(c[f'{sub}__de_ri']).reshape(out['R'][col].shape)
        want_t = np.asarray(c[f'{sub}__de_ti']).reshape(out['T'][col].shape)
        assert np.abs(out['R'][col] - want_r).max() < 1e-12, (name, sub)
        assert np.abs(out['T'][col] - want_t).max() < 1e-12, (name, sub)


def test_toeplitz_tables_are_the_reference_convention():
    """``r - c + 2h`` row-major (factorization.py:276-286, :358-366), bit-exact."""
    for h in range(0, 6):
        got = O.toeplitz_positions(h).reshape(2 * h + 1, 2 * h + 1)
        for r in range(2 * h + 1):
            for c in range(2 * h + 1):
                assert got[r, c] == r - c + 2 * h
    assert list(O.order_labels(3)) == [-3, -2, -1, 0, 1, 2, 3]


def test_uniform_layer_is_exactly_eps_identity():
    """A uniform raster factorizes to exactly ``eps * I`` (test_factorization_core.py:927)."""
    eps = 4.0 + 0.5j
    epx, epy, epz_i = O.li_conv(np.full((7, 9), eps), 2, 3)
    N = epx.shape[0]
    assert np.array_equal(epx, eps * np.eye(N)) or np.abs(epx - eps * np.eye(N)).max() < 1e-15
    assert np.abs(epy - eps * np.eye(N)).max() < 1e-15
    assert np.abs(epz_i - np.eye(N) / eps).max() < 1e-15


@pytest.mark.parametrize('order,pol,want', [
    (3, 's', 0.9822061471), (3, 'p', 0.8913451356)])
def test_oracle_matches_reticolo_li_nesting(order, pol, want):
    """RETICOLO V10 totals for the 2D eps=6 rectangle under fixed nesting
    (tests/references/test_reticolo_li_nesting.py:34-41), TOL 1e-9."""
    n, period = 650, 325.0
    pixel = period / n
    x0, x1 = round((period - 200.0) / 2 / pixel), round((period + 200.0) / 2 / pixel)
    y0, y1 = round((period - 150.0) / 2 / pixel), round((period + 150.0) / 2 / pixel)
    eps = np.ones((1, n, n), complex)
    eps[0, y0:y1, x0:x1] = 6.0
    out = O.solve_stack(eps, np.array([600.0]), 532.0, (period, period), order, order,
                        0.0, 0.0, 1.0, 1.46 ** 2, pol)
    assert abs(out['T'][0].sum() - want) < 1e-9


def test_lossless_energy_balance():
    """R + T = 1 on a lossless stack (test_scattering_core.py:137)."""
    rng = np.random.default_rng(5)
    st = np.where(rng.random((2, 10, 10)) < 0.4, 12.25, 1.0).astype(complex)
    out = O.solve_stack(st, np.array([120.0, 200.0]), 640.0, (900., 800.), 3, 2, 0.3, 0.7,
                        1.0, 2.25, 'p')
    for col in range(3):
        assert abs(out['R'][col].sum() + out['T'][col].sum() - 1) < 1e-12


INTEGRATED_NAMES = list(np.load(os.path.join(GOLDEN, 'ref_integrated.npz'))['names'])


def _integrated():
    return np.load(os.path.join(GOLDEN, 'ref_integrated.npz'))


@pytest.mark.parametrize('name', INTEGRATED_NAMES)
def test_integrated_conv_matrices_match_reference_assemble(name):
    """Integrated (closed-form segment) slots against ``rcwa.operators.assemble`` with
    ``fourier_coefficients='integrated'`` (centre frame)."""
    c = _case(_integrated(), name)
    if 'epx' not in c:
        pytest.skip('no stored slots for this case')
    hu, hv = (int(v) for v in c['orders'])
    mine = O.to_conv_mat_raster_integrated(c['structure'], hu, hv)
    for m, theirs in zip(mine, (c['epx'], c['epy'], c['epz_i'])):
        for i in range(m.shape[0]):
            got = O.swap_fourier_origin(m[i], hu, hv)
            assert np.abs(got - theirs[i]).max() <= 1e-12 * np.abs(theirs[i]).max(), (name, i)


@pytest.mark.parametrize('name', INTEGRATED_NAMES)
def test_integrated_solve_matches_reference_run(name):
    """Per-order R and T of the oracle's solve on integrated slots against the reference's own
    ``rcwa.run`` with ``fourier_coefficients='integrated'``, for s and p."""
    c = _case(_integrated(), name)
    hu, hv = (int(v) for v in c['orders'])
    conv = O.to_conv_mat_raster_integrated(c['structure'], hu, hv)
    for pol in ('s', 'p'):
        o = O.solve_stack(c['structure'], c['thickness'], float(c['wavelength']), tuple(c['period']), hu, hv,
                          float(c['theta']), float(c['phi']), complex(c['eps_top']), complex(c['eps_bot']), pol,
                          conv=conv)
        scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
        assert np.abs(o['R'][0] - c[f'R_{pol}']).max() <= 1e-12 * scale, (name, pol)
        assert np.abs(o['T'][0] - c[f'T_{pol}']).max() <= 1e-12 * scale, (name, pol)


def test_integrated_coefficients_keep_a_uniform_layer_exact():
    """The jump form gives a uniform layer exactly eps * I (factorization.py:457-501)."""
    epx, epy, epz_i = O.li_conv_integrated(np.full((7, 5), 6.25 + 0.5j), 3, 2)
    N = 35
    assert np.array_equal(epx, (6.25 + 0.5j) * np.eye(N)) or np.abs(epx - (6.25 + 0.5j) * np.eye(N)).max() < 1e-15
    assert np.abs(epz_i - np.eye(N) / (6.25 + 0.5j)).max() < 1e-15


SCATTERING_NAMES = list(np.load(os.path.join(GOLDEN, 'ref_scattering.npz'))['names'])


@pytest.mark.parametrize('name', SCATTERING_NAMES)
def test_exported_scattering_matrix_matches_reference(name):
    """The four blocks of the stack's S at the half-space ports, about the cell centre, against
    the reference's ``result.scattering`` (``Outputs(scattering=True)``, scattering.py:482-605)."""
    c = _case(np.load(os.path.join(GOLDEN, 'ref_scattering.npz')), name)
    hu, hv = (int(v) for v in c['orders'])
    out = O.solve_stack(c['structure'], c['thickness'], float(c['wavelength']), tuple(c['period']), hu, hv,
                        float(c['theta']), float(c['phi']), complex(c['eps_top']), complex(c['eps_bot']), 's')
    mine = O.exported_scattering(out['S'], hu, hv)
    for blk, m in zip(('S11', 'S12', 'S21', 'S22'), mine):
        theirs = c[blk]
        assert np.abs(m - theirs).max() <= 1e-12 * max(1.0, np.abs(theirs).max()), (name, blk)
    # the readings the reference documents for the s block: S11 delta = r_s and S21 delta = t_s,
    # both referenced at the cell centre (the solve's own amplitudes are about the corner)
    N = (2 * hu + 1) * (2 * hv + 1)
    m = O.order_labels(hu)[None, :] + O.order_labels(hv)[:, None]
    d = np.where(m.reshape(-1) % 2 == 0, 1.0, -1.0)
    r_s, t_s = out['amps'][0][1].reshape(-1), out['amps'][2][1].reshape(-1)
    assert np.abs(mine[0][:N, N // 2] - d * r_s).max() <= 1e-13
    assert np.abs(mine[2][:N, N // 2] - d * t_s).max() <= 1e-13


FIELD_NAMES = list(np.load(os.path.join(GOLDEN, 'ref_fields.npz'))['names'])


@pytest.mark.parametrize('name', FIELD_NAMES)
def test_field_phasors_match_reference(name):
    """Collocated (Ex, Ey, Ez, Hx, Hy, Hz) at explicit points -- interior heights, internal faces
    (read in the layer above) and both outer faces -- against the reference's
    ``result.field(x=, y=, z=)`` (results.py:148-229), s and p incidence with a source amplitude.
    E and H are each held to 1e-12 of their own largest magnitude."""
    c = _case(np.load(os.path.join(GOLDEN, 'ref_fields.npz')), name)
    hu, hv = (int(v) for v in c['orders'])
    for pol in ('s', 'p'):
        got = O.field_phasors(c['structure'], c['thickness'], float(c['wavelength']), tuple(c['period']), hu, hv,
                              float(c['theta']), float(c['phi']), complex(c['eps_top']), complex(c['eps_bot']), pol,
                              float(c[f'amplitude_{pol}']), c['x'], c['y'], c['z'])
        want = c[f'field_{pol}'][0]
        for part in (slice(0, 3), slice(3, 6)):
            scale = np.abs(want[..., part]).max()
            assert np.abs(got[..., part] - want[..., part]).max() <= 1e-12 * scale, (name, pol, part)


ETM_NAMES = list(np.load(os.path.join(GOLDEN, 'ref_etm.npz'))['names'])


@pytest.mark.parametrize('name', ETM_NAMES)
def test_etm_matches_the_reference_etm_and_the_smm(name):
    """The oracle's ETM connecting algorithm against the reference's
    ``Numerics(algorithm='etm')`` run, and against the oracle's own SMM solve: the two connecting
    algorithms answer one question (solve_2d.py:2619-2843, scattering.py:1185-1456)."""
    c = _case(np.load(os.path.join(GOLDEN, 'ref_etm.npz')), name)
    hu, hv = (int(v) for v in c['orders'])
    args = (c['structure'], c['thickness'], float(c['wavelength']), tuple(c['period']), hu, hv,
            float(c['theta']), float(c['phi']), complex(c['eps_top']), complex(c['eps_bot']), 's')
    etm, smm = O.etm_stack(*args), O.solve_stack(*args)
    for col, pol in ((1, 's'), (2, 'p')):
        scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
        for key in ('R', 'T'):
            assert np.abs(etm[key][col] - c[f'{key}_{pol}']).max() <= 1e-12 * scale, (name, pol, key)
            assert np.abs(etm[key][col] - smm[key][col]).max() <= 1e-12 * scale, (name, pol, key)


RETICOLO_NAMES = list(np.load(os.path.join(GOLDEN, 'reticolo_cases.npz'))['names'])


def _reticolo_solve(c):
    h, per = int(c['h']), float(c['period'])
    o = O.solve_stack(np.asarray(c['structure'], complex), c['thickness'], float(c['wavelength']), (per, per), h, 0,
                      float(c['theta']), float(c['phi']), complex(c['top']), complex(c['bot']), str(c['pol']))
    return o['R'][0].ravel(), o['T'][0].ravel()


@pytest.mark.parametrize('name', RETICOLO_NAMES)
def test_oracle_matches_reticolo_orders(name):
    """Per-order efficiencies of twelve 1D gratings (TE/TM, oblique, quarter duty cycle, two
    layers, orders 30, conical) against RETICOLO (tests/references/test_reticolo_golden.py:115-135
    of the reference, atol 1e-11); every order RETICOLO did not report carries no power."""
    c = _case(np.load(os.path.join(GOLDEN, 'reticolo_cases.npz')), name)
    R, T = _reticolo_solve(c)
    for side, arr in (('ri', R), ('ti', T)):
        idx = c[f'idx_{side}']
        assert np.abs(arr[idx] - c[f'de_{side}']).max() < 1e-11, (name, side)
        assert np.abs(np.delete(arr, idx)).max(initial=0.0) < 1e-14, (name, side)


def _airy(eps1, eps2, eps3, kx, k0d, pol):
    """Specular R, T of a uniform slab by the thin-film (Airy) formulas, exp(-i w t):
    kz = sqrt(eps - kx^2) with Im kz >= 0; the p channel uses the admittance kz/eps."""
    kz = [np.sqrt(complex(e) - kx ** 2) for e in (eps1, eps2, eps3)]
    kz = [k if k.imag > 0 or (k.imag == 0 and k.real >= 0) else -k for k in kz]
    y = kz if pol == 's' else [k / e for k, e in zip(kz, (eps1, eps2, eps3))]
    r12, r23 = (y[0] - y[1]) / (y[0] + y[1]), (y[1] - y[2]) / (y[1] + y[2])
    t12, t23 = 2 * y[0] / (y[0] + y[1]), 2 * y[1] / (y[1] + y[2])
    ph = np.exp(1j * kz[1] * k0d)
    den = 1 + r12 * r23 * ph ** 2
    r, t = (r12 + r23 * ph ** 2) / den, t12 * t23 * ph / den
    if pol == 'p':       # t above transmits the H field; power goes with the admittance kz/eps
        return abs(r) ** 2, (y[2].real / y[0].real) * abs(t) ** 2
    return abs(r) ** 2, (kz[2].real / kz[0].real) * abs(t) ** 2


@pytest.mark.parametrize('eps2', [6.25, 2.1 + 0.4j, -8.0 + 1.2j])
@pytest.mark.parametrize('pol', ['s', 'p'])
def test_uniform_slab_is_the_airy_formula(eps2, pol):
    """A uniform layer at oblique incidence through the full 2D path (orders (2, 2)): the specular
    efficiencies are the thin-film formulas and every other order is empty
    (test_lossy_media.py, test_uniform_interfaces.py of the reference)."""
    eps1, eps3, theta, wl, d = 1.44, 2.25, 0.4, 633.0, 170.0
    st = np.full((1, 4, 4), eps2, dtype=complex)
    out = O.solve_stack(st, np.array([d]), wl, (400.0, 450.0), 2, 2, theta, 0.0, eps1, eps3, pol)
    kx = np.sqrt(eps1) * np.sin(theta)
    R, T = _airy(eps1, eps2, eps3, kx, 2 * np.pi / wl * d, pol)
    spec = (2, 2)
    assert abs(out['R'][0][spec] - R) < 1e-12 and abs(out['T'][0][spec] - T) < 1e-12
    for M in (out['R'][0], out['T'][0]):
        rest = M.copy()
        rest[spec] = 0.0
        assert np.abs(rest).max() < 1e-14


@pytest.mark.parametrize('pol', ['s', 'p'])
def test_a_y_invariant_grating_solves_alike_at_any_hv(pol):
    """1D == 2D on a y-invariant stack at phi = 0 (test_equivalence.py:79-102 of the reference):
    the ky = 0 row at orders (h, 2) is the (h, 0) solution, and the other rows are empty."""
    rng = np.random.default_rng(12)
    row = np.where(rng.random(16) < 0.45, 12.25 + 0.1j, 1.0)
    st = np.stack([np.tile(row, (6, 1)), np.tile(row[::-1], (6, 1))]).astype(complex)
    th = np.array([140.0, 90.0])
    a = O.solve_stack(st, th, 700.0, (800.0, 500.0), 6, 0, 0.3, 0.0, 1.0, 2.25, pol)
    b = O.solve_stack(st, th, 700.0, (800.0, 500.0), 6, 2, 0.3, 0.0, 1.0, 2.25, pol)
    for key in ('R', 'T'):
        assert np.abs(b[key][0][2] - a[key][0][0]).max() < 1e-12
        assert np.abs(np.delete(b[key][0], 2, axis=0)).max() < 1e-14


HALFSPACE_NAMES = list(np.load(os.path.join(GOLDEN, 'ref_halfspace.npz'))['names'])


@pytest.mark.parametrize('name', HALFSPACE_NAMES)
def test_oracle_matches_reference_half_space_branches(name):
    """A lossy and a metallic substrate, total internal reflection under a denser superstrate and
    a denser superstrate at an ordinary angle: per-order R/T against the reference's own run
    (the boundary kz on Maystre's cut, conventions.py:655-760), s and p, 1e-12."""
    c = _case(np.load(os.path.join(GOLDEN, 'ref_halfspace.npz')), name)
    hu, hv = (int(v) for v in c['orders'])
    o = O.solve_stack(c['structure'], c['thickness'], float(c['wavelength']), tuple(c['period']), hu, hv,
                      float(c['theta']), float(c['phi']), complex(c['eps_top']), complex(c['eps_bot']), 's')
    for col, pol in ((1, 's'), (2, 'p')):
        scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
        assert np.abs(o['R'][col] - c[f'R_{pol}']).max() <= 1e-12 * scale, (name, pol)
        assert np.abs(o['T'][col] - c[f'T_{pol}']).max() <= 1e-12 * scale, (name, pol)


BARE_NAMES = list(np.load(os.path.join(GOLDEN, 'ref_bare.npz'))['names'])


@pytest.mark.parametrize('name', BARE_NAMES)
def test_bare_interface_is_a_zero_thickness_layer_of_the_top_medium(name):
    """A stack with no layers against the reference's own run: the oracle through one
    zero-thickness layer of the superstrate, as the lifecycle resolves it (results.py:180-189)."""
    c = _case(np.load(os.path.join(GOLDEN, 'ref_bare.npz')), name)
    hu, hv = (int(v) for v in c['orders'])
    et = complex(c['eps_top'])
    o = O.solve_stack(np.full((1, 1, 1), et), np.array([0.0]), float(c['wavelength']), tuple(c['period']), hu, hv,
                      float(c['theta']), float(c['phi']), et, complex(c['eps_bot']), 's')
    for col, pol in ((1, 's'), (2, 'p')):
        scale = max(np.abs(c[f'R_{pol}']).max(), np.abs(c[f'T_{pol}']).max())
        assert np.abs(o['R'][col] - c[f'R_{pol}']).max() <= 1e-12 * scale, (name, pol)
        assert np.abs(o['T'][col] - c[f'T_{pol}']).max() <= 1e-12 * scale, (name, pol)


AMPLITUDE_NAMES = list(np.load(os.path.join(GOLDEN, 'ref_amplitudes.npz'))['names'])


@pytest.mark.parametrize('name', AMPLITUDE_NAMES)
def test_amplitude_ratios_match_the_reference(name):
    """outputs['reflected'|'transmitted'].amplitude_ratio_s/_p of the reference's own run, p and
    mixed (0.6, 0.8i) incidence: the oracle's Fresnel amplitudes about the cell centre."""
    c = _case(np.load(os.path.join(GOLDEN, 'ref_amplitudes.npz')), name)
    hu, hv = (int(v) for v in c['orders'])
    for tag, pol in (('p', 'p'), ('mix', (0.6, 0.8j))):
        o = O.solve_stack(c['structure'], c['thickness'], float(c['wavelength']), tuple(c['period']), hu, hv,
                          float(c['theta']), float(c['phi']), complex(c['eps_top']), complex(c['eps_bot']), pol)
        rs, rp, ts, tp = O.amplitude_ratios(o['amps'], hu, hv)
        for key, mine in (('reflected_s', rs), ('reflected_p', rp), ('transmitted_s', ts), ('transmitted_p', tp)):
            theirs = c[f'{tag}_{key}']
            assert np.abs(mine[0] - theirs).max() <= 1e-12 * max(1.0, np.abs(theirs).max()), (name, tag, key)


def test_quickstart_totals():
    """The reference README's quickstart (one 300 nm layer [[1, 1, 12.25, 12.25]], period 700 nm,
    eps_sub 2.25, orders (10, 0), normal s incidence at 900 nm): total R and T as the reference
    prints them, R = 0.2053316282584904 and T = 0.7946683717415131."""
    out = O.solve_stack(np.array([[[1.0, 1.0, 12.25, 12.25]]]), np.array([300.0]), 900.0, (700.0, 700.0), 10, 0,
                        0.0, 0.0, 1.0, 2.25, 's')
    assert abs(out['R'][0].sum() - 0.2053316282584904) < 1e-13
    assert abs(out['T'][0].sum() - 0.7946683717415131) < 1e-13
