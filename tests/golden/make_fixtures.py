"""Generate the golden fixtures in this folder from the reference implementation.

Run where the reference source tree is available (read-only), naming its root with
``--reference`` or the ``WAVEBIT_REFERENCE`` environment variable::

    PYTHONPATH=tests/golden/refshim python tests/golden/make_fixtures.py --reference <root>

It writes

* ``ref_cases.npz`` -- seeded small raster stacks solved by the reference's public
  ``rcwa.run`` (NumPy backend, SMM, sampled Li, fixed nesting): per-order R and T for ``'s'``
  and ``'p'`` incidence, and each layer's centre-frame convolution matrices from
  ``rcwa.operators.assemble``;
* ``ref_integrated.npz`` -- the same scenes (but the largest) with the integrated (closed-form
  segment) coefficients, ``fourier_coefficients='integrated'``;
* ``ref_scattering.npz`` -- the stack's exported scattering matrix (``Outputs(scattering=True)``)
  of five of those scenes and the five of ``ref_halfspace.npz``;
* ``ref_fields.npz`` -- collocated field phasors (``Outputs(fields=True)``, ``result.field``) of
  five of those scenes and two of ``ref_halfspace.npz`` (total internal reflection, a metallic
  substrate) at explicit points and counts, plain and Lalanne reconstruction, and the boundary
  fields on both faces, s and p incidence;
* ``ref_etm.npz`` -- per-order R/T of the reference's ETM connecting algorithm on the scenes of
  ``ref_cases.npz`` and ``ref_halfspace.npz``;
* ``ref_halfspace.npz`` -- per-order R/T of the reference's own run on scenes with a lossy or
  metallic substrate, total internal reflection, a denser superstrate, and normal incidence at
  an azimuth with cos(phi) < 0;
* ``ref_amplitudes.npz`` -- the reference's published amplitude ratios of the scenes of
  ``ref_cases.npz`` and ``ref_halfspace.npz`` (p and mixed incidence), and the other per-order
  readings (Cartesian ratios, powers, wavevectors, port references) of a run in micrometres with
  a 2.5 V/m source;
* ``ref_backside.npz`` -- scenes lit from below (``PlaneWave(side='bottom')``): R, T, every
  per-order reading, fields, boundary fields and the incidence-relative scattering matrix;
* ``ref_direct.npz`` -- runs with the incidence given as a wavevector (``PlaneWave(kx=, ky=)``)
  over two wavelengths, from either side;
* ``ref_bare.npz`` -- per-order R/T of the reference's own run on stacks with no layers;
* ``reticolo_cases.npz`` -- RETICOLO's per-order efficiencies of twelve 1D gratings (the
  reference's ``tests/references/golden_reticolo.npz``), lit from above and from below, with
  their inputs;
* ``legacy_cases.npz`` -- the efficiencies that the reference's own frozen legacy golden file
  (``tests/fixtures/legacy_rcwa/golden_legacy.npz``) holds for its 1D, conical and 2D sampled-Li
  cases, with the inputs those cases are defined by (``tests/fixtures/legacy_rcwa/gen_goldens.py``).

The refshim package is a minimal Array-API stand-in so that the reference imports without the
third-party ``array_api_compat``. Nothing at test time needs the reference: the tests read only
the npz files.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
#: the reference's source root (holding ``src/wavebit`` and its ``tests/``), set by
#: :func:`use_reference` from ``--reference`` or ``WAVEBIT_REFERENCE``
REF = None


def use_reference(argv=None):
    """Resolve the reference root from ``--reference PATH`` (or ``WAVEBIT_REFERENCE``) and put
    its ``src`` on the import path."""
    global REF
    argv = list(sys.argv[1:] if argv is None else argv)
    root = os.environ.get('WAVEBIT_REFERENCE')
    if '--reference' in argv:
        root = argv[argv.index('--reference') + 1]
    if not root or not os.path.isdir(os.path.join(root, 'src', 'wavebit')):
        raise SystemExit('name the reference source root with --reference PATH or WAVEBIT_REFERENCE')
    REF = root
    sys.path.insert(0, os.path.join(REF, 'src'))
    return REF


def _rast(rng, ny, nx, values=(12.25,), n_shapes=3, background=1.0):
    a = np.full((ny, nx), background, dtype=np.complex128)
    for _ in range(n_shapes):
        v = values[rng.integers(0, len(values))]
        if rng.random() < 0.5:
            y0, x0 = rng.integers(0, ny), rng.integers(0, nx)
            h, w = rng.integers(1, max(2, ny // 2)), rng.integers(1, max(2, nx // 2))
            a[y0:y0 + h, x0:x0 + w] = v
        else:
            cy, cx, r = rng.uniform(0, ny), rng.uniform(0, nx), rng.uniform(1, min(ny, nx) / 3)
            yy, xx = np.mgrid[0:ny, 0:nx]
            a[(yy + 0.5 - cy) ** 2 + (xx + 0.5 - cx) ** 2 < r * r] = v
    return a


def ref_cases():
    """Seeded scenes, listed in kernel order (entry layer first)."""
    rng = np.random.default_rng(20261203)
    cases = []
    # the 1D binary grating of the quickstart (orders (10, 0))
    cases.append(dict(name='grating_1d', structure=np.array([[[1., 1., 12.25, 12.25]]], complex),
                      thickness=[300.], wavelength=900., period=(700., 700.), orders=(10, 0),
                      theta=0.0, phi=0.0, eps_top=1.0, eps_bot=2.25))
    # crossed gratings: oblique, lossy, negative-eps uniform layer, rectangular cells
    specs = [
        (16, 16, 2, (3, 3), 0.0, 0.0, 700.),
        (16, 16, 2, (3, 3), 0.2, 0.3, 650.),
        (12, 20, 3, (2, 4), 0.4, 1.1, 830.),
        (24, 24, 1, (4, 4), 0.1, 2.5, 900.),
        (8, 8, 2, (2, 2), 0.6, 4.0, 480.),
        (32, 32, 4, (5, 5), 0.0, 0.0, 1000.),
    ]
    for k, (ny, nx, L, orders, theta, phi, wl) in enumerate(specs):
        layers = []
        for i in range(L):
            if i == L - 1 and L > 1:
                layers.append(np.full((ny, nx), -20 + 1.5j))
            else:
                layers.append(_rast(rng, ny, nx, values=(12.25, 2.25, 4.0 + 0.3j)))
        cases.append(dict(name=f'crossed_{k}', structure=np.stack(layers),
                          thickness=list(rng.uniform(100, 400, size=L)), wavelength=wl,
                          period=(1000., 1000. if k != 2 else 1200.), orders=orders,
                          theta=theta, phi=phi, eps_top=1.0, eps_bot=2.25))
    # a symmetric pillar at normal incidence: exactly degenerate mode pairs
    a = np.ones((20, 20), complex)
    a[5:15, 5:15] = 12.25
    cases.append(dict(name='symmetric_pillar', structure=a[None], thickness=[250.],
                      wavelength=760., period=(800., 800.), orders=(3, 3), theta=0.0, phi=0.0,
                      eps_top=1.0, eps_bot=2.25))
    return cases


def run_ref(case, pol, coefficients=None, algorithm='smm'):
    from wavebit import Material, Units, rcwa
    from wavebit.rcwa import operators
    st = case['structure'][::-1]          # public stacks list layers bottom to top
    th = list(case['thickness'])[::-1]
    layers = tuple(rcwa.Layer(thickness=float(t), epsilon=np.asarray(e)) for e, t in zip(st, th))
    prob = rcwa.Problem(
        units=Units(length='nm'),
        stack=rcwa.Stack(period=case['period'], top=Material(epsilon=case['eps_top']),
                         bottom=Material(epsilon=case['eps_bot']), layers=layers),
        excitation=rcwa.Excitation(wavelength=case['wavelength'], sources=(
            rcwa.PlaneWave(polarization=pol, theta=case['theta'], phi=case['phi']),)))
    num = rcwa.Numerics(orders=case['orders'], fourier_coefficients=coefficients, algorithm=algorithm)
    res = rcwa.run(prob, numerics=num)
    ops = operators.assemble(prob, numerics=rcwa.Numerics(orders=case['orders'], fourier_coefficients=coefficients))
    conv = ops.epsilon[0]
    return np.asarray(res.R)[0], np.asarray(res.T)[0], [np.asarray(c) for c in conv[:3]]


def make_ref_cases():
    out = {}
    names = []
    for case in ref_cases():
        n = case['name']
        names.append(n)
        for key in ('structure', 'thickness', 'wavelength', 'period', 'orders', 'theta', 'phi',
                    'eps_top', 'eps_bot'):
            out[f'{n}__{key}'] = np.asarray(case[key])
        for pol in ('s', 'p'):
            R, T, conv = run_ref(case, pol)
            out[f'{n}__R_{pol}'] = R
            out[f'{n}__T_{pol}'] = T
        # public order is bottom to top; store conv in kernel order (entry layer first),
        # only for the smaller cases to keep the fixture small
        if conv[0].shape[-1] <= 50:
            for slot, arr in zip(('epx', 'epy', 'epz_i'), conv):
                out[f'{n}__{slot}'] = arr[::-1]
    out['names'] = np.array(names)
    np.savez_compressed(os.path.join(HERE, 'ref_cases.npz'), **out)
    print('ref_cases.npz:', len(names), 'cases')


def make_integrated_cases():
    """The same scenes with the integrated (closed-form segment) coefficients."""
    out = {}
    names = []
    for case in ref_cases():
        if case['name'] == 'crossed_5':       # the largest scene; the others cover the path
            continue
        n = case['name']
        names.append(n)
        for key in ('structure', 'thickness', 'wavelength', 'period', 'orders', 'theta', 'phi',
                    'eps_top', 'eps_bot'):
            out[f'{n}__{key}'] = np.asarray(case[key])
        for pol in ('s', 'p'):
            R, T, conv = run_ref(case, pol, coefficients='integrated')
            out[f'{n}__R_{pol}'] = R
            out[f'{n}__T_{pol}'] = T
        if conv[0].shape[-1] <= 50:
            for slot, arr in zip(('epx', 'epy', 'epz_i'), conv):
                out[f'{n}__{slot}'] = arr[::-1]
    out['names'] = np.array(names)
    np.savez_compressed(os.path.join(HERE, 'ref_integrated.npz'), **out)
    print('ref_integrated.npz:', len(names), 'cases')


def make_scattering_cases():
    """The stack's scattering matrix (Outputs(scattering=True), scattering.py:482-560) of a few
    small scenes: S11, S12, S21, S22 at the half-space ports, about the cell centre."""
    from wavebit import Material, Units, rcwa
    out = {}
    names = []
    scenes = [c for c in ref_cases() if c['name'] in ('grating_1d', 'crossed_0', 'crossed_1', 'crossed_4',
                                                         'symmetric_pillar')] + halfspace_cases()
    for case in scenes:
        n = case['name']
        names.append(n)
        for key in ('structure', 'thickness', 'wavelength', 'period', 'orders', 'theta', 'phi',
                    'eps_top', 'eps_bot'):
            out[f'{n}__{key}'] = np.asarray(case[key])
        st = case['structure'][::-1]
        th = list(case['thickness'])[::-1]
        layers = tuple(rcwa.Layer(thickness=float(t), epsilon=np.asarray(e)) for e, t in zip(st, th))
        prob = rcwa.Problem(
            units=Units(length='nm'),
            stack=rcwa.Stack(period=case['period'], top=Material(epsilon=case['eps_top']),
                             bottom=Material(epsilon=case['eps_bot']), layers=layers),
            excitation=rcwa.Excitation(wavelength=case['wavelength'], sources=(
                rcwa.PlaneWave(polarization='s', theta=case['theta'], phi=case['phi']),)),
            outputs=rcwa.Outputs(scattering=True))
        res = rcwa.run(prob, numerics=rcwa.Numerics(orders=case['orders']))
        sm = res.scattering[0]
        for blk in ('S11', 'S12', 'S21', 'S22'):
            out[f'{n}__{blk}'] = np.asarray(getattr(sm, blk))
    out['names'] = np.array(names)
    np.savez_compressed(os.path.join(HERE, 'ref_scattering.npz'), **out)
    print('ref_scattering.npz:', len(names), 'cases')


def make_field_cases():
    """Collocated field phasors (``Outputs(fields=True)``, ``result.field(x=, y=, z=)``,
    results.py:148-229) of a few small scenes at explicit points: interior heights, an internal
    face and both outer faces; ``x``, ``y`` from the cell centre."""
    from wavebit import Material, Units, rcwa
    out = {}
    names = []
    scenes = [c for c in ref_cases() if c['name'] in ('grating_1d', 'crossed_0', 'crossed_1', 'crossed_4',
                                                         'symmetric_pillar')]
    scenes += [c for c in halfspace_cases() if c['name'] in ('tir', 'metal_substrate')]
    for case in scenes:
        n = case['name']
        names.append(n)
        for key in ('structure', 'thickness', 'wavelength', 'period', 'orders', 'theta', 'phi',
                    'eps_top', 'eps_bot'):
            out[f'{n}__{key}'] = np.asarray(case[key])
        st = case['structure'][::-1]
        th = np.asarray(case['thickness'], dtype=float)[::-1]
        total = float(th.sum())
        layers = tuple(rcwa.Layer(thickness=float(t), epsilon=np.asarray(e)) for e, t in zip(st, th))
        px, py = (float(v) for v in case['period'])
        x = np.array([-0.31 * px, 0.0, 0.12 * px, 0.45 * px])
        y = np.array([-0.27 * py, 0.08 * py, 0.5 * py])
        faces = np.concatenate([[0.0], np.cumsum(th)])
        z = np.unique(np.concatenate([faces, faces[:-1] + 0.37 * th, faces[:-1] + 0.81 * th]))
        for pol, amp in (('s', 1.0), ('p', 2.5)):
            prob = rcwa.Problem(
                units=Units(length='nm'),
                stack=rcwa.Stack(period=case['period'], top=Material(epsilon=case['eps_top']),
                                 bottom=Material(epsilon=case['eps_bot']), layers=layers),
                excitation=rcwa.Excitation(wavelength=case['wavelength'], sources=(
                    rcwa.PlaneWave(polarization=pol, theta=case['theta'], phi=case['phi'], amplitude=amp),)),
                outputs=rcwa.Outputs(fields=True))
            res = rcwa.run(prob, numerics=rcwa.Numerics(orders=case['orders']))
            f = res.field(x=x, y=y, z=z)
            out[f'{n}__field_{pol}'] = np.asarray(f.values)
            out[f'{n}__amplitude_{pol}'] = np.asarray(amp)
            # counts: a centred grid in x and y, each layer's own heights face to face in z
            fc = res.field(x=3, y=2, z=3)
            out[f'{n}__field_counts_{pol}'] = np.asarray(fc.values)
            out[f'{n}__counts_z_{pol}'] = np.asarray(fc.coordinates['z'])
            # Lalanne's rule: E_x, E_y of patterned layers from the D series line by line
            fl = res.field(x=x, y=y, z=z, reconstruction='lalanne')
            out[f'{n}__field_lalanne_{pol}'] = np.asarray(fl.values)
            # and at counts, whose x samples sit on the cell's two edges
            out[f'{n}__field_counts_lalanne_{pol}'] = np.asarray(
                res.field(x=3, y=2, z=3, reconstruction='lalanne').values)
            # the half-spaces' waves on the two faces (results.py:231-265)
            for side in ('top', 'bottom'):
                for part in ('incoming', 'outgoing', 'total'):
                    b = res.boundary_fields(side=side, x=x, y=y, part=part)
                    out[f'{n}__boundary_{side}_{part}_{pol}'] = np.asarray(b.values)
        out[f'{n}__x'], out[f'{n}__y'], out[f'{n}__z'] = x, y, z
        out[f'{n}__total'] = np.asarray(total)
    out['names'] = np.array(names)
    np.savez_compressed(os.path.join(HERE, 'ref_fields.npz'), **out)
    print('ref_fields.npz:', len(names), 'cases')


def make_etm_cases():
    """Per-order R and T of the reference's ETM connecting algorithm (``Numerics(algorithm='etm')``,
    solve_2d.py:2619-2843) on the reference scenes, s and p incidence."""
    out = {}
    names = []
    for case in ref_cases() + halfspace_cases():
        n = case['name']
        names.append(n)
        for key in ('structure', 'thickness', 'wavelength', 'period', 'orders', 'theta', 'phi',
                    'eps_top', 'eps_bot'):
            out[f'{n}__{key}'] = np.asarray(case[key])
        for pol in ('s', 'p'):
            R, T, _ = run_ref(case, pol, algorithm='etm')
            out[f'{n}__R_{pol}'] = R
            out[f'{n}__T_{pol}'] = T
    out['names'] = np.array(names)
    np.savez_compressed(os.path.join(HERE, 'ref_etm.npz'), **out)
    print('ref_etm.npz:', len(names), 'cases')


def make_legacy_cases():
    """Efficiencies from the reference's frozen legacy golden file, with their inputs."""
    gold = np.load(os.path.join(REF, 'tests/fixtures/legacy_rcwa/golden_legacy.npz'))

    def rand(shape, seed):   # gen_goldens.py: an index raster drawn and squared to permittivity
        return np.random.default_rng(seed).uniform(1.0, 4.0, size=shape) ** 2

    # Inputs as in tests/fixtures/legacy_rcwa/gen_goldens.py CASES (layers listed top to bottom).
    cases = {
        'te_1layer': dict(psi=np.pi / 2, phi=0.0, structure=[[[9., 9., 9., 1., 1., 1.]]], thickness=[0.15], top=4., bot=1., theta=0., orders=[6, 0], period=[0.77, 0.77], wavelength=0.777),
        'tm_1layer': dict(psi=0.0, phi=0.0, structure=[[[9., 9., 9., 1., 1., 1.]]], thickness=[0.15], top=4., bot=1., theta=0., orders=[6, 0], period=[0.77, 0.77], wavelength=0.777),
        'te_oblique': dict(psi=np.pi / 2, phi=0.0, structure=[[[9., 9., 9., 1., 1., 1.]]], thickness=[0.2], top=1., bot=2.25, theta=0.3, orders=[6, 0], period=[0.77, 0.77], wavelength=0.777),
        'tm_oblique': dict(psi=0.0, phi=0.0, structure=[[[9., 9., 9., 1., 1., 1.]]], thickness=[0.2], top=1., bot=2.25, theta=0.3, orders=[6, 0], period=[0.77, 0.77], wavelength=0.777),
        'te_2layer': dict(psi=np.pi / 2, phi=0.0, structure=[[[9., 9., 1., 1., 9., 1.]], [[4., 4., 4., 1., 1., 1.]]], thickness=[0.15, 0.22], top=1., bot=1., theta=0., orders=[5, 0], period=[0.7, 0.7], wavelength=0.9),
        'conical': dict(psi=0.4, phi=0.3, structure=[[[9., 9., 9., 1., 1., 1.]]], thickness=[0.15], top=4., bot=1., theta=0.2, orders=[6, 0], period=[0.77, 0.77], wavelength=0.777),
        'conical_2l': dict(psi=1.1, phi=0.5, structure=[[[9., 9., 1., 1., 9., 1.]], [[4., 4., 4., 1., 1., 1.]]], thickness=[0.15, 0.22], top=1., bot=2.25, theta=0.3, orders=[5, 0], period=[0.7, 0.7], wavelength=0.9),
        '2d_normal': dict(psi=0., phi=0., structure=rand((1, 5, 5), 0), thickness=[0.2], top=1., bot=1., theta=0., orders=[2, 2], period=[1., 1.], wavelength=0.9),
        '2d_oblique': dict(psi=0.9, phi=0.4, structure=rand((1, 6, 6), 1), thickness=[0.3], top=1., bot=2.25, theta=0.3, orders=[2, 2], period=[1., 1.2], wavelength=0.8),
        '2d_2layer': dict(psi=1.1, phi=0.5, structure=rand((2, 4, 4), 2), thickness=[0.15, 0.22], top=1.44, bot=1., theta=0.2, orders=[2, 2], period=[0.9, 0.9], wavelength=0.7),
    }
    out = {}
    for name, kw in cases.items():
        for key, val in kw.items():
            out[f'{name}__{key}'] = np.asarray(val)
        for sub in ('res', 'res_te_inc', 'res_tm_inc'):
            for f in ('de_ri', 'de_ti'):
                key = f'{name}__{sub}__{f}'
                if key in gold.files:
                    out[key] = np.asarray(gold[key])
    out['names'] = np.array(list(cases))
    np.savez_compressed(os.path.join(HERE, 'legacy_cases.npz'), **out)
    print('legacy_cases.npz:', len(cases), 'cases')


def halfspace_cases():
    """Scenes on the other branches of the boundary kz -- a lossy and a metallic substrate, total
    internal reflection under a denser superstrate (theta beyond the critical angle into eps 1), a
    denser superstrate at an ordinary angle -- and of the order azimuth: normal incidence with
    cos(phi) < 0, where the specular order's s/p frame is atan(sin phi / cos phi) + pi."""
    rng = np.random.default_rng(20261204)
    base = dict(thickness=[180., 90.], wavelength=720., period=(900., 800.), orders=(3, 2))

    def stack():
        return np.stack([_rast(rng, 12, 14, values=(12.25, 2.25, 4.0 + 0.3j)), np.full((12, 14), 2.1 + 0j)])
    return [
        dict(base, name='lossy_substrate', structure=stack(), theta=0.3, phi=0.4, eps_top=1.0, eps_bot=2.1 + 0.3j),
        dict(base, name='metal_substrate', structure=stack(), theta=0.2, phi=1.2, eps_top=1.0, eps_bot=-20.0 + 1.5j),
        dict(base, name='tir', structure=stack(), theta=0.8, phi=0.5, eps_top=2.25, eps_bot=1.0),
        dict(base, name='dense_superstrate', structure=stack(), theta=0.35, phi=2.2, eps_top=2.25, eps_bot=1.44),
        dict(base, name='normal_rotated', structure=stack(), theta=0.0, phi=2.5, eps_top=1.0, eps_bot=2.25),
    ]


def make_halfspace_cases():
    """Per-order R/T of the reference's own run on :func:`halfspace_cases`, s and p."""
    out = {}
    names = []
    for case in halfspace_cases():
        n = case['name']
        names.append(n)
        for key in ('structure', 'thickness', 'wavelength', 'period', 'orders', 'theta', 'phi',
                    'eps_top', 'eps_bot'):
            out[f'{n}__{key}'] = np.asarray(case[key])
        for pol in ('s', 'p'):
            R, T, _ = run_ref(case, pol)
            out[f'{n}__R_{pol}'] = R
            out[f'{n}__T_{pol}'] = T
    out['names'] = np.array(names)
    np.savez_compressed(os.path.join(HERE, 'ref_halfspace.npz'), **out)
    print('ref_halfspace.npz:', len(names), 'cases')


def make_amplitude_cases():
    """The reference's published amplitude ratios (outputs['reflected'|'transmitted']
    .amplitude_ratio_s/_p, results.py:357-390) of the reference scenes under p-polarised and
    mixed (s, p) incidence."""
    from wavebit import Material, Units, rcwa
    out = {}
    names = []
    for case in ref_cases() + halfspace_cases():
        n = case['name']
        names.append(n)
        for key in ('structure', 'thickness', 'wavelength', 'period', 'orders', 'theta', 'phi',
                    'eps_top', 'eps_bot'):
            out[f'{n}__{key}'] = np.asarray(case[key])
        st = case['structure'][::-1]
        th = list(case['thickness'])[::-1]
        layers = tuple(rcwa.Layer(thickness=float(t), epsilon=np.asarray(e)) for e, t in zip(st, th))
        for tag, pol in (('p', 'p'), ('mix', (0.6, 0.8j))):
            prob = rcwa.Problem(
                units=Units(length='nm'),
                stack=rcwa.Stack(period=case['period'], top=Material(epsilon=case['eps_top']),
                                 bottom=Material(epsilon=case['eps_bot']), layers=layers),
                excitation=rcwa.Excitation(wavelength=case['wavelength'], sources=(
                    rcwa.PlaneWave(polarization=pol, theta=case['theta'], phi=case['phi']),)))
            res = rcwa.run(prob, numerics=rcwa.Numerics(orders=case['orders']))
            for port in ('reflected', 'transmitted'):
                o = res.outputs[port]
                out[f'{n}__{tag}_{port}_s'] = np.asarray(o.amplitude_ratio_s)[0]
                out[f'{n}__{tag}_{port}_p'] = np.asarray(o.amplitude_ratio_p)[0]
            # the other per-order readings, with a 2.5 V/m source in micrometres (power scales
            # with |amplitude|^2 and the cell measure with the length unit)
            prob_um = rcwa.Problem(
                units=Units(length='um'),
                stack=rcwa.Stack(period=tuple(p / 1000 for p in case['period']),
                                 top=Material(epsilon=case['eps_top']), bottom=Material(epsilon=case['eps_bot']),
                                 layers=tuple(rcwa.Layer(thickness=float(t) / 1000, epsilon=np.asarray(e))
                                              for e, t in zip(st, th))),
                excitation=rcwa.Excitation(wavelength=case['wavelength'] / 1000, sources=(
                    rcwa.PlaneWave(polarization=pol, theta=case['theta'], phi=case['phi'], amplitude=2.5),)))
            res = rcwa.run(prob_um, numerics=rcwa.Numerics(orders=case['orders']))
            for port in ('reflected', 'transmitted'):
                o = res.outputs[port]
                for key in ('amplitude_ratio_xyz', 'power', 'k_parallel', 'k_normal', 'efficiency'):
                    out[f'{n}__{tag}_{port}_{key}'] = np.asarray(getattr(o, key))[0]
                out[f'{n}__{tag}_{port}_plane'] = np.asarray(o.reference['plane'])
                out[f'{n}__{tag}_{port}_cell_measure'] = np.asarray(o.reference['cell_measure'])
                out[f'{n}__{tag}_{port}_incident_power'] = np.asarray(o.reference['incident_power'])
                out[f'{n}__{tag}_{port}_epsilon'] = np.asarray(o.reference['epsilon'])
    out['names'] = np.array(names)
    np.savez_compressed(os.path.join(HERE, 'ref_amplitudes.npz'), **out)
    print('ref_amplitudes.npz:', len(names), 'cases')


def make_backside_cases():
    """The reference's own run of scenes lit from below (``PlaneWave(side='bottom')``: the angles
    in the substrate, R back into it, T into the superstrate): per-order R and T, the amplitude
    ratios and the other per-order readings, fields at explicit points and the boundary fields,
    s and mixed incidence with a 2.5 V/m source."""
    from wavebit import Material, Units, rcwa
    out = {}
    names = []
    scenes = [c for c in ref_cases() if c['name'] in ('grating_1d', 'crossed_1', 'crossed_4', 'symmetric_pillar')]
    scenes += [c for c in halfspace_cases() if c['name'] in ('tir', 'dense_superstrate', 'normal_rotated')]
    for case in scenes:
        n = case['name']
        names.append(n)
        for key in ('structure', 'thickness', 'wavelength', 'period', 'orders', 'theta', 'phi',
                    'eps_top', 'eps_bot'):
            out[f'{n}__{key}'] = np.asarray(case[key])
        st = case['structure'][::-1]
        th = np.asarray(case['thickness'], dtype=float)[::-1]
        layers = tuple(rcwa.Layer(thickness=float(t), epsilon=np.asarray(e)) for e, t in zip(st, th))
        px, py = (float(v) for v in case['period'])
        x = np.array([-0.31 * px, 0.0, 0.45 * px])
        y = np.array([-0.27 * py, 0.5 * py])
        faces = np.concatenate([[0.0], np.cumsum(th)])
        z = np.unique(np.concatenate([faces, faces[:-1] + 0.37 * th]))
        for tag, pol in (('s', 's'), ('mix', (0.6, 0.8j))):
            prob = rcwa.Problem(
                units=Units(length='nm'),
                stack=rcwa.Stack(period=case['period'], top=Material(epsilon=case['eps_top']),
                                 bottom=Material(epsilon=case['eps_bot']), layers=layers),
                excitation=rcwa.Excitation(wavelength=case['wavelength'], sources=(
                    rcwa.PlaneWave(side='bottom', polarization=pol, theta=case['theta'], phi=case['phi'],
                                   amplitude=2.5),)),
                outputs=rcwa.Outputs(fields=True, scattering=True))
            res = rcwa.run(prob, numerics=rcwa.Numerics(orders=case['orders']))
            if tag == 's':
                # the scattering matrix is incidence-relative: S11 reflects back into the substrate
                S = res.scattering[0]
                for blk in ('S11', 'S12', 'S21', 'S22'):
                    out[f'{n}__{blk}'] = np.asarray(getattr(S, blk))
                out[f'{n}__entry_index'] = np.asarray(S.entry_port.refractive_index)
            out[f'{n}__R_{tag}'] = np.asarray(res.R)[0]
            out[f'{n}__T_{tag}'] = np.asarray(res.T)[0]
            for port in ('reflected', 'transmitted'):
                o = res.outputs[port]
                for key in ('amplitude_ratio_s', 'amplitude_ratio_p', 'amplitude_ratio_xyz', 'power', 'k_parallel',
                            'k_normal'):
                    out[f'{n}__{tag}_{port}_{key}'] = np.asarray(getattr(o, key))[0]
                out[f'{n}__{tag}_{port}_plane'] = np.asarray(o.reference['plane'])
                out[f'{n}__{tag}_{port}_port'] = np.asarray(o.reference['port'])
                out[f'{n}__{tag}_{port}_incident_power'] = np.asarray(o.reference['incident_power'])
            out[f'{n}__field_{tag}'] = np.asarray(res.field(x=x, y=y, z=z).values)
            out[f'{n}__field_lalanne_{tag}'] = np.asarray(res.field(x=x, y=y, z=z, reconstruction='lalanne').values)
            for side in ('top', 'bottom'):
                for part in ('incoming', 'outgoing'):
                    b = res.boundary_fields(side=side, x=x, y=y, part=part)
                    out[f'{n}__boundary_{side}_{part}_{tag}'] = np.asarray(b.values)
        out[f'{n}__x'], out[f'{n}__y'], out[f'{n}__z'] = x, y, z
    out['names'] = np.array(names)
    np.savez_compressed(os.path.join(HERE, 'ref_backside.npz'), **out)
    print('ref_backside.npz:', len(names), 'cases')


def make_direct_cases():
    """The reference's own run with the incidence given as a wavevector
    (``PlaneWave(kx=, ky=)``, rad per length unit, fixed across two wavelengths so the angle
    changes with the wavelength), lit from either side, and at exactly normal incidence: per-order
    R and T and the amplitude ratios, s and mixed incidence."""
    from wavebit import Material, Units, rcwa
    out = {}
    names = []
    plans = [('crossed_1', 'top', 0.003, -0.002), ('crossed_4', 'top', -0.0041, 0.0007),
             ('symmetric_pillar', 'top', 0.0, 0.0), ('tir', 'bottom', 0.0025, 0.001),
             ('grating_1d', 'bottom', -0.002, 0.0)]
    cases = {c['name']: c for c in ref_cases() + halfspace_cases()}
    for n, side, kx, ky in plans:
        case = cases[n]
        names.append(n)
        for key in ('structure', 'thickness', 'period', 'orders', 'eps_top', 'eps_bot'):
            out[f'{n}__{key}'] = np.asarray(case[key])
        wls = np.array([0.92, 1.07]) * float(case['wavelength'])
        out[f'{n}__wavelengths'], out[f'{n}__kx'], out[f'{n}__ky'] = wls, np.asarray(kx), np.asarray(ky)
        out[f'{n}__side'] = np.asarray(side)
        st = case['structure'][::-1]
        th = np.asarray(case['thickness'], dtype=float)[::-1]
        layers = tuple(rcwa.Layer(thickness=float(t), epsilon=np.asarray(e)) for e, t in zip(st, th))
        for tag, pol in (('s', 's'), ('mix', (0.6, 0.8j))):
            prob = rcwa.Problem(
                units=Units(length='nm'),
                stack=rcwa.Stack(period=case['period'], top=Material(epsilon=case['eps_top']),
                                 bottom=Material(epsilon=case['eps_bot']), layers=layers),
                excitation=rcwa.Excitation(wavelength=wls, sources=(
                    rcwa.PlaneWave(side=side, polarization=pol, kx=kx, ky=ky),)))
            res = rcwa.run(prob, numerics=rcwa.Numerics(orders=case['orders']))
            out[f'{n}__R_{tag}'] = np.asarray(res.R)
            out[f'{n}__T_{tag}'] = np.asarray(res.T)
            for port in ('reflected', 'transmitted'):
                o = res.outputs[port]
                for comp in ('s', 'p'):
                    out[f'{n}__{tag}_{port}_{comp}'] = np.asarray(getattr(o, f'amplitude_ratio_{comp}'))
                out[f'{n}__{tag}_{port}_k_parallel'] = np.asarray(o.k_parallel)
    out['names'] = np.array(names)
    np.savez_compressed(os.path.join(HERE, 'ref_direct.npz'), **out)
    print('ref_direct.npz:', len(names), 'cases')


def make_bare_cases():
    """Stacks with no layers: the reference solves the bare interface between its half-spaces
    (results.py:180-189) -- per-order R/T of its own run, s and p."""
    out = {}
    scenes = [dict(name='bare_oblique', eps_top=1.0, eps_bot=2.25, theta=0.4, phi=0.3),
              dict(name='bare_lossy', eps_top=2.25, eps_bot=-8.0 + 1.2j, theta=0.25, phi=1.1)]
    for sc in scenes:
        case = dict(sc, structure=np.zeros((0, 1, 1), complex), thickness=[], wavelength=633.0,
                    period=(500.0, 600.0), orders=(2, 1))
        n = sc['name']
        for key in ('wavelength', 'period', 'orders', 'theta', 'phi', 'eps_top', 'eps_bot'):
            out[f'{n}__{key}'] = np.asarray(case[key])
        for pol in ('s', 'p'):
            R, T, _ = run_ref(case, pol)
            out[f'{n}__R_{pol}'] = R
            out[f'{n}__T_{pol}'] = T
    out['names'] = np.array([sc['name'] for sc in scenes])
    np.savez_compressed(os.path.join(HERE, 'ref_bare.npz'), **out)
    print('ref_bare.npz:', len(scenes), 'cases')


def make_reticolo_cases():
    """RETICOLO's per-order efficiencies of twelve 1D binary gratings (the reference's
    tests/references/golden_reticolo.npz, read by test_reticolo_golden.py), with their inputs as
    that test spells them (restated top layer first, permittivities; TE/TM are the s/p columns at
    phi = 0, the conical cases take psi). RETICOLO reports the propagating orders only: ``idx_*``
    are their positions in the order vector -h..h."""
    gold = np.load(os.path.join(REF, 'tests/references/golden_reticolo.npz'))
    half = [[[9.0] * 5 + [1.0] * 5]]
    quarter = [[[12.25] * 3 + [1.0] * 9]]
    # the test hands the factory `_TWO_LAYER[::-1]` with thickness [0.22, 0.15], layers listed from
    # the bottom up: top first, that is the eps-9 layer (0.15) over the eps-4.84 layer (0.22)
    two = [[[9.0] * 6 + [1.0] * 6], [[4.840000000000001] * 8 + [1.0] * 4]]
    base = dict(theta=0.0, phi=0.0, top=1.0, bot=2.25, h=10, period=0.7, wavelength=0.9, structure=half,
                thickness=[0.15])
    cases = {
        'te_normal': dict(base, pol='s'),
        'te_oblique': dict(base, pol='s', theta=0.2),
        'tm_normal': dict(base, pol='p'),
        'tm_oblique': dict(base, pol='p', theta=0.2),
        'te_quarter': dict(base, pol='s', theta=0.15, h=12, period=0.8, wavelength=0.7, structure=quarter,
                           thickness=[0.25]),
        'tm_quarter': dict(base, pol='p', theta=0.15, h=12, period=0.8, wavelength=0.7, structure=quarter,
                           thickness=[0.25]),
        'te_two_layer': dict(base, pol='s', theta=0.25, bot=4.0, wavelength=0.85, structure=two,
                             thickness=[0.15, 0.22]),
        'tm_two_layer': dict(base, pol='p', theta=0.25, bot=4.0, wavelength=0.85, structure=two,
                             thickness=[0.15, 0.22]),
        'te_high_order': dict(base, pol='s', theta=0.2, h=30),
        'tm_high_order': dict(base, pol='p', theta=0.2, h=30),
        'conical_te': dict(base, pol='s', theta=0.2, phi=0.3),
        'conical_tm': dict(base, pol='p', theta=0.2, phi=0.3),
    }
    out = {}
    for name, kw in cases.items():
        for key, val in kw.items():
            out[f'{name}__{key}'] = np.asarray(val)
        for side in ('ri', 'ti'):
            out[f'{name}__idx_{side}'] = np.asarray(gold[f'{name}__idx_{side}'])
            out[f'{name}__de_{side}'] = np.asarray(gold[f'{name}__de_{side}'])
            # the same scene lit from below at the same in-plane wavevector (RETICOLO's inc_bottom):
            # reflection back into the substrate, transmission into the superstrate
            out[f'{name}__de_{side}_bot'] = np.asarray(gold[f'{name}__de_{side}_bot'])
    out['names'] = np.array(list(cases))
    np.savez_compressed(os.path.join(HERE, 'reticolo_cases.npz'), **out)
    print('reticolo_cases.npz:', len(cases), 'cases')


if __name__ == '__main__':
    use_reference()
    make_ref_cases()
    make_integrated_cases()
    make_scattering_cases()
    make_field_cases()
    make_etm_cases()
    make_halfspace_cases()
    make_bare_cases()
    make_backside_cases()
    make_direct_cases()
    make_amplitude_cases()
    make_legacy_cases()
    make_reticolo_cases()
