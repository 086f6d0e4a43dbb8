"""Benchmark of the RCWA raster layer path on GB300.

Default workload (one "step"): points of the orders-(12, 12) sweep — four seeded 256x256 binary
rasters (eps 1 / 12.25, rectangles and discs), period 1000 nm, superstrate 1, substrate 2.25,
625 harmonics and 1250x1250 mode matrices, 256 wavelengths over 400-1000 nm x theta in
{0, 0.2, 0.4, 0.6}. A step solves ``--solves`` of those 1024 points, evenly spaced over the
sweep, in the mixed form; one solve is one (wavelength, theta) S-matrix answering s and p. The
per-step working set (tens of GB of mode matrices) is far larger than L2, so no flush is needed
between steps. ``--workload crossed_sweep`` is the orders-(7, 7) sweep (three rasters and a
metallic film, 128 wavelengths at normal incidence) in the FP64 form.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload mixed_sweep|crossed_sweep]
                  [--precision double|mixed|...] [--solves B] [--impl reference]
  python bench.py --profile-calls C ...      # stage A, then C solves of the batch; for profilers
  python bench.py --workload adjoint_layer   # gradient timing and finite-difference check

Prints one JSON line (rank 0). ``value`` is the chosen form's rate; ``mixed_vs_fp64`` times the
other form on the same batch (one call) and reports both rates, the speed-up and the max |dR,T|
between them; ``oracle_check`` compares the GPU's R/T with the CPU oracle on one point of the
batch. ``--impl reference`` times the reference's own public ``rcwa.run`` (a copy of its source
under ``baseline/_ref``) on the host cores, or the oracle (its NumPy restatement) when that copy is
absent.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

UNIT = 'solves/s'

WORKLOADS = {
    'mixed_sweep': dict(precision='mixed', solves=38),
    'crossed_sweep': dict(precision='double', solves=128),
}


def metric(workload, precision):
    form = {'double': 'plain FP64 form', 'mixed': 'mixed form (FP32 eigen-solve and cascade + FP64 Newton '
                                                  'and refinement), |dR,T| <= 1e-6 vs FP64'}.get(precision, precision + ' form')
    if workload == 'mixed_sweep':
        what = 'orders (12,12) sweep, 4 layers of 256^2, 1250x1250 mode matrices'
    else:
        what = 'orders (7,7) crossed-grating sweep, 4 layers of 256^2, 450x450 mode matrices'
    return f'RCWA solves/s, {form} ({what}; one solve = one (wavelength, theta) S-matrix, s and p)'


def _dist():
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return world, rank, local


def max_over_ranks(t, world, dist=None, device='cpu'):
    """The slowest rank's time (all_reduce MAX; one value per rank, FP64). Every rank times the
    same region between the same two barriers, and the job's throughput is set by the rank that
    took longest."""
    if world <= 1:
        return float(t)
    import torch
    tt = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def whole_job_rate(world, units_per_rank, steps, t_max):
    """Units per second of the whole job: every rank solves its own ``units_per_rank`` per step
    (replicas, weak scaling), all of them within the slowest rank's ``t_max``."""
    return world * units_per_rank * steps / t_max


def load_workload(name, solves):
    """The workload's stack and the batch of points a step solves."""
    from wavebit_gb300 import workloads as WL
    if name == 'crossed_sweep':
        cfg = WL.crossed_sweep(n_wavelengths=solves)
        cfg['points'] = np.arange(solves)
    else:
        cfg = WL.mixed_sweep()
        keep = np.linspace(0, len(cfg['wavelengths']) - 1, solves).round().astype(int)
        cfg['points'] = keep
        for k in ('wavelengths', 'thetas', 'phis'):
            cfg[k] = cfg[k][keep]
    return cfg


def _config(workload, precision, impl, B):
    if workload == 'crossed_sweep':
        desc = ('crossed_sweep: 3x 256^2 binary rasters + 50 nm eps=-20+1.5j layer, period 1000 nm, '
                f'eps_top 1, eps_bot 2.25, orders (7,7), N=225, n=450, {B} wavelengths 400-1000 nm, theta 0, '
                's+p per solve')
        orders = [7, 7]
    else:
        desc = ('mixed_sweep: 4x 256^2 binary rasters, period 1000 nm, eps_top 1, eps_bot 2.25, orders (12,12), '
                f'N=625, n=1250, {B} of the 1024 (wavelength 400-1000 nm x theta 0/0.2/0.4/0.6) points per step, '
                'evenly spaced, s+p per solve')
        orders = [12, 12]
    return {'workload': desc, 'orders': orders, 'layers': 4, 'solves_per_step': B, 'raster': [256, 256],
            'precision': precision, 'impl': impl, 'parallelism': 'replicas (one sweep per GPU)',
            'l2': 'inputs larger than L2: per-step working set of GBs >> 129 MB (no flush needed)'}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,'
         'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
         'clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), f'--query-gpu={self.Q}',
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in self.lines:
            parts = [p.strip() for p in line.split(',')]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0])); mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == 'active':
                    reasons.add(nm)
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': max(mx) if mx else None,
                'reasons': sorted(reasons), 'samples': len(sm)}


# ------------------------------------------------------------------------------ CPU legs

def oracle_solve(cfg, i):
    """One point of the batch through the oracle (NumPy restatement of the reference path):
    R, T as (3, N) for [given (s), pure s, pure p] and the seconds it took."""
    from oracle import rcwa_oracle as O
    hu, hv = cfg['orders']
    if 'oracle_conv' not in cfg:
        cfg['oracle_conv'] = O.to_conv_mat_raster_sampled(cfg['eps'], hu, hv)
    t0 = time.perf_counter()
    o = O.solve_stack(cfg['eps'], cfg['thickness'], float(cfg['wavelengths'][i]), cfg['period'], hu, hv,
                      float(cfg['thetas'][i]), 0.0, cfg['eps_top'], cfg['eps_bot'], 's', conv=cfg['oracle_conv'])
    dt = time.perf_counter() - t0
    return o['R'].reshape(3, -1), o['T'].reshape(3, -1), dt


def reference_available():
    return os.path.isdir(os.path.join(ROOT, 'baseline', '_ref', 'wavebit'))


def reference_point(cfg, i):
    """One point through the reference's own public API (``rcwa.run``, NumPy backend, its
    defaults: SMM, sampled Li, fixed nesting) from the copy of its source under ``baseline/_ref``.
    The reference answers one polarization per run, so a point is an s run and a p run. Returns
    the s and p per-order R, T and the seconds both runs took."""
    ref = os.path.join(ROOT, 'baseline', '_ref')
    if ref not in sys.path:
        sys.path.insert(0, ref)
    from wavebit import Material, Units, rcwa
    st = cfg['eps'][::-1]                       # the public stack lists layers bottom to top
    th = list(cfg['thickness'])[::-1]
    layers = tuple(rcwa.Layer(thickness=float(t), epsilon=np.asarray(e)) for e, t in zip(st, th))
    out = {}
    t0 = time.perf_counter()
    for pol in ('s', 'p'):
        prob = rcwa.Problem(
            units=Units(length='nm'),
            stack=rcwa.Stack(period=tuple(cfg['period']), top=Material(epsilon=cfg['eps_top']),
                             bottom=Material(epsilon=cfg['eps_bot']), layers=layers),
            excitation=rcwa.Excitation(wavelength=float(cfg['wavelengths'][i]), sources=(
                rcwa.PlaneWave(polarization=pol, theta=float(cfg['thetas'][i]), phi=0.0),)))
        res = rcwa.run(prob, numerics=rcwa.Numerics(orders=tuple(cfg['orders'])))
        out[pol] = (np.asarray(res.R)[0].reshape(-1), np.asarray(res.T)[0].reshape(-1))
    return out, time.perf_counter() - t0


def cpu_baseline(cfg, n_points):
    """The reference's own NumPy path on the host cores (``kind`` "reference"), or the oracle
    port when the reference's source is not present (``kind`` "port"), on a bounded sample."""
    idx = np.linspace(0, len(cfg['wavelengths']) - 1, max(1, n_points)).round().astype(int)
    ts = []
    if reference_available():
        for i in idx:
            ts.append(reference_point(cfg, int(i))[1])
        kind, what = 'reference', 'the reference rcwa.run (NumPy backend, baseline/_ref), an s and a p run per point'
    else:
        for i in idx:
            ts.append(oracle_solve(cfg, int(i))[2])
        kind, what = 'port', 'oracle/rcwa_oracle.py (the NumPy restatement), s and p from one S-matrix'
    dt = sum(ts)
    return {'value': len(idx) / dt, 'unit': UNIT, 'cores': os.cpu_count(), 'kind': kind,
            'sample': f'{len(idx)} point(s) of the step\'s batch through {what}, {dt:.1f} s, '
                      f'all {os.cpu_count()} host cores available to BLAS'}


def run_reference(args, world, rank):
    """The reference arm: the reference's own CPU path on this workload, on rank 0 only. A step is
    one point of the batch (an s and a p run of ``rcwa.run``); the warm-up is a ``rcwa.prepare`` of
    the stack (imports, checks), and the timed steps stop early once ``--ref-budget`` seconds
    are spent, so that the arm ends within a few minutes (the line reports the steps it timed)."""
    if rank != 0:
        return
    cfg = load_workload(args.workload, args.solves or WORKLOADS[args.workload]['solves'])
    B = len(cfg['wavelengths'])
    order = np.linspace(0, B - 1, max(1, args.steps)).round().astype(int)
    times = []
    use_ref = reference_available()
    if use_ref and args.warmup > 0:
        reference_point_warm(cfg)
    t_start = time.perf_counter()
    for i in order:
        if use_ref:
            times.append(reference_point(cfg, int(i))[1])
        else:
            times.append(oracle_solve(cfg, int(i))[2])
        if time.perf_counter() - t_start > args.ref_budget:
            break
    per_step = statistics.mean(times)
    value = 1.0 / per_step
    kind = 'reference' if use_ref else 'port'
    what = ('the reference rcwa.run (NumPy backend, its defaults; source copy under baseline/_ref), an s and a '
            'p run per point' if use_ref else 'oracle/rcwa_oracle.py, the NumPy restatement (the reference source '
            'is absent here)')
    precision = args.precision or WORKLOADS[args.workload]['precision']
    line = {'impl': 'reference', 'metric': metric(args.workload, precision), 'value': value, 'unit': UNIT,
            'n_gpus': args.gpus, 'steps': len(times), 'steps_requested': args.steps, 'warmup': args.warmup,
            'ms_per_step': per_step * 1e3, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'c128', 'data': 'synthetic', 'config': _config(args.workload, 'double', 'reference', 1),
            'cpu_baseline': {'value': value, 'unit': UNIT, 'cores': os.cpu_count(), 'kind': kind,
                             'sample': f'{len(times)} point(s) of the batch, one per step, through {what}; '
                                       f'{sum(times):.1f} s'},
            'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def reference_point_warm(cfg):
    """Imports the reference and prepares the stack once (no solve)."""
    ref = os.path.join(ROOT, 'baseline', '_ref')
    if ref not in sys.path:
        sys.path.insert(0, ref)
    from wavebit import Material, Units, rcwa
    layers = tuple(rcwa.Layer(thickness=float(t), epsilon=np.asarray(e))
                   for e, t in zip(cfg['eps'][::-1], list(cfg['thickness'])[::-1]))
    prob = rcwa.Problem(units=Units(length='nm'),
                        stack=rcwa.Stack(period=tuple(cfg['period']), top=Material(epsilon=cfg['eps_top']),
                                         bottom=Material(epsilon=cfg['eps_bot']), layers=layers),
                        excitation=rcwa.Excitation(wavelength=float(cfg['wavelengths'][0]), sources=(
                            rcwa.PlaneWave(polarization='s', theta=float(cfg['thetas'][0]), phi=0.0),)))
    rcwa.prepare(prob, numerics=rcwa.Numerics(orders=tuple(cfg['orders'])))


# ------------------------------------------------------------------------------ GPU legs

def hbm_peak():
    """Measured HBM copy bandwidth of the GB300s (GB/s), or the 6.8 TB/s fallback."""
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    try:
        with open(path) as f:
            return float(json.load(f)['hbm_gbs']), 'MEASURED_PEAKS.json hbm_gbs (measured)'
    except (OSError, KeyError, ValueError):
        return 6800.0, 'fallback 6.8 TB/s'


#: DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) per algorithmic byte of the QR
#: sweep, from one small-case capture of each kernel (profiles/hseqr_*); the bench scales its live
#: algorithmic bytes by it.
QR_TRAFFIC_PER_ALGORITHMIC_BYTE = {'float': 643547068928 / 7.58558e11}
QR_TRAFFIC_SOURCE = ('ncu dram__bytes_read.sum + dram__bytes_write.sum of one hseqr_kernel<float> launch on 4 '
                     'solves (16 matrices, 643.5 GB against 758.6 GB algorithmic), scaled by the live '
                     'algorithmic bytes (profiles/hseqr_fp32_orders12_4solves.md)')


def qr_profile(handle, real_type):
    """Summed CUDA-event time, launches and algorithmic bytes of the QR sweeps recorded since
    wb_profile_qr(1); profiling is switched off again."""
    import ctypes
    from wavebit_gb300 import _lib
    ms, la, by = ctypes.c_double(0), ctypes.c_longlong(0), ctypes.c_double(0)
    _lib.check(handle.lib.wb_profile_qr_read(real_type, ctypes.byref(ms), ctypes.byref(la), ctypes.byref(by)))
    _lib.check(handle.lib.wb_profile_qr(0))
    return {'ms': ms.value, 'launches': la.value, 'bytes': by.value,
            'type': {0: 'double', 1: 'float', 2: 'df64'}[real_type]}


def batch_inputs(cfg, B):
    from wavebit_gb300 import workloads as WL
    L = cfg['eps'].shape[0]
    return dict(li=np.tile(np.arange(L, dtype=np.int32), (B, 1)), th=np.tile(cfg['thickness'], (B, 1)),
                wl=np.asarray(cfg['wavelengths'], np.float64), per=np.tile(cfg['period'], (B, 1)),
                theta=np.asarray(cfg['thetas'], np.float64), phi=np.zeros(B),
                et=np.full(B, cfg['eps_top'], complex), eb=np.full(B, cfg['eps_bot'], complex),
                pol=np.tile(np.array(WL.pol_pair('s'), complex), (B, 1)))


def profile_calls(args):
    """Stage A once, then ``--profile-calls`` solves of the step's batch; one status line. For
    profilers (ncu launch lists and captures), so that they see the solve alone."""
    import torch
    from wavebit_gb300 import engine as E
    precision = args.precision or WORKLOADS[args.workload]['precision']
    B = args.solves or WORKLOADS[args.workload]['solves']
    cfg = load_workload(args.workload, B)
    hu, hv = cfg['orders']
    dev = torch.device('cuda', 0)
    eps_dev = torch.as_tensor(cfg['eps'], device=dev)
    E.assemble(eps_dev, hu, hv)                        # warm (library load, arena)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    conv = E.assemble(eps_dev, hu, hv)
    ev1.record()
    torch.cuda.synchronize()
    stage_a_ms = ev0.elapsed_time(ev1)
    x = batch_inputs(cfg, B)
    inp = E.BatchInputs(x['li'], x['th'], x['wl'], x['per'], x['theta'], x['phi'], x['et'], x['eb'], x['pol'],
                        device=dev)
    from wavebit_gb300 import _lib
    h = _lib.handle(0)
    _lib.check(h.lib.wb_profile_qr(1))
    st = None
    ev2, ev3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev2.record()
    for _ in range(args.profile_calls):
        R, T, st = E.solve_batch(conv, inp, precision=precision)
    ev3.record()
    torch.cuda.synchronize()
    solve_ms = ev2.elapsed_time(ev3) / args.profile_calls
    qr = qr_profile(h, 0 if precision == 'double' else 1 if precision == 'mixed' else 2)
    print(f'{args.workload} {precision} solves={B} calls={args.profile_calls} '
          f'status_nonzero={int((st.cpu().numpy() & ~8).astype(bool).sum())} '
          f"qr_sweep_{qr['type']}: launches={qr['launches']} ms={qr['ms']:.1f} algorithmic_bytes={qr['bytes']:.6g} "
          f"stage_a_ms={stage_a_ms:.2f} solve_ms={solve_ms:.1f}")


def adjoint_check(args):
    """The adjoint-gradient workload: one 220 nm layer, a 128x128 continuous raster, orders
    (9, 9), 32 wavelengths over 1000-1600 nm, p, loss = sum of T(0, 0). Times one forward+reverse
    pass (16384 pixel gradients and the thickness) and compares with central finite differences
    of the same forward: 16 seeded pixels at steps 1e-6 and 1e-5 (two steps measure the
    difference quotient's own noise), the thickness at 1e-4 nm."""
    import torch
    from wavebit_gb300 import adjoint as AD
    from wavebit_gb300 import workloads as WL
    cfg = WL.adjoint_layer(side=128, n_wavelengths=args.adjoint_wavelengths)
    h = cfg['orders'][0]
    N = (2 * h + 1) ** 2
    Bw = len(cfg['wavelengths'])
    wR, wT = np.zeros((Bw, N)), np.zeros((Bw, N))
    wT[:, N // 2] = 1.0
    kw = dict(wavelengths=cfg['wavelengths'], period=cfg['period'], hu=h, hv=h, theta=0.0, phi=0.0,
              eps_top=cfg['eps_top'], eps_bot=cfg['eps_bot'], pol=(0.0, 1.0), impl='gb300', device='cuda',
              modes=args.precision or 'double')
    eps, th = cfg['eps'], cfg['thickness']
    AD.solve_and_grad(eps, th, weights_R=wR, weights_T=wT, grad=False, **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss, R, T, g_eps, g_th = AD.solve_and_grad(eps, th, weights_R=wR, weights_T=wT, **kw)
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    rng = np.random.default_rng(16)
    pix = [tuple(int(v) for v in rng.integers(0, eps.shape[1], size=2)) for _ in range(args.pixels)]

    def fd(y, x, step):
        ep, em = eps.copy(), eps.copy()
        ep[0, y, x] += step
        em[0, y, x] -= step
        return (AD.solve_and_grad(ep, th, weights_R=wR, weights_T=wT, grad=False, **kw)[0]
                - AD.solve_and_grad(em, th, weights_R=wR, weights_T=wT, grad=False, **kw)[0]) / (2 * step)
    rows = []
    for (y, x) in pix:
        rows.append(dict(y=y, x=x, fd_1e6=fd(y, x, 1e-6), fd_1e5=fd(y, x, 1e-5), adjoint=float(g_eps[0, y, x])))
    gmax = float(g_eps.abs().max())
    err6 = max(abs(r['fd_1e6'] - r['adjoint']) for r in rows) / gmax
    err5 = max(abs(r['fd_1e5'] - r['adjoint']) for r in rows) / gmax
    fdfd = max(abs(r['fd_1e6'] - r['fd_1e5']) for r in rows) / gmax
    tp, tm = th.copy(), th.copy()
    tp[0] += 1e-4
    tm[0] -= 1e-4
    fd_t = (AD.solve_and_grad(eps, tp, weights_R=wR, weights_T=wT, grad=False, **kw)[0]
            - AD.solve_and_grad(eps, tm, weights_R=wR, weights_T=wT, grad=False, **kw)[0]) / 2e-4
    print(json.dumps({'workload': f'adjoint_layer 128x128, orders ({h},{h}), {Bw} wavelengths, p, sum T(0,0)',
                      'modes': kw['modes'], 'loss': loss, 'grad_seconds': t_grad, 'fd_pixels': len(pix),
                      'max_abs_err_over_max_grad': {'fd_step_1e-6': err6, 'fd_step_1e-5': err5,
                                                    'fd_1e-6_vs_fd_1e-5': fdfd},
                      'thickness_grad': float(g_th[0]), 'thickness_fd': fd_t,
                      'thickness_rel_err': abs(fd_t - float(g_th[0])) / max(abs(fd_t), 1e-300),
                      'samples': rows[:4]}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=3)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--workload', default='mixed_sweep', choices=['mixed_sweep', 'crossed_sweep', 'adjoint_layer'])
    ap.add_argument('--precision', default=None,
                    choices=['double', 'mixed', 'mixed_fp32', 'mixed_df64', 'mixed_df64_eig'])
    ap.add_argument('--solves', type=int, default=None)
    ap.add_argument('--e2e-calls', type=int, default=5)
    ap.add_argument('--ref-sample', type=int, default=1, help='points of the batch in cpu_baseline')
    ap.add_argument('--ref-budget', type=float, default=150.0, help='seconds of timed steps in --impl reference')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-compare', action='store_true', help='skip the other form and the oracle check')
    ap.add_argument('--profile-calls', type=int, default=0)
    ap.add_argument('--tensor-cores', default='on', choices=['on', 'off'],
                    help='off: the FP32 complex products on the SIMT kernel instead of tcgen05 (for comparison)')
    ap.add_argument('--tune', action='append', default=[], metavar='KEY=VALUE',
                    help='set a launch-shape tunable before the run (wb_set_tuning; keys WB_TUNE_*)')
    ap.add_argument('--pixels', type=int, default=16)
    ap.add_argument('--adjoint-wavelengths', type=int, default=32)
    args = ap.parse_args()
    world, rank, local = _dist()
    if args.tensor_cores == 'off' and args.impl != 'reference':
        from wavebit_gb300 import _lib
        _lib.check(_lib.load().wb_set_tuning(_lib.WB_TUNE_TENSOR_CORES, 1))
    if args.tune and args.impl != 'reference':
        from wavebit_gb300 import _lib
        for kv in args.tune:
            key, val = (int(x) for x in kv.split('='))
            _lib.check(_lib.load().wb_set_tuning(key, val))
    if args.workload == 'adjoint_layer':
        return adjoint_check(args)
    if args.impl == 'reference':
        return run_reference(args, world, rank)
    if args.profile_calls:
        return profile_calls(args)

    import torch
    import torch.distributed as dist
    from wavebit_gb300 import _lib, engine as E
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    if world > 1:
        dist.init_process_group('nccl')
    precision = args.precision or WORKLOADS[args.workload]['precision']
    B = args.solves or WORKLOADS[args.workload]['solves']
    cfg = load_workload(args.workload, B)
    hu, hv = cfg['orders']
    L = cfg['eps'].shape[0]
    N = E.n_orders(hu, hv)
    handle = _lib.handle(local)
    eps_host = np.ascontiguousarray(cfg['eps'])
    x = batch_inputs(cfg, B)
    # inputs resident in HBM
    conv = E.assemble(torch.as_tensor(eps_host, device=dev), hu, hv, handle=handle)
    inp = E.BatchInputs(x['li'], x['th'], x['wl'], x['per'], x['theta'], x['phi'], x['et'], x['eb'], x['pol'],
                        device=dev)
    out = (torch.empty((B, 3, N), dtype=torch.float64, device=dev), torch.empty((B, 3, N), dtype=torch.float64, device=dev),
           torch.zeros(B, dtype=torch.int32, device=dev), None)

    def step():
        return E.solve_batch(conv, inp, precision=precision, handle=handle, out=out)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    barrier()
    stream = torch.cuda.current_stream()
    launches0 = handle.launches()
    _lib.check(handle.lib.wb_profile_qr(1))       # live CUDA-event timing of the QR sweeps
    clocks = ClockSampler(local)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    barrier()
    clk = clocks.stop()
    launches = handle.launches() - launches0
    qr = qr_profile(handle, 0 if precision == 'double' else 1 if precision == 'mixed' else 2)
    t = ev0.elapsed_time(ev1) / 1e3
    R0, T0 = out[0].clone(), out[1].clone()
    st = out[2].cpu().numpy()
    t = max_over_ranks(t, world, dist, dev)
    value = whole_job_rate(world, B, args.steps, t)

    # the metric compares the mixed form with the FP64 one: the other form times one call on the
    # same batch (CUDA events on the launching stream), and the max |dR,T| between the two
    mixed_vs_fp64 = None
    if rank == 0 and not args.no_compare:
        other = 'mixed' if precision == 'double' else 'double'
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        R1, T1, st1 = E.solve_batch(conv, inp, precision=other, handle=handle)
        e1.record(stream)
        torch.cuda.synchronize()
        t1 = e0.elapsed_time(e1) / 1e3
        d = max(float((R0.view(B, 3, -1) - R1.view(B, 3, -1)).abs().max()),
                float((T0.view(B, 3, -1) - T1.view(B, 3, -1)).abs().max()))
        t_self = t / args.steps
        t64, tmx = (t_self, t1) if precision == 'double' else (t1, t_self)
        Rf = (R0 if precision == 'double' else R1).view(B, 3, -1).cpu().numpy()
        Tf = (T0 if precision == 'double' else T1).view(B, 3, -1).cpu().numpy()
        mixed_vs_fp64 = {'fp64_value': B / t64, 'fp64_ms_per_step': t64 * 1e3, 'fp64_calls_timed': 1 if precision != 'double' else args.steps,
                         'mixed_value': B / tmx, 'mixed_ms_per_step': tmx * 1e3, 'speedup': t64 / tmx,
                         'mixed_form': 'mixed' if precision == 'double' else precision,
                         'max_abs_dRT': d, 'target': 1e-6, 'within_target': d <= 1e-6,
                         'fp64_status_nonzero': int(((st1.cpu().numpy() if precision != 'double' else st) & ~8).astype(bool).sum())}
    else:
        Rf = R0.view(B, 3, -1).cpu().numpy() if precision == 'double' else None
        Tf = T0.view(B, 3, -1).cpu().numpy() if precision == 'double' else None

    # the GPU's R/T against the CPU oracle on one point of the batch (FP64 form at 1e-10 of the
    # largest efficiency; the chosen form too)
    oracle_check = None
    if rank == 0 and not args.no_compare:
        i = B // 2
        Ro, To, t_or = oracle_solve(cfg, i)
        scale = max(np.abs(Ro).max(), np.abs(To).max())
        Rs, Ts = R0.view(B, 3, -1)[i].cpu().numpy(), T0.view(B, 3, -1)[i].cpu().numpy()
        oracle_check = {'point': int(cfg['points'][i]), 'wavelength': float(cfg['wavelengths'][i]),
                        'theta': float(cfg['thetas'][i]), 'oracle_seconds': t_or,
                        f'max_abs_dRT_{precision}': float(max(np.abs(Rs - Ro).max(), np.abs(Ts - To).max()) / scale)}
        if Rf is not None:
            oracle_check['max_abs_dRT_fp64'] = float(max(np.abs(Rf[i] - Ro).max(), np.abs(Tf[i] - To).max()) / scale)
            oracle_check['fp64_within_1e-10'] = oracle_check['max_abs_dRT_fp64'] <= 1e-10
        oracle_check['note'] = 'relative to the largest efficiency of the point; columns given (s), pure s, pure p'

    # roofline of the dominant kernel, the Schur-form QR sweep of the running form: its launches
    # timed live with CUDA events on the launching stream over the timed region, against the
    # measured HBM copy bandwidth (the sweep is bound by moving H and Z, one bulge step at a time)
    roof = None
    if rank == 0:
        hbm, hbm_src = hbm_peak()
        n = 2 * N
        achieved = qr['bytes'] / (qr['ms'] * 1e-3) / 1e9 if qr['ms'] > 0 else None
        per_launch = qr['bytes'] / qr['launches'] if qr['launches'] else None
        ratio = QR_TRAFFIC_PER_ALGORITHMIC_BYTE.get(qr['type'])
        roof = {'bound': 'hbm', 'kernel': f"wb::hseqr_kernel<{qr['type']}> (Schur-form QR sweeps, {B * L} "
                f"matrices of {n}x{n} per launch, one CTA each)",
                'achieved': achieved, 'peak': hbm, 'unit': 'GB/s', 'frac': achieved / hbm if achieved else None,
                'peak_source': hbm_src,
                'algorithmic_bytes_per_launch': per_launch,
                'bytes_convention': 'every bulge step reads and writes each of its 2n - 2 element pairs\' moving '
                                    'element once (H row or column, Z row), counted on the device per step',
                'launch_ms': qr['ms'] / qr['launches'] if qr['launches'] else None, 'launches': qr['launches'],
                'traffic': per_launch * ratio if (per_launch and ratio) else None,
                'traffic_source': QR_TRAFFIC_SOURCE if ratio else None,
                'share_of_step': (qr['ms'] / 1e3) / t if t > 0 else None,
                'limiter': ('the bulge step\'s barrier rather than bandwidth: ncu warp-state stalls of one launch on '
                            '4 solves (FP32 form) give 7.2 barrier and 2.9 long-scoreboard cycles of 17.7 per issued '
                            'instruction'),
                'whole_step': {'achieved': (280 * L + 192) * n ** 3 * B / (t / args.steps) / 1e12,
                               'unit': 'TFLOP/s', 'flops_convention': '(280 L + 192) n^3 per solve (the reference '
                               'formulation; the cascade here does about 53 n^3 per layer against its 168 n^3)'}}

    # stage A (convolution-matrix assembly of the stack's layers): HBM bytes per layer are the
    # raster read plus the three N x N slots written
    stage_a = None
    if rank == 0:
        eps_dev = torch.as_tensor(eps_host, device=dev)
        E.assemble(eps_dev, hu, hv, handle=handle)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 5
        e0.record(stream)
        for _ in range(reps):
            E.assemble(eps_dev, hu, hv, handle=handle)
        e1.record(stream)
        torch.cuda.synchronize()
        ta = e0.elapsed_time(e1) / 1e3 / reps
        ny, nx = eps_host.shape[1:]
        nbytes = L * (16 * ny * nx + 3 * 16 * N * N)
        hbm, hbm_src = hbm_peak()
        stage_a = {'layers': L, 'ms': ta * 1e3, 'bytes': nbytes, 'achieved_GBps': nbytes / ta / 1e9,
                   'hbm_peak_GBps': hbm, 'peak_source': hbm_src, 'frac': nbytes / ta / 1e9 / hbm,
                   'note': 'runs once per stack and is cached across the sweep'}

    # energy balance |1 - sum R - sum T| for lossless stacks (no absorbing layer)
    energy = None
    if rank == 0 and not np.any(np.imag(eps_host)):
        Rs_, Ts_ = R0.view(B, 3, -1).sum(-1), T0.view(B, 3, -1).sum(-1)
        energy = float((1.0 - Rs_ - Ts_).abs().max())

    # end to end through the C ABI with pinned host buffers: copies in, stage A, solve, copies
    # out, every call
    e2e = None
    if rank == 0 and args.e2e_calls > 0:
        def pinned(a):
            tt = torch.empty(a.shape, dtype=torch.from_numpy(np.zeros(1, a.dtype)).dtype, pin_memory=True)
            v = tt.numpy()
            v[...] = a
            return v, tt
        keep = []
        host = {}
        for k, v in dict(eps=eps_host, **x).items():
            arr, tt = pinned(np.ascontiguousarray(v))
            host[k] = arr
            keep.append(tt)
        outs = []
        for shp, dt in (((B, 3, N), np.float64), ((B, 3, N), np.float64), ((B,), np.int32)):
            arr, tt = pinned(np.zeros(shp, dt))
            outs.append(arr)
            keep.append(tt)
        args_h = (host['eps'], host['li'], host['th'], host['wl'], host['per'], host['theta'], host['phi'],
                  host['et'], host['eb'], host['pol'], hu, hv)
        E.solve_host(*args_h, precision=precision, handle=handle, out=outs)
        te = []
        for _ in range(args.e2e_calls):
            t0 = time.perf_counter()
            E.solve_host(*args_h, precision=precision, handle=handle, out=outs)
            te.append(time.perf_counter() - t0)
        h2d = sum(host[k].nbytes for k in host)
        d2h = sum(o.nbytes for o in outs)
        e2e = {'value': B / statistics.mean(te), 'unit': UNIT, 'h2d_bytes_per_step': int(h2d),
               'd2h_bytes_per_step': int(d2h), 'calls_timed': len(te),
               'entry': 'wb_solve_host (C ABI, pinned host buffers; stage A included)'}

    if rank == 0:
        line = {'metric': metric(args.workload, precision), 'value': value, 'unit': UNIT, 'n_gpus': world,
                'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': t / args.steps * 1e3,
                'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
                'dtype': 'c128' if precision == 'double' else 'c128+c64', 'data': 'synthetic',
                'config': _config(args.workload, precision, 'gb300', B), 'e2e': e2e,
                'gpu_launches': int(launches), 'roofline': roof, 'clocks': clk,
                'status_nonzero': int((st & ~8).astype(bool).sum()), 'grazing_flags': int(((st & 8) != 0).sum()),
                'mixed_vs_fp64': mixed_vs_fp64, 'oracle_check': oracle_check, 'stage_a': stage_a,
                'energy_balance_max': energy}
        if not args.no_cpu_baseline and world == 1:
            line['cpu_baseline'] = cpu_baseline(cfg, args.ref_sample)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
