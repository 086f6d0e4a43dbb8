"""Benchmark of the RCWA raster layer path on GB300.

Workload (one "step"): the crossed-grating sweep — three 256x256 binary rasters + one uniform
eps=-20+1.5j layer, orders (7, 7) (225 harmonics, 450x450 mode matrices), 128 wavelengths over
400-1000 nm at normal incidence; every wavelength is one S-matrix solve that answers s and p
(the pure-s and pure-p columns of the same S-matrix). Inputs are seeded synthetic rasters
(wavebit_gb300/workloads.py). The per-step working set (~8 GB of per-layer matrices) is far
larger than L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision double|mixed|...] [--impl reference]

Prints one JSON line (rank 0). ``value`` is the form chosen by ``--precision`` (FP64 by default);
``mixed_vs_fp64`` times the other form on the same batch and gives both rates, the speed-up and
the max |dR,T| between them (the metric: mixed against FP64 at |dR,T| <= 1e-6). ``--impl reference`` times the CPU restatement of the
reference's NumPy path (oracle/rcwa_oracle.py) on the host cores instead: the reference
package itself is pure Python and is not present on the GPU host.
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

METRIC = 'RCWA solves/s (crossed-grating sweep, orders (7,7), 4 layers; one solve = one wavelength, s and p)'
UNIT = 'solves/s'


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


def _config(precision, impl, B, workload='crossed_sweep'):
    if workload == 'crossed_sweep':
        desc = ('crossed_sweep: 3x 256^2 binary rasters + 50 nm eps=-20+1.5j layer, period 1000 nm, '
                f'eps_top 1, eps_bot 2.25, orders (7,7), N=225, n=450, {B} wavelengths 400-1000 nm, theta 0, '
                's+p per solve')
        orders, layers = [7, 7], 4
    else:
        desc = ('mixed_sweep: 4x 256^2 binary rasters, period 1000 nm, eps_top 1, eps_bot 2.25, orders (12,12), '
                f'N=625, n=1250, {B} of the 1024 (wavelength 400-1000 nm x theta 0/0.2/0.4/0.6) points, '
                'evenly spaced, s+p per solve')
        orders, layers = [12, 12], 4
    return {'workload': desc, 'orders': orders, 'layers': layers, 'solves_per_step': B, 'raster': [256, 256],
            'precision': precision, 'impl': impl, 'parallelism': 'replicas (one sweep per GPU)',
            'l2': 'per-step working set of GBs >> 129 MB L2 (no flush needed)'}


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


def cpu_baseline(cfg, n_solves, threads=None):
    """The oracle (NumPy restatement of the reference path) on the host cores."""
    from oracle import rcwa_oracle as O
    hu, hv = cfg['orders']
    t0 = time.perf_counter()
    conv = O.to_conv_mat_raster_sampled(cfg['eps'], hu, hv)
    ta = time.perf_counter() - t0
    t0 = time.perf_counter()
    for i in range(n_solves):
        O.solve_stack(cfg['eps'], cfg['thickness'], float(cfg['wavelengths'][i]), cfg['period'], hu, hv,
                      0.0, 0.0, cfg['eps_top'], cfg['eps_bot'], 's', conv=conv)
    dt = time.perf_counter() - t0
    return {'value': n_solves / dt, 'unit': UNIT, 'cores': threads or os.cpu_count(), 'kind': 'port',
            'sample': f'{n_solves} wavelengths of the sweep (oracle/rcwa_oracle.py, NumPy complex128, '
                      f'stage A {ta:.2f}s once, not counted), {dt:.1f}s'}


def run_reference(args, world, rank):
    if rank != 0:
        return
    from wavebit_gb300 import workloads as WL
    cfg = WL.crossed_sweep()
    n = max(1, args.ref_sample)
    times = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(cfg, n)
        if i >= args.warmup:
            times.append(n / r['value'])
    per_step = statistics.mean(times)
    value = n / per_step
    line = {'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': args.gpus,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': per_step * 1e3,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'c128',
            'data': 'synthetic', 'config': _config('double', 'reference', n),
            'cpu_baseline': {'value': value, 'unit': UNIT, 'cores': os.cpu_count(), 'kind': 'port',
                             'sample': f'{n} wavelengths of the sweep per step (oracle/rcwa_oracle.py, '
                                       'the NumPy restatement of the reference path; the reference '
                                       'package is pure Python and absent on the GPU host)'},
            'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def hbm_peak():
    """Measured HBM copy bandwidth of the GB300s (GB/s), or the 6.8 TB/s fallback."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'MEASURED_PEAKS.json')
    try:
        with open(path) as f:
            return float(json.load(f)['hbm_gbs'])
    except (OSError, KeyError, ValueError):
        return 6800.0


def fp64_peak(torch, dev):
    """cuBLAS DGEMM 4096^3 rate measured now (the FP64 roofline denominator)."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    b = torch.randn_like(a)
    a @ b
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(); a @ b; e.record(); e.synchronize()
        best = max(best, 2 * 4096 ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    return best


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=3)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--precision', default='double', choices=['double', 'mixed', 'mixed_fp32', 'mixed_df64', 'mixed_df64_eig'])
    ap.add_argument('--workload', default='crossed_sweep', choices=['crossed_sweep', 'mixed_sweep'])
    ap.add_argument('--solves', type=int, default=128)
    ap.add_argument('--ref-sample', type=int, default=4)
    ap.add_argument('--no-cpu-baseline', action='store_true')
    args = ap.parse_args()
    world, rank, local = _dist()
    if args.impl == 'reference':
        return run_reference(args, world, rank)

    import torch
    import torch.distributed as dist
    from wavebit_gb300 import _lib, engine as E, workloads as WL
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    if world > 1:
        dist.init_process_group('nccl')
    if args.workload == 'crossed_sweep':
        cfg = WL.crossed_sweep(n_wavelengths=args.solves)
    else:
        cfg = WL.mixed_sweep()
        keep = np.linspace(0, len(cfg['wavelengths']) - 1, args.solves).round().astype(int)
        for k in ('wavelengths', 'thetas', 'phis'):
            cfg[k] = cfg[k][keep]
    hu, hv = cfg['orders']
    B = args.solves
    L = cfg['eps'].shape[0]
    handle = _lib.handle(local)
    eps_host = np.ascontiguousarray(cfg['eps'])
    li = np.tile(np.arange(L, dtype=np.int32), (B, 1))
    th = np.tile(cfg['thickness'], (B, 1))
    wl = cfg['wavelengths']
    per = np.tile(cfg['period'], (B, 1))
    zeros = np.zeros(B)
    thetas = np.asarray(cfg['thetas'], dtype=np.float64)
    et, eb = np.full(B, cfg['eps_top'], complex), np.full(B, cfg['eps_bot'], complex)
    pol = np.tile(np.array(WL.pol_pair('s'), complex), (B, 1))
    # inputs resident in HBM
    conv = E.assemble(torch.as_tensor(eps_host, device=dev), hu, hv, handle=handle)
    inp = E.BatchInputs(li, th, wl, per, thetas, zeros, et, eb, pol, device=dev)
    N = E.n_orders(hu, hv)
    out = (torch.empty((B, 3, N), dtype=torch.float64, device=dev), torch.empty((B, 3, N), dtype=torch.float64, device=dev),
           torch.zeros(B, dtype=torch.int32, device=dev), None)

    def step():
        return E.solve_batch(conv, inp, precision=args.precision, handle=handle, out=out)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    barrier()
    stream = torch.cuda.current_stream()
    launches0 = handle.launches()
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
    t = ev0.elapsed_time(ev1) / 1e3
    # the metric compares the mixed form with the FP64 one: every line carries both, timed with
    # CUDA events on the same batch (the other form over max(1, steps) steps after one warm-up),
    # and the max |dR,T| between them
    mixed_vs_fp64 = None
    if rank == 0:
        other = 'mixed' if args.precision == 'double' else 'double'
        R0, T0 = out[0].clone(), out[1].clone()
        E.solve_batch(conv, inp, precision=other, handle=handle)
        torch.cuda.synchronize()
        n_other = max(1, args.steps)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(torch.cuda.current_stream())
        for _ in range(n_other):
            R1, T1, st1 = E.solve_batch(conv, inp, precision=other, handle=handle)
        e1.record(torch.cuda.current_stream())
        torch.cuda.synchronize()
        t1 = e0.elapsed_time(e1) / 1e3 / n_other
        d = max(float((R0.view(B, 3, -1) - R1.view(B, 3, -1)).abs().max()),
                float((T0.view(B, 3, -1) - T1.view(B, 3, -1)).abs().max()))
        t_self = t / args.steps
        t64, tmx = (t_self, t1) if args.precision == 'double' else (t1, t_self)
        mixed_vs_fp64 = {'fp64_value': B / t64, 'fp64_ms_per_step': t64 * 1e3,
                         'mixed_value': B / tmx, 'mixed_ms_per_step': tmx * 1e3, 'speedup': t64 / tmx,
                         'mixed_form': 'mixed' if args.precision == 'double' else args.precision,
                         'max_abs_dRT': d, 'target': 1e-6, 'within_target': d <= 1e-6}
    t = max_over_ranks(t, world, dist, dev)
    value = whole_job_rate(world, B, args.steps, t)
    st = out[2].cpu().numpy()

    # stage-B (eigen-solve pipeline) timing for the roofline: one wb_layer_modes launch over the
    # sweep's P = B*L (solve, layer) pairs, on the launching stream
    roof = None
    if rank == 0:
        from wavebit_gb300.adjoint import ports
        P = B * L
        kxs, kys = [], []
        for b in range(B):
            pv = ports(float(wl[b]), cfg['period'], float(thetas[b]), 0.0, cfg['eps_top'], cfg['eps_bot'], hu, hv, 'cpu')
            for _ in range(L):
                kxs.append(pv['kx'].numpy()); kys.append(pv['ky'].numpy())
        kxs, kys = np.array(kxs), np.array(kys)
        pl = np.tile(np.arange(L), B)
        E.layer_modes(conv, pl, kxs, kys, handle=handle)   # warm
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        E.layer_modes(conv, pl, kxs, kys, handle=handle)
        e1.record(stream)
        torch.cuda.synchronize()
        tb = e0.elapsed_time(e1) / 1e3
        n = 2 * N
        flops = P * (4 + 100 + 8) * n ** 3            # per pair: Omega^2 4n^3 + eig 100n^3 + V 8n^3
        peak = fp64_peak(torch, dev)
        roof = {'bound': 'tensor', 'pipe': 'fp64 (DFMA; DMMA runs at the same rate on GB300)',
                'kernel': 'stage B: wb_layer_modes (Omega^2 GEMM, Hessenberg, shifted QR, back-substitution, V GEMM)',
                'achieved': flops / tb / 1e12, 'peak': peak, 'unit': 'TFLOP/s', 'frac': flops / tb / 1e12 / peak,
                'peak_source': 'cuBLAS DGEMM 4096^3 measured in this run (MEASURED_PEAKS.json has no FP64 entry)',
                'flops_per_launch': flops, 'launch_ms': tb * 1e3, 'traffic': None,
                'whole_step': {'achieved': (280 * L + 192) * n ** 3 * B / (t / args.steps) / 1e12,
                               'unit': 'TFLOP/s', 'flops_convention': '(280 L + 192) n^3 per solve'}}

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
        hbm = hbm_peak()
        stage_a = {'layers': L, 'ms': ta * 1e3, 'bytes': nbytes, 'achieved_GBps': nbytes / ta / 1e9,
                   'hbm_peak_GBps': hbm, 'frac': nbytes / ta / 1e9 / hbm if hbm else None,
                   'note': 'latency bound (direct DFT, Toeplitz inverses and two N x N inverses per layer); '
                           'runs once per stack and is cached across the sweep'}

    # energy balance |1 - sum R - sum T| for lossless stacks (no absorbing layer)
    energy = None
    if rank == 0 and not np.any(np.imag(eps_host)):
        Rs, Ts = out[0].view(B, 3, -1).sum(-1), out[1].view(B, 3, -1).sum(-1)
        energy = float((1.0 - Rs - Ts).abs().max())

    # end to end through the C ABI with host buffers (copies in, stage A, solve, copies out)
    e2e = None
    if rank == 0:
        E.solve_host(eps_host, li, th, wl, per, thetas, zeros, et, eb, pol, hu, hv, precision=args.precision,
                     handle=handle)
        te = []
        for _ in range(max(1, min(args.steps, 2))):
            t0 = time.perf_counter()
            R_h, T_h, st_h = E.solve_host(eps_host, li, th, wl, per, thetas, zeros, et, eb, pol, hu, hv,
                                          precision=args.precision, handle=handle)
            te.append(time.perf_counter() - t0)
        h2d = (eps_host.nbytes + li.nbytes + th.nbytes + wl.nbytes + per.nbytes + 2 * zeros.nbytes + et.nbytes
               + eb.nbytes + pol.nbytes)
        d2h = R_h.nbytes + T_h.nbytes + st_h.nbytes
        e2e = {'value': B / statistics.mean(te), 'unit': UNIT, 'h2d_bytes_per_step': int(h2d),
               'd2h_bytes_per_step': int(d2h), 'entry': 'wb_solve_host (C ABI, host buffers)'}

    if rank == 0:
        line = {'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
                'warmup': args.warmup, 'ms_per_step': t / args.steps * 1e3, 'higher_is_better': True,
                'scaling': 'weak', 'vs_baseline': None, 'dtype': 'c128' if args.precision == 'double' else 'c128+c64',
                'data': 'synthetic', 'config': _config(args.precision, 'gb300', B, args.workload), 'e2e': e2e,
                'gpu_launches': int(launches), 'roofline': roof, 'clocks': clk,
                'status_nonzero': int((st & ~8).astype(bool).sum()), 'grazing_flags': int(((st & 8) != 0).sum()),
                'mixed_vs_fp64': mixed_vs_fp64, 'stage_a': stage_a, 'energy_balance_max': energy}
        if not args.no_cpu_baseline and world == 1:
            line['cpu_baseline'] = cpu_baseline(cfg, args.ref_sample)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
