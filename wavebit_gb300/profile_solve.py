"""Run ``wb_solve_batch`` on a benchmark workload a fixed number of times, for profilers.

    python -m wavebit_gb300.profile_solve [--workload crossed_sweep|mixed_sweep] [--solves 128]
                                          [--precision double|mixed|...] [--calls 2]

Stage A runs once before the calls; inputs are resident on the device. Prints one line with the
status summary. Used by the ncu launch lists and captures whose summaries are kept with the
repository, so that they profile the solve alone (``bench.py`` adds its comparison and roofline
legs to the same process).
"""
import argparse

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--workload', default='crossed_sweep', choices=['crossed_sweep', 'mixed_sweep'])
    ap.add_argument('--solves', type=int, default=128)
    ap.add_argument('--precision', default='mixed')
    ap.add_argument('--calls', type=int, default=2)
    args = ap.parse_args()
    import torch
    from . import engine as E, workloads as WL
    if args.workload == 'crossed_sweep':
        cfg = WL.crossed_sweep(n_wavelengths=args.solves)
        idx = np.arange(args.solves)
    else:
        cfg = WL.mixed_sweep()
        idx = np.linspace(0, len(cfg['wavelengths']) - 1, args.solves).round().astype(int)
    hu, hv = cfg['orders']
    L = cfg['eps'].shape[0]
    B = len(idx)
    dev = torch.device('cuda', 0)
    conv = E.assemble(torch.as_tensor(cfg['eps'], device=dev), hu, hv)
    pol = np.array(WL.pol_pair('s'), complex)
    inp = E.BatchInputs(np.tile(np.arange(L, dtype=np.int32), (B, 1)), np.tile(cfg['thickness'], (B, 1)),
                        cfg['wavelengths'][idx], np.tile(cfg['period'], (B, 1)), cfg['thetas'][idx], np.zeros(B),
                        np.full(B, cfg['eps_top'], complex), np.full(B, cfg['eps_bot'], complex),
                        np.tile(pol, (B, 1)), device=dev)
    st = None
    for _ in range(args.calls):
        R, T, st = E.solve_batch(conv, inp, precision=args.precision)
    torch.cuda.synchronize()
    print(f'{args.workload} {args.precision} solves={B} calls={args.calls} '
          f'status_nonzero={int((st.cpu().numpy() & ~8).astype(bool).sum())}')


if __name__ == '__main__':
    main()
