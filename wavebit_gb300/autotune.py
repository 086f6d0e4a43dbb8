"""Autotuner of the library's launch shapes and of the serving loop's batch limits.

A *bucket* is one shape of work: orders, layer count, batch size and precision form. For a bucket
the tuner times candidate settings of the launch-shape tunables that ``wb_set_tuning`` exposes:

* ``qr_threads`` (``WB_TUNE_QR_THREADS``): threads of a QR-sweep CTA;
* ``hrd_threads`` (``WB_TUNE_HRD_THREADS``): threads of a Hessenberg-reduction CTA.

It searches by coordinate descent from the library's own choice (0), one tunable at a time,
keeping a candidate only when it is faster by more than ``min_gain``. The choices are persisted
in a JSON file keyed by bucket, so that a server tunes offline and applies them at run time.
These tunables change launch shapes only, never a result. ``tune_batch_limit`` picks, among batch
sizes that fit a worker's memory share, the one with the most solves per second.

The tunables are process-wide. A server whose workers run different buckets at once applies each
bucket's choice before launching it. A concurrent launch may then run with another bucket's
shape, which costs time but never changes an answer.

    python -m wavebit_gb300.autotune --orders 12 --layers 4 --batch 38 --precision mixed --path tuning.json
"""
import argparse
import json
import os
import time

#: tunable name -> (wb_set_tuning key, candidate values; 0 is the library's own choice)
KNOBS = {
    'qr_threads': (0, (0, 256, 384, 512, 768)),
    'hrd_threads': (1, (0, 256, 512, 1024)),
}


def bucket_key(orders, layers, batch, precision):
    """The persisted key of a bucket, e.g. ``'12x12/L4/B38/mixed'``."""
    hu, hv = (int(v) for v in orders)
    return f'{hu}x{hv}/L{int(layers)}/B{int(batch)}/{precision}'


def gpu_timer(run):
    """Seconds of one ``run()``, the device synchronised on both sides."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run()
    torch.cuda.synchronize()
    return time.perf_counter() - t0


class Autotuner:
    """Timed trials per bucket, persisted choices, and their application.

    ``lib`` is the loaded library (anything with ``wb_set_tuning`` / ``wb_get_tuning``), ``timer``
    a callable timing one run (``gpu_timer`` by default), ``path`` the JSON file of choices (kept
    in memory only when None), ``repeats`` the timed runs per trial (the minimum is kept).
    """

    def __init__(self, lib=None, timer=None, path=None, repeats=1, min_gain=0.02):
        if lib is None:
            from . import _lib
            lib = _lib.load()
        self.lib = lib
        self.timer = timer or gpu_timer
        self.path = path
        self.repeats = max(1, int(repeats))
        self.min_gain = float(min_gain)
        self.table = {}
        if path and os.path.exists(path):
            with open(path) as f:
                self.table = json.load(f)

    # ---- settings
    def settings(self, key):
        """The persisted tunable settings of ``key``, or None."""
        entry = self.table.get(key)
        return dict(entry['settings']) if entry and 'settings' in entry else None

    def apply(self, settings):
        """Set the library's tunables (names absent from ``settings`` go back to 0)."""
        settings = settings or {}
        for name, (k, _) in KNOBS.items():
            rc = self.lib.wb_set_tuning(k, int(settings.get(name, 0)))
            if rc != 0:
                raise ValueError(f'wb_set_tuning({name}={settings.get(name)}) refused')

    def reset(self):
        self.apply({})

    def current(self):
        return {name: int(self.lib.wb_get_tuning(k)) for name, (k, _) in KNOBS.items()}

    def _time(self, run):
        return min(self.timer(run) for _ in range(self.repeats))

    def _save(self):
        if self.path:
            tmp = self.path + '.tmp'
            with open(tmp, 'w') as f:
                json.dump(self.table, f, indent=1, sort_keys=True)
            os.replace(tmp, self.path)

    # ---- tuning
    def tune(self, key, run, knobs=None):
        """Coordinate descent over ``knobs`` (all by default) for bucket ``key``; ``run()``
        executes one batch of the bucket. Returns the chosen settings, applied and persisted."""
        names = list(knobs or KNOBS)
        best = {name: 0 for name in KNOBS}
        self.apply(best)
        run()                                         # warm: first launches, arena growth
        t_best = self._time(run)
        trials = [{'settings': dict(best), 'seconds': t_best}]
        for name in names:
            for v in KNOBS[name][1]:
                if v == best[name]:
                    continue
                cand = dict(best, **{name: v})
                self.apply(cand)
                t = self._time(run)
                trials.append({'settings': cand, 'seconds': t})
                if t < t_best * (1.0 - self.min_gain):
                    best, t_best = cand, t
        self.apply(best)
        entry = self.table.setdefault(key, {})
        entry.update(settings=best, seconds=t_best, trials=trials)
        self._save()
        return best

    def tune_batch_limit(self, key, run_batch, batches):
        """The batch size of ``batches`` with the most solves per second: ``run_batch(b)`` runs
        one batch of ``b`` solves. Persisted as the bucket's ``batch_limit``."""
        rates = {}
        for b in batches:
            run_batch(b)                              # warm
            rates[int(b)] = b / self._time(lambda: run_batch(b))
        best = max(rates, key=lambda b: (rates[b], -b))
        entry = self.table.setdefault(key, {})
        entry.update(batch_limit=best, batch_rates={str(b): r for b, r in rates.items()})
        self._save()
        return best

    def lookup(self, orders, layers, batch, precision):
        """Settings of the tuned bucket with these orders, layers and form whose batch is
        nearest to ``batch`` (None when none was tuned)."""
        hu, hv = (int(v) for v in orders)
        prefix = f'{hu}x{hv}/L{int(layers)}/'
        best, dist = None, None
        for key, entry in self.table.items():
            if not key.startswith(prefix) or not key.endswith('/' + precision) or 'settings' not in entry:
                continue
            b = int(key[len(prefix):].split('/')[0][1:])
            if dist is None or abs(b - batch) < dist:
                best, dist = dict(entry['settings']), abs(b - batch)
        return best

    def batch_limit(self, key):
        entry = self.table.get(key)
        return int(entry['batch_limit']) if entry and 'batch_limit' in entry else None


def main():
    ap = argparse.ArgumentParser(description='Tune the launch shapes for one bucket of the orders sweep.')
    ap.add_argument('--orders', type=int, default=12)
    ap.add_argument('--layers', type=int, default=4)
    ap.add_argument('--batch', type=int, default=38)
    ap.add_argument('--precision', default='mixed')
    ap.add_argument('--path', default='tuning.json')
    ap.add_argument('--repeats', type=int, default=1)
    args = ap.parse_args()
    import numpy as np
    import torch
    from . import engine as E, workloads as WL
    cfg = WL.mixed_sweep()
    h = args.orders
    L = min(args.layers, cfg['eps'].shape[0])
    B = args.batch
    keep = np.linspace(0, len(cfg['wavelengths']) - 1, B).round().astype(int)
    conv = E.assemble(torch.as_tensor(cfg['eps'][:L], device='cuda'), h, h)
    inp = E.BatchInputs(np.tile(np.arange(L, dtype=np.int32), (B, 1)), np.tile(cfg['thickness'][:L], (B, 1)),
                        cfg['wavelengths'][keep], np.tile(cfg['period'], (B, 1)), cfg['thetas'][keep], np.zeros(B),
                        np.full(B, cfg['eps_top'], complex), np.full(B, cfg['eps_bot'], complex),
                        np.tile(np.array(WL.pol_pair('s'), complex), (B, 1)), device='cuda')
    tuner = Autotuner(path=args.path, repeats=args.repeats)
    key = bucket_key((h, h), L, B, args.precision)
    best = tuner.tune(key, lambda: E.solve_batch(conv, inp, precision=args.precision))
    print(json.dumps({'bucket': key, 'settings': best, 'seconds': tuner.table[key]['seconds'],
                      'trials': tuner.table[key]['trials']}))


if __name__ == '__main__':
    main()
