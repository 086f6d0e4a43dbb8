"""Continuous-batching request loop for RCWA solves on one GPU.

Requests (a raster stack, orders, wavelength, angles, polarization) arrive over time. The loop
keeps a pool of workers, each with its own CUDA stream and its own libwbgpu.so handle (so each
has its own scratch arena, sized from the HBM budget). Whenever a worker is free it takes the
oldest waiting request's bucket — requests with the same orders and layer count — packs up to
the bucket's batch limit into one ``wb_solve_batch`` launch sequence and starts it; requests
that arrive while others are on the GPU are admitted as soon as a worker and memory free up,
and the workers' batches overlap on the device.

* Admission: a bucket's batch limit is the largest batch whose workspace
  (``wb_workspace_bytes`` of the serving precision) fits one worker's share of the budget; a request that cannot
  fit even alone is refused with an error result (it never blocks the queue).
* Resident convolution matrices: stage A runs once per distinct raster (keyed by its bytes and
  the orders) and the result stays on the device in an LRU cache charged to the budget.
* Resident eigenpairs (``--eig-cache``): the per-layer modes of every (layer, wavelength,
  k-parallel) stay on the device; a batch runs the eigen-solve only for pairs not seen before and
  then stage C alone (``wb_smm_solve``).
* A request whose solve reports a non-zero status (singular, non-convergent, non-finite) gets an
  error result; the other requests of its batch keep theirs. In the mixed form it is first solved
  once more with the double-float eigen-solve. A batch whose launch raises is taken apart and its
  requests launched one at a time, so the one at fault gets the error result (status -2) alone.

The solver is a small interface (``GpuBackend`` here; the CPU tests pass a fake one), so the
scheduling logic is tested without a GPU. ``python -m wavebit_gb300.serving`` replays a seeded
request stream with Poisson arrivals and prints throughput and p50/p99 latency.
"""
import argparse
import collections
import hashlib
import json
import math
import time

import numpy as np

Result = collections.namedtuple('Result', 'id R T status error latency')


class Request:
    __slots__ = ('id', 'eps', 'thickness', 'orders', 'period', 'wavelength', 'theta', 'phi', 'pol',
                 'eps_top', 'eps_bot', 'arrival', 'start', 'layer_keys', 'retry')

    def __init__(self, id, eps, thickness, orders, period, wavelength, theta, phi, pol, eps_top=1.0,
                 eps_bot=1.0, arrival=0.0):
        self.id = id
        self.eps = np.ascontiguousarray(eps, dtype=np.complex128)      # (L, ny, nx), entry face first
        self.thickness = np.asarray(thickness, dtype=np.float64)
        self.orders = tuple(int(v) for v in orders)
        self.period = tuple(float(v) for v in period)
        self.wavelength = float(wavelength)
        self.theta = float(theta)
        self.phi = float(phi)
        self.pol = pol
        self.eps_top = complex(eps_top)
        self.eps_bot = complex(eps_bot)
        self.arrival = float(arrival)
        self.start = None
        self.layer_keys = None
        self.retry = False

    @property
    def bucket(self):
        return (self.orders, self.eps.shape[0])

    @classmethod
    def from_workload(cls, r):
        return cls(r['id'], r['eps'], r['thickness'], r['orders'], r['period'], r['wavelength'], r['theta'],
                   r['phi'], r['pol'], r.get('eps_top', 1.0), r.get('eps_bot', 1.0), r.get('arrival', 0.0))


def _pol_pair(pol):
    if isinstance(pol, str):
        return (1.0 + 0j, complex(math.cos(math.pi / 2))) if pol == 's' else (0j, 1.0 + 0j)
    a, b = (complex(v) for v in pol)
    nrm = math.sqrt(abs(a) ** 2 + abs(b) ** 2)
    return a / nrm, b / nrm


class GpuBackend:
    """libwbgpu.so behind the serving loop: one handle and one CUDA stream per worker."""

    def __init__(self, n_workers, hbm_budget, precision='double', device=0, eig_cache=False, coefficients='sampled',
                 tuning=None, graphs=False, max_graphs=32):
        import torch
        from . import _lib, engine
        self.torch, self.lib, self.engine = torch, _lib, engine
        # launch shapes chosen offline per bucket (wavebit_gb300/autotune.py), applied per batch
        self.tuner = None
        if tuning:
            from .autotune import Autotuner
            self.tuner = Autotuner(path=tuning)
        self.device = torch.device('cuda', device)
        torch.cuda.set_device(self.device)
        self.precision = precision
        if coefficients not in ('sampled', 'integrated'):
            raise ValueError("coefficients must be 'sampled' or 'integrated'")
        # integrated (closed-form segment) coefficients assemble each raster's compressed cell
        self.coefficients = coefficients
        # a mixed-form solve that reports a failure (a group of near-degenerate modes too large
        # for the Newton step, an FP32 QR that did not converge) is solved again with the
        # double-float eigen-solve
        self.fallback_precision = 'mixed_df64_eig' if precision == 'mixed' else None
        self.per_worker = int(hbm_budget // (n_workers + 1))          # one share for the conv cache
        self.cache_budget = int(hbm_budget - n_workers * self.per_worker)
        self.handles = [_lib.Handle(device, self.per_worker) for _ in range(n_workers)]
        for h in self.handles:                       # grow every arena now, never inside the loop
            _lib.check(h.lib.wb_reserve(h.h, self.per_worker))
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(n_workers)]
        self.cache = collections.OrderedDict()      # key -> ((3, N, N) tensor, ready event)
        self.cache_bytes = 0
        # per-layer eigenpairs kept on the device, keyed by (layer, wavelength, k-parallel): the
        # raster and orders, the wavelength, and period, angles and superstrate (which fix the
        # order wavevectors). A batch whose pairs are all present skips the eigen-solve and runs
        # stage C alone (wb_smm_solve). Charged to half of the cache share.
        self.eig_modes = {'double': 'double', 'mixed': 'mixed'}.get(precision) if eig_cache else None
        self.eig = collections.OrderedDict()        # key -> (q, W, V, ready event)
        self.eig_bytes = 0
        if self.eig_modes:
            self.eig_budget = self.cache_budget // 2
            self.cache_budget -= self.eig_budget
        self.eig_hits = self.eig_misses = 0
        # captured batches: per (worker, orders, layers, batch size, form) one CUDA graph of the
        # whole wb_solve_batch launch sequence over static device buffers, replayed for every
        # later batch of the same shape (the library allocates nothing inside a solve: the
        # worker's arena was reserved above, so the sequence is capturable)
        self.graphs = bool(graphs)
        self.max_graphs = int(max_graphs)
        self.graph_cache = collections.OrderedDict()
        self.graph_refused = set()
        self.graph_captures = self.graph_replays = 0
        self.launches0 = self.handles[0].launches()     # the library's count is process-wide

    # ---- admission
    def max_batch(self, orders, L, limit):
        hu, hv = orders
        b = limit
        while b >= 1:
            if int(self.lib.load().wb_workspace_bytes(hu, hv, L, b, self.lib.PRECISION[self.precision])) \
                    <= self.per_worker:
                return b
            b //= 2
        return 0

    # ---- resident convolution matrices
    def conv_for(self, req, worker):
        torch = self.torch
        hu, hv = req.orders
        keys = []
        for l in range(req.eps.shape[0]):
            raster = req.eps[l]
            key = (hashlib.blake2b(raster.tobytes(), digest_size=16).hexdigest(), raster.shape, hu, hv,
                   self.coefficients)
            keys.append(key)
            if key in self.cache:
                self.cache.move_to_end(key)
                continue
            edges = None
            if self.coefficients == 'integrated':
                from .rcwa import compression
                raster, x_edges, y_edges = compression(raster)
                edges = (x_edges[None], y_edges[None])
            with torch.cuda.stream(self.streams[worker]):
                cs = self.engine.assemble(torch.as_tensor(raster[None], device=self.device), hu, hv,
                                          handle=self.handles[worker], edges=edges)
                ev = torch.cuda.Event()
                ev.record(self.streams[worker])
            t = cs.buf[0]
            self.cache[key] = (t, ev)
            self.cache_bytes += t.numel() * 16
            while self.cache_bytes > self.cache_budget and len(self.cache) > 1:
                _, (old, _) = self.cache.popitem(last=False)
                self.cache_bytes -= old.numel() * 16
        return keys

    # ---- resident eigenpairs
    def _pair_key(self, layer_key, r):
        return (layer_key, r.wavelength, r.theta, r.phi, r.period, r.eps_top)

    def modes_for(self, reqs, keys_all, conv, index, worker):
        """(q, W, V) stacked over the batch's (solve, layer) pairs, computing the missing ones."""
        torch, engine = self.torch, self.engine
        from .adjoint import ports
        hu, hv = reqs[0].orders
        stream = self.streams[worker]
        pkeys = [[self._pair_key(k, r) for k in ks] for r, ks in zip(reqs, keys_all)]
        missing = list(dict.fromkeys(pk for row in pkeys for pk in row if pk not in self.eig))
        self.eig_hits += sum(1 for row in pkeys for pk in row if pk in self.eig)
        self.eig_misses += len(missing)
        if missing:
            where = {}
            for r, ks, row in zip(reqs, keys_all, pkeys):
                for k, pk in zip(ks, row):
                    where.setdefault(pk, (r, k))
            kx, ky, pl = [], [], []
            for pk in missing:
                r, k = where[pk]
                pv = ports(r.wavelength, r.period, r.theta, r.phi, r.eps_top, r.eps_bot, hu, hv, self.device)
                kx.append(pv['kx']); ky.append(pv['ky']); pl.append(index[k])
            w, q, W, V, st = engine.layer_modes(conv, pl, torch.stack(kx), torch.stack(ky),
                                                precision=self.eig_modes, handle=self.handles[worker])
            ev = torch.cuda.Event()
            for i, pk in enumerate(missing):
                entry = (q[i].clone(), W[i].clone(), V[i].clone())
                self.eig[pk] = entry + (ev,)
                self.eig_bytes += sum(t.numel() * 16 for t in entry)
            ev.record(stream)
            while self.eig_bytes > self.eig_budget and len(self.eig) > len(missing):
                _, old = self.eig.popitem(last=False)
                self.eig_bytes -= sum(t.numel() * 16 for t in old[:3])
        flat = [pk for row in pkeys for pk in row]
        for pk in dict.fromkeys(flat):
            q, W, V, ev = self.eig[pk]
            self.eig.move_to_end(pk)
            stream.wait_event(ev)
            for t in (q, W, V):
                t.record_stream(stream)
        return (torch.stack([self.eig[pk][0] for pk in flat]), torch.stack([self.eig[pk][1] for pk in flat]),
                torch.stack([self.eig[pk][2] for pk in flat]))

    # ---- captured batches
    def _graph_solve(self, worker, reqs, conv_list, inp, prec):
        """Solve the batch through this shape's CUDA graph: fill its static inputs (one slot set per
        (solve, layer), the per-solve parameters), replay it on the worker's stream and return its
        static outputs. The first batch of a shape runs eagerly on the static buffers and is then
        captured; a shape whose capture fails is solved eagerly from then on."""
        torch, engine = self.torch, self.engine
        hu, hv = reqs[0].orders
        B, L = len(reqs), reqs[0].eps.shape[0]
        key = (worker, hu, hv, L, B, prec)
        if key in self.graph_refused:
            return None
        stream = self.streams[worker]
        entry = self.graph_cache.get(key)
        fresh = entry is None
        if fresh:
            N = engine.n_orders(hu, hv)
            conv_s = engine.ConvStack(torch.empty((B * L, 3, N, N), dtype=torch.complex128, device=self.device),
                                      hu, hv)
            inp_s = engine.BatchInputs(np.arange(B * L, dtype=np.int32).reshape(B, L), inp.thickness.clone(),
                                       inp.wavelength.clone(), inp.period.clone(), inp.theta.clone(),
                                       inp.phi.clone(), inp.eps_top.clone(), inp.eps_bot.clone(), inp.pol.clone(),
                                       device=self.device)
            entry = dict(conv=conv_s, inp=inp_s, graph=None, out=None)
        conv_s, inp_s = entry['conv'], entry['inp']
        for b in range(B):
            for l in range(L):
                conv_s.buf[b * L + l].copy_(conv_list[b][l], non_blocking=True)
        for name in ('thickness', 'wavelength', 'period', 'theta', 'phi', 'eps_top', 'eps_bot', 'pol'):
            getattr(inp_s, name).copy_(getattr(inp, name), non_blocking=True)
        if not fresh:
            self.graph_cache.move_to_end(key)
            entry['graph'].replay()
            self.graph_replays += 1
            return entry['out']
        out = engine.solve_batch(conv_s, inp_s, precision=prec, handle=self.handles[worker])
        g = torch.cuda.CUDAGraph()
        try:
            with torch.cuda.graph(g, stream=stream):
                entry['out'] = engine.solve_batch(conv_s, inp_s, precision=prec, handle=self.handles[worker])
        except Exception:
            self.graph_refused.add(key)
            return out
        entry['graph'] = g
        self.graph_cache[key] = entry
        self.graph_captures += 1
        while len(self.graph_cache) > self.max_graphs:
            # the evicted shape's last replay may still run on its worker's stream: let it finish
            # before the graph is destroyed
            old_key, _ = next(iter(self.graph_cache.items()))
            self.streams[old_key[0]].synchronize()
            self.graph_cache.popitem(last=False)
        return out

    # ---- one batch
    def launch(self, worker, reqs):
        torch, engine = self.torch, self.engine
        hu, hv = reqs[0].orders
        L = reqs[0].eps.shape[0]
        N = engine.n_orders(hu, hv)
        stream = self.streams[worker]
        keys_all = [self.conv_for(r, worker) for r in reqs]
        uniq = list(dict.fromkeys(k for ks in keys_all for k in ks))
        index = {k: i for i, k in enumerate(uniq)}
        with torch.cuda.stream(stream):
            for k in uniq:                      # matrices assembled on another worker's stream
                t, ev = self.cache[k]
                stream.wait_event(ev)
                t.record_stream(stream)
            conv = engine.ConvStack(torch.stack([self.cache[k][0] for k in uniq]), hu, hv)
            li = [[index[k] for k in ks] for ks in keys_all]
            inp = engine.BatchInputs(li, [r.thickness for r in reqs], [r.wavelength for r in reqs],
                                     [r.period for r in reqs], [r.theta for r in reqs], [r.phi for r in reqs],
                                     [r.eps_top for r in reqs], [r.eps_bot for r in reqs],
                                     [_pol_pair(r.pol) for r in reqs], device=self.device)
            prec = self.fallback_precision if reqs[0].retry and self.fallback_precision else self.precision
            if self.tuner is not None:
                self.tuner.apply(self.tuner.lookup((hu, hv), L, len(reqs), prec))
            solved = None
            if self.eig_modes and not reqs[0].retry:
                q, W, V = self.modes_for(reqs, keys_all, conv, index, worker)
                solved = engine.smm_solve(W, V, q, inp, hu, hv, precision=self.precision,
                                          handle=self.handles[worker])
            elif self.graphs and not reqs[0].retry:
                slots = [[self.cache[k][0] for k in ks] for ks in keys_all]
                solved = self._graph_solve(worker, reqs, slots, inp, prec)
            if solved is None:
                solved = engine.solve_batch(conv, inp, precision=prec, handle=self.handles[worker])
            R, T, st = solved
            Rh = torch.empty(R.shape, dtype=R.dtype, pin_memory=True)
            Th = torch.empty(T.shape, dtype=T.dtype, pin_memory=True)
            sh = torch.empty(st.shape, dtype=st.dtype, pin_memory=True)
            Rh.copy_(R, non_blocking=True); Th.copy_(T, non_blocking=True); sh.copy_(st, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        return dict(event=ev, R=Rh, T=Th, status=sh, keep=(conv, inp, R, T, st))

    def done(self, token):
        return token['event'].query()

    def results(self, token):
        return token['R'].numpy()[:, 0], token['T'].numpy()[:, 0], token['status'].numpy()

    def launches(self):
        return self.handles[0].launches() - self.launches0


class Server:
    """The continuous-batching loop over a backend (see the module docstring)."""

    def __init__(self, backend, n_workers=4, max_batch=64, clock=time.perf_counter, idle_sleep=2e-4):
        self.backend = backend
        self.n_workers = n_workers
        self.max_batch_cap = max_batch
        self.clock = clock
        self.idle_sleep = idle_sleep
        self.limits = {}

    def _limit(self, bucket):
        if bucket not in self.limits:
            self.limits[bucket] = self.backend.max_batch(bucket[0], bucket[1], self.max_batch_cap)
        return self.limits[bucket]

    def run(self, requests, realtime=True):
        """Replay ``requests`` (sorted by arrival, seconds from t=0). Returns (results, stats)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        waiting = collections.OrderedDict()          # bucket -> deque of requests (FIFO)
        inflight = [None] * self.n_workers           # (token, reqs)
        results = {}
        nxt = 0
        t0 = self.clock()
        busy_batches = 0
        fallbacks = 0
        can_retry = getattr(self.backend, 'fallback_precision', None) is not None

        def now():
            return self.clock() - t0

        while len(results) < len(reqs):
            t = now()
            while nxt < len(reqs) and (not realtime or reqs[nxt].arrival <= t):
                r = reqs[nxt]
                nxt += 1
                b = r.bucket
                if self._limit(b) < 1:
                    results[r.id] = Result(r.id, None, None, -1,
                                           'refused: the request does not fit the HBM budget', 0.0)
                    continue
                waiting.setdefault(b, collections.deque()).append(r)
            progressed = False
            for w in range(self.n_workers):
                if inflight[w] is not None and self.backend.done(inflight[w][0]):
                    token, batch = inflight[w]
                    Rr, Tr, st = self.backend.results(token)
                    tdone = now()
                    for i, r in enumerate(batch):
                        err = None if (int(st[i]) & ~8) == 0 else f'solve status {int(st[i])}'
                        if err and can_retry and not r.retry:
                            # once more in the fallback precision, in a bucket of its own; its
                            # arrival time puts it at the head of the queue
                            r.retry = True
                            fallbacks += 1
                            waiting.setdefault(r.bucket + ('fallback',), collections.deque()).append(r)
                            continue
                        lat = tdone - (r.arrival if realtime else 0.0)
                        results[r.id] = Result(r.id, None if err else Rr[i], None if err else Tr[i],
                                               int(st[i]), err, lat)
                    inflight[w] = None
                    progressed = True
                if inflight[w] is None and waiting:
                    # the bucket holding the oldest waiting request
                    b = min(waiting, key=lambda k: waiting[k][0].arrival)
                    q = waiting[b]
                    take = [q.popleft() for _ in range(min(self._limit(b), len(q)))]
                    if not q:
                        del waiting[b]
                    for r in take:
                        r.start = now()
                    progressed = True
                    try:
                        token = self.backend.launch(w, take)
                    except Exception as e:
                        # a batch the backend refuses: its requests go again one per batch, so
                        # that the one at fault fails alone and the others are served
                        if len(take) > 1:
                            for r in take:
                                waiting.setdefault(r.bucket + ('alone', r.id), collections.deque()).append(r)
                        else:
                            r = take[0]
                            results[r.id] = Result(r.id, None, None, -2, f'launch failed: {e}',
                                                   now() - (r.arrival if realtime else 0.0))
                        continue
                    inflight[w] = (token, take)
                    busy_batches += 1
            if not progressed:
                if realtime and nxt < len(reqs) and not waiting and all(f is None for f in inflight):
                    gap = reqs[nxt].arrival - now()
                    if gap > 0:
                        time.sleep(min(gap, 0.01))
                else:
                    time.sleep(self.idle_sleep)
        wall = now()
        lat = np.array([r.latency for r in results.values() if r.error is None])
        ok = len(lat)
        errs = collections.Counter(r.status for r in results.values() if r.error is not None)
        stats = {'requests': len(reqs), 'completed': ok, 'errors': len(reqs) - ok,
                 'error_status_counts': {str(k): v for k, v in sorted(errs.items())}, 'wall_s': wall,
                 'throughput_rps': ok / wall if wall > 0 else 0.0, 'batches': busy_batches, 'fallbacks': fallbacks,
                 'p50_latency_s': float(np.percentile(lat, 50)) if ok else None,
                 'p99_latency_s': float(np.percentile(lat, 99)) if ok else None}
        return results, stats


def _stream(n, rate, seed, orders=None, max_layers=6, sides=(64, 128, 256)):
    from . import workloads as WL
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    out = []
    for i in range(n):
        r = WL.serving_request(rng, i, tuple(orders) if orders else WL.ORDER_CHOICES, tuple(sides), max_layers)
        r['arrival'] = float(t[i])
        out.append(Request.from_workload(r))
    return out


def _repeat(reqs, times, rate):
    """The stream replayed `times` times back to back, with new ids and later arrivals."""
    out = []
    span = (reqs[-1].arrival if reqs else 0.0) + 1.0 / rate
    for k in range(times):
        for r in reqs:
            c = Request(k * len(reqs) + r.id, r.eps, r.thickness, r.orders, r.period, r.wavelength, r.theta, r.phi,
                        r.pol, r.eps_top, r.eps_bot, r.arrival + k * span)
            out.append(c)
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument('--requests', type=int, default=256)
    ap.add_argument('--rate', type=float, default=20.0, help='Poisson arrival rate, requests/s')
    ap.add_argument('--precision', default='double', choices=['double', 'mixed', 'mixed_fp32', 'mixed_df64', 'mixed_df64_eig'])
    ap.add_argument('--workers', type=int, default=4)
    ap.add_argument('--max-batch', type=int, default=64)
    ap.add_argument('--budget-gb', type=float, default=120.0)
    ap.add_argument('--orders', default='5,8,11,15', help='half-orders drawn from (comma list)')
    ap.add_argument('--max-layers', type=int, default=6)
    ap.add_argument('--seed', type=int, default=5)
    ap.add_argument('--eig-cache', action='store_true', help='keep per-layer eigenpairs on the device')
    ap.add_argument('--coefficients', default='sampled', choices=['sampled', 'integrated'],
                    help='Li coefficients: sampled staircase or integrated segments of the compressed raster')
    ap.add_argument('--tuning', default=None, help='JSON of launch shapes per bucket (python -m wavebit_gb300.autotune)')
    ap.add_argument('--save-results', default=None,
                    help='write every request\'s R, T, status and latency to this .npz (to compare two forms)')
    ap.add_argument('--graphs', action='store_true',
                    help='replay each batch shape (orders, layers, batch size) through a captured CUDA graph')
    ap.add_argument('--repeat', type=int, default=1,
                    help='replay each request this many times (as new requests), e.g. to exercise the caches')
    args = ap.parse_args()
    orders = [(int(v), int(v)) for v in args.orders.split(',')]
    reqs = _stream(args.requests, args.rate, args.seed, orders, args.max_layers)
    if args.repeat > 1:
        reqs = _repeat(reqs, args.repeat, args.rate)
    backend = GpuBackend(args.workers, int(args.budget_gb * 2 ** 30), args.precision, eig_cache=args.eig_cache,
                         coefficients=args.coefficients, tuning=args.tuning, graphs=args.graphs)
    server = Server(backend, args.workers, args.max_batch)
    results, stats = server.run(reqs)
    if args.save_results:
        out = {}
        for r in results.values():
            if r.R is not None:
                out[f'{r.id}__R'] = np.asarray(r.R)
                out[f'{r.id}__T'] = np.asarray(r.T)
            out[f'{r.id}__status'] = np.asarray(r.status)
            out[f'{r.id}__latency'] = np.asarray(r.latency if r.latency is not None else np.nan)
        np.savez_compressed(args.save_results, **out)
    stats.update(precision=args.precision, rate=args.rate, workers=args.workers, orders=args.orders,
                 max_layers=args.max_layers, gpu_launches=backend.launches(), eig_cache=args.eig_cache,
                 eig_hits=backend.eig_hits, eig_misses=backend.eig_misses, repeat=args.repeat,
                 coefficients=args.coefficients, graphs=args.graphs, graph_captures=backend.graph_captures,
                 graph_replays=backend.graph_replays)
    print(json.dumps(stats))


if __name__ == '__main__':
    main()
