"""The continuous-batching loop's scheduling, on a fake backend (CPU) and on the GPU."""
import collections

import numpy as np
import pytest

from wavebit_gb300.serving import Request, Server


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 1e-4          # every look at the clock advances it a little
        return self.t


class FakeBackend:
    """Deterministic stand-in: a batch takes `cost` seconds per request; R = id, T = 1 - id."""

    def __init__(self, clock, limit=4, cost=0.01, poisoned=(), refuse=()):
        self.clock, self.limit, self.cost = clock, limit, cost
        self.poisoned, self.refuse = set(poisoned), set(refuse)
        self.batches = []

    def max_batch(self, orders, L, cap):
        return 0 if (orders, L) in self.refuse else min(cap, self.limit)

    def launch(self, worker, reqs):
        start = self.clock()
        tok = dict(end=start + self.cost * len(reqs), reqs=reqs, worker=worker, start=start)
        self.batches.append(tok)
        return tok

    def done(self, tok):
        return self.clock() >= tok['end']

    def results(self, tok):
        ids = np.array([r.id for r in tok['reqs']], float)
        st = np.array([1 if r.id in self.poisoned else 0 for r in tok['reqs']], np.int32)
        return ids[:, None], 1 - ids[:, None], st


def _reqs(n, rate=200.0, seed=0, buckets=((1, 1), (2, 2))):
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    out = []
    for i in range(n):
        o = buckets[int(rng.integers(0, len(buckets)))]
        L = 1 + int(rng.integers(0, 2))
        out.append(Request(i, np.ones((L, 4, 4)), np.full(L, 100.0), o, (500., 500.), 600.0, 0.0, 0.0, 's',
                           arrival=float(t[i])))
    return out


def test_every_request_completes_in_buckets_within_limits():
    clock = FakeClock()
    be = FakeBackend(clock, limit=4)
    res, st = Server(be, n_workers=3, max_batch=8, clock=clock, idle_sleep=0).run(_reqs(60))
    assert st['completed'] == 60 and st['errors'] == 0
    for tok in be.batches:
        assert 1 <= len(tok['reqs']) <= 4
        assert len({r.bucket for r in tok['reqs']}) == 1
    for rid, r in res.items():
        assert float(r.R[0]) == rid and float(r.T[0]) == 1 - rid


def test_requests_are_admitted_while_others_run():
    clock = FakeClock()
    be = FakeBackend(clock, limit=2, cost=0.05)
    Server(be, n_workers=3, max_batch=8, clock=clock, idle_sleep=0).run(_reqs(30, rate=100.0))
    # some batch starts while another worker's batch is still running
    overlaps = sum(1 for a in be.batches for b in be.batches
                   if a is not b and a['worker'] != b['worker'] and a['start'] < b['start'] < a['end'])
    assert overlaps > 0


def test_a_poisoned_request_fails_alone():
    clock = FakeClock()
    be = FakeBackend(clock, limit=8, poisoned={5})
    res, st = Server(be, n_workers=2, max_batch=8, clock=clock, idle_sleep=0).run(_reqs(20))
    assert res[5].error is not None and res[5].R is None
    assert st['errors'] == 1 and st['completed'] == 19
    mates = [r for tok in be.batches if any(q.id == 5 for q in tok['reqs']) for r in tok['reqs'] if r.id != 5]
    assert all(res[r.id].error is None for r in mates)


class RaisingBackend(FakeBackend):
    """Raises from launch whenever a listed request is in the batch (an input the library refuses)."""

    def launch(self, worker, reqs):
        if any(r.id in self.poisoned for r in reqs):
            raise RuntimeError('wb_solve_batch: refused')
        return super().launch(worker, reqs)


def test_a_batch_whose_launch_raises_is_taken_apart():
    clock = FakeClock()
    be = RaisingBackend(clock, limit=8, poisoned={7})
    res, st = Server(be, n_workers=2, max_batch=8, clock=clock, idle_sleep=0).run(_reqs(24))
    assert res[7].error is not None and res[7].status == -2 and 'refused' in res[7].error
    assert st['errors'] == 1 and st['completed'] == 23
    assert all(res[i].error is None and res[i].R[0] == i for i in range(24) if i != 7)


class FallbackBackend(FakeBackend):
    """Fails the listed requests' first attempt (status 2); their retry, run in the fallback
    precision, succeeds."""
    fallback_precision = 'mixed_df64_eig'

    def results(self, tok):
        ids = np.array([r.id for r in tok['reqs']], float)
        st = np.array([2 if (r.id in self.poisoned and not r.retry) else 0 for r in tok['reqs']], np.int32)
        return ids[:, None], 1 - ids[:, None], st


def test_a_failed_mixed_solve_is_solved_again_in_the_fallback_precision():
    clock = FakeClock()
    be = FallbackBackend(clock, limit=4, poisoned={5, 17})
    res, st = Server(be, n_workers=2, max_batch=8, clock=clock, idle_sleep=0).run(_reqs(30))
    assert st['completed'] == 30 and st['errors'] == 0 and st['fallbacks'] == 2
    for rid in (5, 17):
        assert res[rid].error is None and float(res[rid].R[0]) == rid
    # a retry runs in a batch of retries only
    for tok in be.batches:
        assert len({r.retry for r in tok['reqs']}) == 1


def test_requests_that_cannot_fit_are_refused_not_queued():
    clock = FakeClock()
    be = FakeBackend(clock, refuse={((2, 2), 2)})
    reqs = _reqs(40)
    res, st = Server(be, n_workers=2, clock=clock, idle_sleep=0).run(reqs)
    refused = [r for r in reqs if r.bucket == ((2, 2), 2)]
    assert refused and all(res[r.id].error.startswith('refused') for r in refused)
    assert st['completed'] == 40 - len(refused)


@pytest.mark.gpu
def test_each_result_is_the_same_alone_and_in_the_mix():
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300.serving import GpuBackend, _stream
    reqs = _stream(24, rate=400.0, seed=9, orders=[(2, 2), (3, 3)], max_layers=3, sides=(32,))
    mixed, st = Server(GpuBackend(3, 8 << 30), n_workers=3, max_batch=8).run(reqs)
    assert st['completed'] == 24
    for r in reqs[:8]:
        alone, _ = Server(GpuBackend(1, 4 << 30), n_workers=1, max_batch=1).run(
            [Request(r.id, r.eps, r.thickness, r.orders, r.period, r.wavelength, r.theta, r.phi, r.pol,
                     r.eps_top, r.eps_bot)],
            realtime=False)
        a, m = alone[r.id], mixed[r.id]
        scale = max(np.abs(a.R).max(), np.abs(a.T).max())
        assert np.abs(a.R - m.R).max() <= 1e-12 * scale and np.abs(a.T - m.T).max() <= 1e-12 * scale


@pytest.mark.gpu
@pytest.mark.parametrize('precision,tol', [('double', 1e-12), ('mixed', 1e-9)])
def test_resident_eigenpairs_are_reused_and_give_the_same_results(precision, tol):
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300.serving import GpuBackend, _stream, _repeat
    reqs = _repeat(_stream(12, rate=400.0, seed=13, orders=[(2, 2), (3, 3)], max_layers=3, sides=(32,)), 2, 400.0)
    ref, st0 = Server(GpuBackend(2, 6 << 30, 'double'), n_workers=2, max_batch=8).run(reqs)
    be = GpuBackend(2, 6 << 30, precision, eig_cache=True)
    got, st = Server(be, n_workers=2, max_batch=8).run(reqs)
    assert st['completed'] == len(reqs) and st0['completed'] == len(reqs)
    assert be.eig_hits > 0 and be.eig_misses > 0
    for r in reqs:
        a, m = ref[r.id], got[r.id]
        assert np.abs(a.R - m.R).max() <= tol and np.abs(a.T - m.T).max() <= tol, r.id


@pytest.mark.gpu
@pytest.mark.parametrize('precision', ['double', 'mixed'])
def test_captured_batches_replay_to_the_eager_results(precision):
    """With graphs on, every batch shape is solved eagerly once, captured, and replayed for the
    later batches of that shape; the replayed results equal the eager loop's."""
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from wavebit_gb300.serving import GpuBackend, _repeat, _stream
    reqs = _repeat(_stream(8, rate=400.0, seed=17, orders=[(3, 3)], max_layers=2, sides=(32,)), 4, 400.0)
    ref, st0 = Server(GpuBackend(1, 6 << 30, precision), n_workers=1, max_batch=2).run(reqs, realtime=False)
    be = GpuBackend(1, 6 << 30, precision, graphs=True)
    got, st = Server(be, n_workers=1, max_batch=2).run(reqs, realtime=False)
    assert st['completed'] == len(reqs) and st0['completed'] == len(reqs)
    assert be.graph_captures >= 1 and be.graph_replays >= 1 and not be.graph_refused
    for r in reqs:
        a, m = ref[r.id], got[r.id]
        scale = max(np.abs(a.R).max(), np.abs(a.T).max())
        assert np.abs(a.R - m.R).max() <= 1e-12 * scale and np.abs(a.T - m.T).max() <= 1e-12 * scale, r.id
