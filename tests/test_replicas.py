"""The bench's multi-rank host logic on the CPU: replicas timed between barriers, the whole-job
rate from the slowest rank (gloo, world size 2), and the reference arm under torchrun, where rank
0 alone runs and prints."""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip('torch')
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group('gloo', init_method=f'tcp://127.0.0.1:{port}', rank=rank, world_size=world)
    try:
        dist.barrier()
        t = bench.max_over_ranks(times[rank], world, dist, 'cpu')
        out.put((rank, t, bench.whole_job_rate(world, 128, 3, t)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_the_slowest_rank_sets_the_whole_job_rate():
    world, times = 2, [1.5, 2.5]
    ctx = mp.get_context('spawn')
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, times, out)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=60) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, value in got:
        assert t == 2.5
        assert value == pytest.approx(2 * 128 * 3 / 2.5)


def test_a_single_rank_keeps_its_own_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.25, 1) == 1.25
    assert bench.whole_job_rate(1, 128, 3, 1.25) == pytest.approx(128 * 3 / 1.25)


def test_reference_arm_under_torchrun_prints_once_from_rank_zero():
    """``torch.distributed.run --nproc-per-node 2 bench.py --impl reference``: one JSON line, from
    rank 0, on the same metric and unit as the GB300 arm; the other rank exits 0 without work."""
    env = dict(os.environ, OMP_NUM_THREADS='2', MKL_NUM_THREADS='2', OPENBLAS_NUM_THREADS='2')
    cmd = [sys.executable, '-m', 'torch.distributed.run', '--nnodes=1', '--nproc-per-node', '2',
           '--master-addr', '127.0.0.1', '--master-port', str(_free_port()), os.path.join(ROOT, 'bench.py'),
           '--impl', 'reference', '--gpus', '2', '--steps', '1', '--warmup', '0', '--workload', 'crossed_sweep']
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line['impl'] == 'reference' and line['n_gpus'] == 2 and line['unit'] == 'solves/s'
    sys.path.insert(0, ROOT)
    import bench
    want = 'reference' if bench.reference_available() else 'port'
    assert line['cpu_baseline']['kind'] == want and line['e2e']['h2d_bytes_per_step'] == 0
    assert line['steps'] == 1 and line['metric'] == bench.metric('crossed_sweep', 'double')
