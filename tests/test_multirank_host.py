"""The N > 1 host logic of bench.py on CPU ranks (gloo, world size 2): every rank
trains its own replica, the timed region's duration is the maximum over ranks,
and the whole-job throughput counts every rank's rays; under torchrun the
reference arm prints one JSON line from rank 0 and nothing from the others."""
import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=2)
    t = bench.max_over_ranks(1.0 + rank, 'cpu')    # rank 1 is the slower replica
    out[rank] = (t, bench.job_rays_per_s(dist.get_world_size(), 4096, 20, t))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_job_throughput_with_two_gloo_ranks():
    ctx = mp.get_context('spawn')
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(_free_port(), out), nprocs=2, join=True, start_method='spawn')
        res = dict(out)
    assert res[0] == res[1] == (2.0, 2 * 4096 * 20 / 2.0)


def test_single_process_aggregation_is_identity():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(3.5, 'cpu') == 3.5
    assert bench.job_rays_per_s(1, 4096, 10, 2.0) == 4096 * 10 / 2.0


def test_reference_arm_under_torchrun_prints_from_rank_zero_only():
    cmd = [sys.executable, '-m', 'torch.distributed.run', '--nnodes=1', '--nproc-per-node', '2', '--master-addr',
           '127.0.0.1', '--master-port', str(_free_port()), os.path.join(REPO, 'bench.py'), '--impl', 'reference',
           '--gpus', '2', '--steps', '1', '--warmup', '3']
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith('{')]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line['impl'] == 'reference' and line['n_gpus'] == 2 and line['value'] > 0
    assert line['e2e']['h2d_bytes_per_step'] == 0 and line['cpu_baseline']['kind'] == 'port'
