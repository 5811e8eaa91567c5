"""Multi-process paths on CPU (gloo, world size 2): bench.py's reference
arm (rank 0 alone prints the JSON line, the other ranks exit 0 without
work), the max-over-ranks timing, and the split of an ensemble's members
across ranks (each rank computes its own share; together the shares hold
every member exactly once, balanced by cells; no data-path collective)."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_reference_arm_two_ranks_gloo():
    env = dict(os.environ, OMP_NUM_THREADS='2')
    cmd = [sys.executable, '-m', 'torch.distributed.run', '--nnodes=1', '--nproc-per-node', '2',
           '--master-addr', '127.0.0.1', '--master-port', str(_free_port()), os.path.join(ROOT, 'bench.py'),
           '--impl', 'reference', '--gpus', '2', '--steps', '3', '--warmup', '3', '--members', '6']
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d['impl'] == 'reference' and d['n_gpus'] == 2 and d['value'] > 0
    assert d['e2e']['h2d_bytes_per_step'] == 0 and d['cpu_baseline']['kind'] == 'port'


def test_allmax_over_gloo_ranks():
    code = r'''
import os, sys
sys.path.insert(0, %r)
import torch.distributed as dist
import bench
rank, ws = bench.dist_setup(None)
bench.barrier(ws)
v = bench.allmax(ws, float(rank + 1))
assert v == 2.0, v
dist.destroy_process_group()
''' % ROOT
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE='2', MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port),
                   LOCAL_RANK=str(rank))
        procs.append(subprocess.Popen([sys.executable, '-c', code], env=env, cwd=ROOT,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err[-2000:]


def test_member_partition_over_gloo_ranks():
    code = r'''
import os, sys
sys.path.insert(0, %r)
import torch
import torch.distributed as dist
import bench
from swm_gb300.host.partition import member_cells, partition_members
rank, ws = bench.dist_setup(None)
cases = bench.ensemble_cases(64 * ws, 10)
cells = [member_cells(c) for c in cases]
mine = partition_members(cells, ws)[rank]
got = [None] * ws
dist.all_gather_object(got, mine)
flat = sorted(i for s in got for i in s)
assert flat == list(range(len(cases))), flat
load = [sum(cells[i] for i in s) for s in got]
assert max(load) - min(load) <= max(cells), (load, max(cells))
assert bench.allsum(ws, float(sum(cells[i] for i in mine))) == float(sum(cells))
dist.destroy_process_group()
''' % ROOT
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE='2', MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port),
                   LOCAL_RANK=str(rank))
        procs.append(subprocess.Popen([sys.executable, '-c', code], env=env, cwd=ROOT,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err[-2000:]


def test_member_partition_balance():
    from swm_gb300.host.partition import partition_members
    import random
    rnd = random.Random(3)
    for nranks in (1, 2, 3, 8):
        cells = [rnd.randint(64 * 64, 512 * 512) for _ in range(100)]
        shares = partition_members(cells, nranks)
        assert sorted(i for s in shares for i in s) == list(range(100))
        load = [sum(cells[i] for i in s) for s in shares]
        assert max(load) - min(load) <= max(cells)
    assert partition_members([5, 4, 3, 3], 2) == [[0, 3], [1, 2]]
