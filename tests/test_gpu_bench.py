"""bench.py's JSON line: a short run on the GPU prints one line with every
key and type the benchmark contract names (metric, value, roofline, e2e,
launch count, clocks), and the reference arm prints its own line."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, 'bench.py'), *args], capture_output=True, text=True,
                       cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith('{')]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


def test_bench_line_carries_the_contract_keys():
    d = run_bench('--quick', '--steps', '5', '--warmup', '3', '--members', '16', '--e2e-steps', '20')
    assert d['metric'] and d['unit'] == 'cell-steps/s'
    assert d['value'] > 0 and d['ms_per_step'] > 0
    assert d['n_gpus'] == 1 and d['steps'] == 5 and d['warmup'] == 3
    assert d['higher_is_better'] is True and d['scaling'] == 'weak' and d['vs_baseline'] is None
    assert d['dtype'] and d['data'] and d['config']['workload']
    roof = d['roofline']
    assert roof['bound'] == 'hbm' and roof['unit'] == 'GB/s' and roof['achieved'] > 0 and roof['peak'] > 0
    assert abs(roof['frac'] - roof['achieved'] / roof['peak']) < 1e-9
    assert roof['traffic'] is None or roof['traffic'] > 0
    e2e = d['e2e']
    assert e2e['value'] > 0 and e2e['unit'] == d['unit']
    assert e2e['h2d_bytes_per_step'] > 0 and e2e['d2h_bytes_per_step'] > 0
    assert d['gpu_launches'] == 5
    clk = d['clocks']
    assert 'sm_mhz' in clk and 'sm_max_mhz' in clk and isinstance(clk['reasons'], list)
    assert d['config']['members'] == 16 and d['config']['rows_per_strip'] >= 16
    assert d['e2e']['steps'] == 20 and d['e2e']['d2h_bytes_per_step'] == 16 * 3 * 8


def test_single_basin_line():
    d = run_bench('--workload', 'double_gyre', '--quick', '--steps', '5', '--warmup', '3', '--cells', '256',
                  '--e2e-steps', '20')
    assert d['value'] > 0 and d['gpu_launches'] == 5 and d['roofline']['achieved'] > 0
    tiles = d['config']['step_kernel_tiles']
    assert tiles['rows_per_warp'] >= 4 and tiles['blocks'] > 0


def test_reference_arm_line():
    d = run_bench('--impl', 'reference', '--steps', '2', '--warmup', '1', '--members', '12')
    assert d['impl'] == 'reference' and d['value'] > 0 and d['unit'] == 'cell-steps/s'
    assert d['cpu_baseline']['kind'] in ('port', 'reference') and d['cpu_baseline']['cores'] >= 1
    assert d['e2e']['h2d_bytes_per_step'] == 0 and d['e2e']['d2h_bytes_per_step'] == 0
