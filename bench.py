"""Benchmark of the SWM time step on GB300 (one JSON line on stdout).

Headline workload (the metric's "FP32 batched"): an ensemble of 256
nonlinear wind-driven basins of uneven sizes (Nx, Ny log-uniform in 64-512,
dx 5-20 km, wind amplitude 0.05-0.2 N/m^2, seeded coastline, Laplacian Ah =
500 m^2/s, rest start), synthetic seeded inputs, FP32 compensated state,
stepped by one persistent launch per step.  One bench step = one model time
step (SWM_timestep + model_advance) of every member.

value: cell-steps/s of the batched path with the state resident in HBM;
the state (1.07 GB) is larger than the 129 MB L2, so no flush is needed
between steps; the K steps are timed with CUDA events on the ensemble's
stream.  e2e: the same metric through the C ABI with host buffers: every
step takes every member's wind-stress rows from pinned host memory (H2D)
and returns every member's FP64 domain integrals to pinned host memory
(D2H), swm_gpu_ensemble_run_monitor, wall clock.  Under torchrun the
members of an N x 256-member ensemble are split across the ranks by cell
count (weak scaling, no collective on the data path).

Side measurements (rank 0): the same members one by one on the FP64 plain
path (the metric's "FP64 plain"), the batched members' error against FP64
after --error-steps, the single 1024^2 double gyre, the tracer, Helmholtz,
SOR and linear reduced-gravity workloads, and the CPU restatement of the
reference's loops on a sample of the ensemble.  --impl reference times that
CPU restatement (the Fortran reference cannot be built: no Fortran compiler)
on the host cores, on the headline ensemble.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'grid-cell-steps/s on 1 GB300, FP32 batched vs FP64 plain, at stated L2 error'
_T0 = time.time()


def note(msg):
    """Progress of the run on stderr (stdout carries the one JSON line)."""
    print('[bench %7.1f s] %s' % (time.time() - _T0, msg), file=sys.stderr, flush=True)
BYTES_PER_POINT = {'fused_fp32c': 89, 'fused_fp64': 129, 'plain_fp64': 129}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=1000)
    ap.add_argument('--warmup', type=int, default=20)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--members', type=int, default=256, help='ensemble members per GPU')
    ap.add_argument('--path', default='fused_fp32c', choices=['fused_fp32c', 'fused_fp64', 'plain_fp64'],
                    help='path of the single-basin double gyre (--workload double_gyre)')
    ap.add_argument('--cells', type=int, default=1024, help='cells per side of the single-basin double gyre')
    ap.add_argument('--error-steps', type=int, default=10000)
    ap.add_argument('--e2e-steps', type=int, default=1000)
    ap.add_argument('--quick', action='store_true', help='skip the side measurements')
    ap.add_argument('--device-only', action='store_true',
                    help='only the warm-up and timed device steps (the form to run under ncu)')
    ap.add_argument('--workload', default='ensemble',
                    choices=['ensemble', 'double_gyre', 'tracer', 'helmholtz', 'linear_rg', 'sor', 'output'],
                    help='ensemble: the headline line; the others print that measurement alone')
    return ap.parse_args()


def dist_setup(args):
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group('gloo')
    return rank, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def peaks():
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d['hbm_gbs']), 'measured'
    return 6800.0, 'fallback'


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    Q = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
         'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
         'clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.gpu), '--query-gpu=' + self.Q,
                                          '--format=csv,noheader,nounits', '-lms', '50'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for l in getattr(self, 'lines', []):
            f = [x.strip() for x in l.split(',')]
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith('active'):
                    reasons.add(n)
        return {'sm_mhz': float(np.median(sm)) if sm else None, 'sm_max_mhz': mx or None,
                'reasons': sorted(reasons), 'samples': len(sm)}


def build_model(path, cells, nsteps):
    from swm_gb300.host import synthetic
    from swm_gb300.host.driver import Driver
    from swm_gb300.model import GpuModel
    case = synthetic.double_gyre(cells, biharmonic=True, nsteps=nsteps)
    g = GpuModel(path)
    d = Driver(case, g)
    d.init(with_diag=False)
    return case, g, d


def timed_steps(g, itt0, k, flush=None, stream=None):
    """Device time (ms) of each of k steps, CUDA events on the library's stream."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
    with torch.cuda.stream(stream):
        for s in range(k):
            if flush is not None:
                flush.zero_()
            ev[s][0].record(stream)
            g.run(itt0 + s, 1)
            ev[s][1].record(stream)
    g.synchronize()
    torch.cuda.synchronize()
    return np.array([a.elapsed_time(b) for a, b in ev])


def double_gyre_line(args, rank, ws, steps, warmup, side=True):
    """The single-basin double gyre (args.cells^2, biharmonic) on args.path:
    device steps with the L2 flushed before each, back-to-back steps, the
    monitored end-to-end run, and (side) the FP64 paths and the FP32 error
    against FP64 after args.error_steps."""
    import torch
    cells = args.cells
    npts = (cells + 1) * (cells + 1)  # array points (Nx, Ny) = cells + 1: the bytes moved
    ncell = cells * cells              # cells: the unit of the metric
    case, g, drv = build_model(args.path, cells, warmup + steps)
    stream = torch.cuda.ExternalStream(g.stream())
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device='cuda')
    itt = 0
    g.run(itt, warmup)
    itt += warmup
    g.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    l0 = g.launch_count()
    t0 = time.perf_counter()
    with ClockSampler(int(os.environ.get('LOCAL_RANK', '0'))) as clk:
        ms = timed_steps(g, itt, steps, flush, stream)
    wall = time.perf_counter() - t0
    launches = g.launch_count() - l0
    itt += steps
    barrier(ws)
    step_ms = allmax(ws, float(ms.mean()))
    value = ncell * ws / (step_ms * 1e-3)
    line = {'metric': METRIC, 'value': value, 'unit': 'cell-steps/s', 'n_gpus': ws, 'steps': steps,
            'warmup': warmup, 'ms_per_step': step_ms, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32' if args.path == 'fused_fp32c' else 'f64',
            'data': 'synthetic (seeded double-gyre basin, rest start)',
            'config': {'workload': 'double_gyre_%dx%d_biharmonic' % (cells, cells), 'cells': cells * cells,
                       'array_points': npts, 'path': args.path, 'dt_s': case['config']['dt'],
                       'l2': 'flushed (512 MB write) before every timed step',
                       'parallelism': 'replicas x%d' % ws if ws > 1 else 'single GPU'},
            'gpu_launches': int(launches), 'wall_s_timed_region': wall}
    if args.path == 'fused_fp32c':
        rows, cost, blocks = g.step_shape()
        line['config']['step_kernel_tiles'] = {'rows_per_warp': rows, 'masked_row_cost': cost, 'blocks': blocks}
    line['clocks'] = clk.summary()
    peak, kind = peaks()
    alg = BYTES_PER_POINT[args.path] * npts
    achieved = alg / (step_ms * 1e-3) / 1e9
    kname = {'fused_fp32c': 'k_march', 'fused_fp64': 'k_fused'}.get(args.path)
    traffic = profiled_traffic('%s_double_gyre_%d.md' % (kname, cells)) if kname else None
    line['roofline'] = {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                        'frac': achieved / peak, 'traffic': traffic, 'peak_kind': kind,
                        'algorithmic_bytes_per_launch': alg,
                        'kernel': 'k_march<2>' if args.path == 'fused_fp32c' else args.path}
    if args.device_only:
        g.close()
        return line
    # steady state without L2 flush (back-to-back steps)
    ms_nf = timed_steps(g, itt, 200, None, stream)
    itt += 200
    line['no_flush'] = {'ms_per_step': float(ms_nf.mean()), 'value': ncell / (ms_nf.mean() * 1e-3)}
    # e2e through the C ABI with host buffers: every step takes its own
    # wind-stress row profile from pinned host memory and returns the FP64
    # domain integrals of its result into pinned host memory, through
    # swm_gpu_run_monitor (one C call issues all steps; no host wait per step)
    k_e2e = args.e2e_steps
    ny = case['config']['ny']
    rows_pin = torch.empty((k_e2e, ny), dtype=torch.float64).pin_memory().numpy()
    prof = case['streams'][0]['rec1'][0][:, 0]
    rows_pin[:] = prof[None, :] * (1.0 + 1e-3 * np.cos(np.arange(k_e2e) * 2e-3))[:, None]
    outs = torch.empty((k_e2e, 3), dtype=torch.float64).pin_memory().numpy()
    # untimed warm-up steps of the same call (its first use sets up the
    # monitor's device tables)
    w_e2e = min(E2E_WARMUP, k_e2e)
    g.run_monitor(itt, w_e2e, 0, rows_pin[:w_e2e], outs[:w_e2e])
    itt += w_e2e
    g.synchronize()
    t0 = time.perf_counter()
    g.run_monitor(itt, k_e2e, 0, rows_pin, outs)
    e2e_s = time.perf_counter() - t0
    itt += k_e2e
    assert np.isfinite(outs).all()
    line['e2e'] = {'value': ncell * k_e2e / e2e_s, 'unit': 'cell-steps/s', 'h2d_bytes_per_step': ny * 8,
                   'd2h_bytes_per_step': 3 * 8, 'steps': k_e2e,
                   'per_step': "H2D: the step's wind-stress row profile, read from pinned host memory by the "
                               'step kernel before the step; swm_gpu_step + swm_gpu_advance; D2H: the FP64 '
                               'domain integrals of the new state, written into pinned host memory; all steps '
                               'issued by swm_gpu_run_monitor; wall clock including the final wait; no L2 flush; '
                               'after %d untimed monitored warm-up steps' % w_e2e}
    if rank == 0 and side:
        line.update(side_measurements(args, case, g, stream, flush, ncell))
        line['speedup_vs_fp64_plain'] = line['plain_fp64']['ms_per_step'] / step_ms
    g.close()
    return line


def profiled_traffic(fname):
    """DRAM bytes per launch of a kernel from its committed ncu summary."""
    f = os.path.join(ROOT, 'profiles', fname)
    if not os.path.exists(f):
        return None
    with open(f) as fh:
        for l in fh:
            if l.startswith('dram_bytes_per_launch:'):
                return float(l.split(':')[1])
    return None


def side_measurements(args, case, g32, stream, flush, ncell):
    """FP64 paths on the same workload, and the FP32 error against FP64."""
    out = {}
    for path, k in (('plain_fp64', 20), ('fused_fp64', 50)):
        _, g, _ = build_model(path, args.cells, 100)
        g.run(0, 3)
        ms = timed_steps(g, 3, k, flush, __import__('torch').cuda.ExternalStream(g.stream()))
        out[path] = {'ms_per_step': float(ms.mean()), 'value': ncell / (ms.mean() * 1e-3), 'steps': k}
        g.close()
    # FP32C against the bit-exact FP64 plain path from the same start, with
    # the relative L2 errors along the way (error against time)
    e = args.error_steps
    _, gp, _ = build_model('plain_fp64', args.cells, e)
    _, gc, _ = build_model('fused_fp32c', args.cells, e)
    masks = {grid: gp.ocean(grid).astype(bool) for grid in ('u', 'v', 'eta')}
    curve, done = [], 0
    for c in sorted({c for c in (1000, 2000, 5000, 10000, 20000) if c < e} | {e}):
        gp.run(done, c - done)
        gc.run(done, c - done)
        done = c
        errs = {}
        for f in ('u', 'v', 'eta'):
            m = masks[f]
            a, b = gc.field(f), gp.field(f)
            den = np.linalg.norm(b[m])
            errs[f] = {'rel_l2': float(np.linalg.norm((a - b)[m]) / den) if den > 0 else None,
                       'rel_max': float(np.abs(a - b)[m].max() / max(np.abs(b[m]).max(), 1e-300))}
        curve.append({'steps': c, **{f: errs[f]['rel_l2'] for f in errs}})
    out['fp32c_error_vs_fp64'] = {'steps': e, 'fields': errs, 'rel_l2_curve': curve}
    gp.close()
    gc.close()
    return out


def ensemble_cases(n, nsteps):
    from swm_gb300.host import synthetic
    return synthetic.ensemble_members(n=n, nsteps=nsteps)


def ensemble_models(cases):
    from swm_gb300.host.driver import Driver
    from swm_gb300.model import GpuEnsemble, GpuModel
    ms = []
    for c in cases:
        g = GpuModel('fused_fp32c')
        Driver(c, g).init(with_diag=False)
        ms.append(g)
    return ms, GpuEnsemble(ms)


def ensemble_line(args, rank, ws):
    """The headline: this rank's share of an (args.members x ws)-member
    ensemble stepped by the batched path (K device-timed steps, then
    args.e2e_steps monitored steps through the C ABI with host buffers)."""
    import torch
    from swm_gb300.host.partition import member_cells, partition_members
    torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', '0')))
    W, K = args.warmup, args.steps
    all_cases = ensemble_cases(args.members * ws, W + K + args.e2e_steps + 10)
    share = partition_members([member_cells(c) for c in all_cases], ws)[rank]
    cases = [all_cases[i] for i in share]
    cells = sum(member_cells(c) for c in cases)
    pts = sum(c['config']['nx'] * c['config']['ny'] for c in cases)
    note('ensemble: %d members, set-up' % len(cases))
    ms, ens = ensemble_models(cases)
    note('ensemble: warm-up and timed steps')
    st = torch.cuda.ExternalStream(ens.stream())
    ens.run(0, W)
    ens.synchronize()
    itt = W
    barrier(ws)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = ens.launch_count()
    t0 = time.perf_counter()
    with ClockSampler(int(os.environ.get('LOCAL_RANK', '0'))) as clk:
        with torch.cuda.stream(st):
            a.record(st)
            ens.run(itt, K)
            b.record(st)
        ens.synchronize()
        torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    launches = ens.launch_count() - l0
    itt += K
    ms_step = allmax(ws, a.elapsed_time(b) / K)
    barrier(ws)
    cells_all = allsum(ws, float(cells))
    peak, kind = peaks()
    ach = 89 * pts / (ms_step * 1e-3) / 1e9
    traffic = profiled_traffic('k_march_ens_ensemble_256.md')
    if traffic is not None:
        traffic *= pts / ENSEMBLE_256_POINTS
    line = {'metric': METRIC, 'value': cells_all / (ms_step * 1e-3), 'unit': 'cell-steps/s', 'n_gpus': ws,
            'steps': K, 'warmup': W, 'ms_per_step': ms_step, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32',
            'data': 'synthetic (seeded basins of uneven sizes, rest start)',
            'config': {'workload': 'ensemble_%d_uneven_basins_laplacian' % args.members,
                       'members_per_gpu': args.members, 'members': len(cases), 'cells': cells,
                       'array_points': pts, 'path': 'fused_fp32c batched (one persistent launch per step)',
                       'rows_per_strip': ens.rows(),
                       'l2': 'not flushed: the state (%.2f GB) is larger than the 129 MB L2' % (89 * pts / 1e9),
                       'parallelism': ('members split across %d ranks by cell count, no collective' % ws
                                       if ws > 1 else 'single GPU')},
            'gpu_launches': int(launches), 'wall_s_timed_region': wall,
            'roofline': {'bound': 'hbm', 'achieved': ach, 'peak': peak, 'unit': 'GB/s', 'frac': ach / peak,
                         'traffic': traffic, 'peak_kind': kind, 'algorithmic_bytes_per_launch': 89 * pts,
                         'kernel': 'k_march_ens<1>', 'bytes_per_point': 89},
            'clocks': clk.summary()}
    # e2e: every step takes every member's wind rows from pinned host memory
    # and returns every member's integrals into pinned host memory
    k_e2e = args.e2e_steps
    ny = [c['config']['ny'] for c in cases]
    off = np.concatenate([[0], np.cumsum(ny)]).astype(int)
    rows = torch.empty((k_e2e, int(off[-1])), dtype=torch.float64).pin_memory().numpy()
    mod = 1.0 + 1e-3 * np.cos(np.arange(k_e2e) * 2e-3)
    for i, c in enumerate(cases):
        rows[:, off[i]:off[i + 1]] = c['streams'][0]['rec1'][0][:, 0][None, :] * mod[:, None]
    outs = torch.empty((k_e2e, len(cases), 3), dtype=torch.float64).pin_memory().numpy()
    # untimed warm-up steps of the same call (its first use sets up the
    # monitor's device tables)
    w_e2e = min(E2E_WARMUP, k_e2e)
    ens.run_monitor(itt, w_e2e, rows[:w_e2e], outs[:w_e2e])
    itt += w_e2e
    ens.synchronize()
    barrier(ws)
    note('ensemble: end-to-end steps')
    t0 = time.perf_counter()
    ens.run_monitor(itt, k_e2e, rows, outs)
    e2e_s = allmax(ws, time.perf_counter() - t0)
    itt += k_e2e
    assert np.isfinite(outs).all()
    line['e2e'] = {'value': cells_all * k_e2e / e2e_s, 'unit': 'cell-steps/s',
                   'h2d_bytes_per_step': int(off[-1]) * 8, 'd2h_bytes_per_step': 3 * len(cases) * 8,
                   'steps': k_e2e,
                   'per_step': "H2D: every member's wind-stress row profile for the step (one copy from pinned "
                               'host memory); the batched step; D2H: every member\'s FP64 domain integrals '
                               '(volume, potential and kinetic energy) of the new state into pinned host memory; '
                               'all steps issued by swm_gpu_ensemble_run_monitor; wall clock including the final '
                               'wait; after %d untimed monitored warm-up steps' % w_e2e}
    ens.close()
    for g in ms:
        g.close()
    if rank == 0 and not args.quick:
        note('members one by one on the FP64 plain path')
        one = plain_one_by_one(cases)
        line['plain_fp64_one_by_one'] = one
        line['speedup_vs_plain_fp64_one_by_one'] = one['ms_per_step'] / ms_step
        note('batched error against FP64 after %d steps' % args.error_steps)
        line['fp32c_error_vs_fp64'] = ensemble_error(cases, args.error_steps)
        note('single basin')
        line['single_basin'] = double_gyre_line(args, 0, 1, 200, 5, side=True)
        note('tracer')
        line['tracer'] = tracer_measurement(args)
        note('helmholtz')
        line['helmholtz'] = helmholtz_measurement(args)
        note('sor')
        line['sor'] = sor_measurement(args)
        note('linear reduced gravity')
        line['linear_rg'] = linear_rg_measurement(args)
        note('diagnostics output')
        line['output'] = output_measurement(args)
    if rank == 0 and ws == 1 and not args.quick:
        note('cpu baseline')
        line['cpu_baseline'] = cpu_baseline(cases)
    note('done')
    return line


# array points of the 256-member ensemble the committed ncu summary covers
ENSEMBLE_256_POINTS = 12043762
E2E_WARMUP = 3  # untimed monitored steps before the timed end-to-end call


def plain_one_by_one(cases, steps=12):
    """The same members one by one on the FP64 plain path: per member, after
    the start-up and the capture of its step graph, `steps` steps (two
    six-step graph replays) timed with CUDA events on its stream; the
    members' times summed."""
    import torch
    from swm_gb300.host.driver import Driver
    from swm_gb300.model import GpuModel
    tot = 0.0
    for c in cases:
        g = GpuModel('plain_fp64')
        Driver(c, g).init(with_diag=False)
        g.run(0, 14)  # start-up, then the graph is captured and replayed
        g.synchronize()
        st = torch.cuda.ExternalStream(g.stream())
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        g.run(14, steps)
        b.record(st)
        g.synchronize()
        tot += a.elapsed_time(b) * 1e-3 / steps
        g.close()
    cells = sum((c['config']['nx'] - 1) * (c['config']['ny'] - 1) for c in cases)
    return {'ms_per_step': tot * 1e3, 'value': cells / tot, 'unit': 'cell-steps/s',
            'timing': 'CUDA events per member (%d steps after its start-up and graph capture), summed' % steps}


def ensemble_error(cases, steps, picks=8):
    """The batched path's error against the FP64 plain path from the same
    start after `steps` steps: a fresh ensemble of the same members runs
    `steps` steps; picks members spread over the sizes are compared."""
    from swm_gb300.host.driver import Driver
    from swm_gb300.model import GpuModel
    ms, ens = ensemble_models(cases)
    ens.run(0, steps)
    ens.synchronize()
    n = len(cases)
    order = sorted(range(n), key=lambda i: cases[i]['config']['nx'] * cases[i]['config']['ny'])
    pick = sorted({order[round(q * (n - 1) / max(picks - 1, 1))] for q in range(min(picks, n))})
    worst = {f: {'rel_l2': 0.0, 'rel_max': 0.0} for f in ('u', 'v', 'eta')}
    for i in pick:
        ref = GpuModel('plain_fp64')
        Driver(cases[i], ref).init(with_diag=False)
        ref.run(0, steps)
        for f in ('u', 'v', 'eta'):
            m = ref.ocean(f).astype(bool)
            x, y = ms[i].field(f)[m], ref.field(f)[m]
            den = max(float(np.linalg.norm(y)), 1e-300)
            worst[f]['rel_l2'] = max(worst[f]['rel_l2'], float(np.linalg.norm(x - y)) / den)
            worst[f]['rel_max'] = max(worst[f]['rel_max'], float(np.abs(x - y).max() / max(np.abs(y).max(), 1e-300)))
        ref.close()
    ens.close()
    for g in ms:
        g.close()
    return {'steps': steps, 'members': len(pick),
            'sizes': [[cases[i]['config']['nx'], cases[i]['config']['ny']] for i in pick],
            'worst_over_members': worst}


def ensemble_device_only(args):
    """Warm-up and K timed ensemble steps only (the form to run under ncu)."""
    import torch
    cases = ensemble_cases(args.members, args.warmup + args.steps + 10)
    ms, ens = ensemble_models(cases)
    st = torch.cuda.ExternalStream(ens.stream())
    ens.run(0, args.warmup)
    ens.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    ens.run(args.warmup, args.steps)
    b.record(st)
    ens.synchronize()
    ms_step = a.elapsed_time(b) / args.steps
    pts = sum(c['config']['nx'] * c['config']['ny'] for c in cases)
    return {'workload': 'ensemble_%d' % args.members, 'ms_per_step': ms_step, 'rows_per_strip': ens.rows(),
            'array_points': pts, 'achieved_GBps': 89 * pts / (ms_step * 1e-3) / 1e9}


def tracer_measurement(args, cells=2048, steps=200, err_steps=1000):
    """Two tracers in a steady nondivergent flow (2048^2 cells at 2.5 km,
    upwind-biased flux, kappa = 50, 30-day relaxation, dt = 60 s) on the FP32
    compensated tracer kernel; error and tracer-mass drift against the FP64
    plain tracer kernels (bit-exact with the oracle) after err_steps."""
    import torch
    from swm_gb300.host import synthetic
    from swm_gb300.host.driver import Driver
    from swm_gb300.model import GpuModel
    case = synthetic.tracer_flow(cells, nsteps=err_steps + steps + 10)
    pts = case['config']['nx'] * case['config']['ny']
    g = GpuModel('fused_fp32c', tracer_nan_guard=True)
    Driver(case, g).init(with_diag=False)
    st = torch.cuda.ExternalStream(g.stream())
    g.run(0, 6)
    g.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = g.launch_count()
    a.record(st)
    g.run(6, steps)
    b.record(st)
    g.synchronize()
    launches = g.launch_count() - l0
    ms = a.elapsed_time(b) / steps
    bpp = 78  # per point: u, v, H, mask 14 B; per tracer CH pair r/w 16, increments r2/w1 12, C0 4
    peak, kind = peaks()
    ach = bpp * pts / (ms * 1e-3) / 1e9
    out = {'workload': 'tracer_flow_%dx%d_2tracers_upwind_biased' % (cells, cells), 'cells': cells * cells,
           'array_points': pts, 'steps': steps, 'ms_per_step': ms, 'value': cells * cells / (ms * 1e-3),
           'unit': 'cell-steps/s', 'gpu_launches': launches,
           'l2': 'not flushed: the tracer state (%.0f MB) is larger than L2' % (bpp * pts / 1e6),
           'roofline': {'bound': 'hbm', 'achieved': ach, 'peak': peak, 'unit': 'GB/s', 'frac': ach / peak,
                        'peak_kind': kind, 'kernel': 'k_trc32', 'bytes_per_point': bpp}}
    g.close()
    if err_steps <= 0:
        return out
    # accuracy and mass drift against the FP64 tracer kernels from the same start
    cos = None
    res = {}
    for path in ('fused_fp32c', 'plain_fp64'):
        m = GpuModel(path, tracer_nan_guard=True)
        Driver(case, m).init(with_diag=False)
        if cos is None:
            cos = m.lat('cos_eta')[:, None]
            ocean = m.ocean('eta').astype(bool)
        mass0 = [float((m.tracer_field(t, 'CH') * cos).sum()) for t in range(2)]
        m.run(0, err_steps)
        ch = [m.tracer_field(t, 'CH') for t in range(2)]
        res[path] = (ch, [float((c * cos).sum()) / m0 - 1.0 for c, m0 in zip(ch, mass0)])
        m.close()
    errs = [float(np.linalg.norm((res['fused_fp32c'][0][t] - res['plain_fp64'][0][t])[ocean]) /
                  np.linalg.norm(res['plain_fp64'][0][t][ocean])) for t in range(2)]
    out['fp32c_error_vs_fp64'] = {'steps': err_steps, 'rel_l2_CH': errs}
    out['mass_change'] = {'steps': err_steps, 'fp32c': res['fused_fp32c'][1], 'fp64': res['plain_fp64'][1],
                          'note': 'relative change of sum(CH*cos) over the run (relaxation changes it too)'}
    return out


def helmholtz_measurement(args, cells=4096, rtol=1e-10):
    """div(H^-1 grad psi) - lam psi = rhs on 4096^2 cells at 5 km (seeded
    depth 50-5000 m, coastline, wind-curl rhs): the autotuner picks the
    relaxation factor in 1.8-1.99 and the sweep block shape; then FP64 SOR and
    mixed-precision SOR (FP32 sweeps, FP64 residual refinement) each solve to
    a relative residual of 1e-10 from psi = 0."""
    import torch
    from swm_gb300.host import synthetic
    from swm_gb300.model import GpuHelmholtz
    case = synthetic.helmholtz_case(cells)
    g = GpuHelmholtz(case['H'], case['ocean'], case['dx'], case['dy'], case['lam'])
    st = torch.cuda.ExternalStream(g.stream())
    t0 = time.perf_counter()
    om, blk = g.autotune(case['rhs'], 1.8, 1.99, 12, 64)
    t_tune = time.perf_counter() - t0
    out = {'workload': 'helmholtz_%dx%d' % (cells, cells), 'cells': cells * cells, 'lambda': case['lam'],
           'rtol': rtol, 'omega': om, 'block': list(blk), 'autotune_s': t_tune}
    peak, kind = peaks()
    for name, mixed, bps in (('fp64', False, 32), ('mixed', True, 16)):
        g.solve(case['rhs'], omega=om, rtol=1e-3, mixed=mixed)  # warm-up
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        a.record(st)
        psi, sweeps, outer, rel, rc = g.solve(case['rhs'], omega=om, rtol=rtol, mixed=mixed, inner_tol=1e-4)
        b.record(st)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        dev = a.elapsed_time(b) * 1e-3
        ach = bps * case['H'].size * sweeps / dev / 1e9
        out[name] = {'time_to_solution_s': wall, 'device_s': dev, 'sweeps': sweeps, 'outer_iterations': outer,
                     'relres': rel, 'converged': rc == 0,
                     'roofline': {'bound': 'hbm', 'achieved': ach, 'peak': peak, 'unit': 'GB/s', 'frac': ach / peak,
                                  'peak_kind': kind, 'bytes_per_cell_sweep': bps,
                                  'note': 'sweeps only counted; residual passes included in the time'}}
    out['mixed_speedup'] = out['fp64']['time_to_solution_s'] / out['mixed']['time_to_solution_s']
    g.close()
    return out


def output_measurement(args, cells=1024, steps=2000, records=4):
    """Diagnostics output while the model steps: the 1024^2 double gyre on
    the FP32 pair path with snapshot tasks of u, v and eta (`records`
    records each over `steps` steps, netCDF files in the reference's layout
    in a scratch directory), written synchronously in the time loop as the
    reference does, or by the asynchronous writer (device copies into
    pinned buffers, a writer thread), against the same steps without
    output.  Wall clock around the time loop and the writer's drain."""
    import shutil
    import tempfile
    from swm_gb300.host import synthetic
    from swm_gb300.host.driver import Driver
    from swm_gb300.host.writer import AsyncWriter
    from swm_gb300.model import GpuModel
    base = synthetic.double_gyre(cells, nsteps=steps)
    base['diag'] = [dict(filename='%s.nc' % v.lower(), varname=v, type='S', frequency=records, period=2.628e6,
                         process='A') for v in ('U', 'V', 'ETA')]
    out = {'workload': 'double_gyre_%dx%d_fp32c_snapshots' % (cells, cells), 'steps': steps,
           'records_per_field': records, 'fields': 3,
           'bytes_per_record': base['config']['nx'] * base['config']['ny'] * 8}
    tmp = tempfile.mkdtemp(prefix='swm_out_')
    try:
        for mode in ('none', 'synchronous', 'asynchronous'):
            g = GpuModel('fused_fp32c')
            w = None if mode == 'none' else AsyncWriter(os.path.join(tmp, mode), inline=(mode == 'synchronous'))
            drv = Driver(base, g, writer=w)
            drv.init(with_diag=mode != 'none')
            drv.run(10, with_diag=False)  # tuning and warm-up
            g.synchronize()
            t0 = time.perf_counter()
            drv.run(steps, with_diag=mode != 'none')
            g.synchronize()
            drv.finish()
            out['ms_per_step_' + mode] = (time.perf_counter() - t0) / steps * 1e3
            if w is not None:
                out['records_' + mode] = w.written
            g.close()
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    a, b, c = out['ms_per_step_none'], out['ms_per_step_synchronous'], out['ms_per_step_asynchronous']
    out['output_cost_hidden'] = 1.0 - (c - a) / (b - a) if b > a else None
    return out


def linear_rg_measurement(args, steps=2000, cpu_budget_s=5.0):
    """The reference's plain linear reduced-gravity configuration (256 x 128
    cells, FP64, Laplacian mixing, Rayleigh damping, AB3 dt = 1800 s) on the
    plain FP64 GPU path (bit-exact with the oracle), beside the oracle on the
    host cores; also the relative L2 of eta after the timed steps between the
    two (0 when bit-exact)."""
    import torch
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    from oracle import OracleBackend
    from swm_gb300.host import synthetic
    from swm_gb300.host.driver import Driver
    from swm_gb300.model import GpuModel
    case = synthetic.linear_rg(256, 128, nsteps=steps + 10)
    cells = 256 * 128
    g = GpuModel('plain_fp64')
    Driver(case, g).init(with_diag=False)
    g.run(0, 10)
    g.synchronize()
    st = torch.cuda.ExternalStream(g.stream())
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    g.run(10, steps)
    b.record(st)
    g.synchronize()
    ms = a.elapsed_time(b) / steps
    o = OracleBackend()
    Driver(case, o).init(with_diag=False)
    o.run_steady(10)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < cpu_budget_s and n < steps:
        o.run_steady(50)
        n += 50
    tcpu = time.perf_counter() - t0
    same = None
    if n == steps:
        same = bool(np.array_equal(o.field('eta'), g.field('eta')))
    out = {'workload': 'linear_rg_256x128_fp64', 'cells': cells, 'steps': steps, 'gpu_ms_per_step': ms,
           'gpu_value': cells / (ms * 1e-3), 'cpu_value': cells * n / tcpu, 'cpu_steps': n,
           'cpu_cores': os.cpu_count(), 'unit': 'cell-steps/s', 'bit_identical_after_timed_steps': same}
    g.close()
    return out


def oracle_ensemble(cases, warmup, steps, budget_s, threads=None):
    """The FP64 CPU restatement of the reference (oracle) stepping ensemble
    members on the host cores: a pool of `threads` host threads, each
    stepping one member at a time with OpenMP off inside the member (the
    members are independent, as the reference's one-basin-per-process runs
    are).  A bench step advances every member by one model step; when that
    would take the whole run past budget_s, each bench step advances a
    round-robin share of the members instead.  Returns (cell-steps/s, ms per
    bench step, sample description, threads)."""
    import concurrent.futures as cf
    import ctypes
    import math
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    from oracle import OracleBackend
    from swm_gb300.host.driver import Driver
    from swm_gb300.host.partition import member_cells
    threads = threads or os.cpu_count() or 1
    try:
        gomp = ctypes.CDLL('libgomp.so.1')
        init = lambda: gomp.omp_set_num_threads(1)  # noqa: E731
    except OSError:
        init = None
    n = len(cases)
    cells = [member_cells(c) for c in cases]
    order = sorted(range(n), key=lambda i: -cells[i])  # largest first keeps the pool busy to the end
    with cf.ThreadPoolExecutor(threads, initializer=init) as pool:
        def make(c):
            o = OracleBackend()
            Driver(c, o).init(with_diag=False)
            o.run_steady(2)  # Adams-Bashforth start-up (untimed)
            return o
        models = list(pool.map(make, cases))

        def advance(idx):
            list(pool.map(lambda i: models[i].run_steady(1), idx))

        t0 = time.perf_counter()
        advance(order)  # first warm-up step, also the calibration
        t_full = time.perf_counter() - t0
        per = n
        if t_full * (warmup + steps) > budget_s:
            per = min(n, max(threads, int(math.ceil(n * budget_s / (t_full * (warmup + steps))))))
        pos = 0

        def share():
            nonlocal pos
            idx = [order[(pos + k) % n] for k in range(per)]
            pos = (pos + per) % n
            return sorted(idx, key=lambda i: -cells[i])

        for _ in range(max(warmup - 1, 0)):
            advance(share())
        done, t = 0, 0.0
        for _ in range(steps):
            idx = share()
            t0 = time.perf_counter()
            advance(idx)
            t += time.perf_counter() - t0
            done += sum(cells[i] for i in idx)
    sample = ('%d members, one model step of every member per bench step' % n if per == n else
              '%d members; each bench step advances a round-robin share of %d members by one model step '
              '(bounded run time); value = member-cells advanced / time' % (n, per))
    return done / t, t / steps * 1e3, sample, threads


def cpu_baseline(cases, steps=200, budget_s=15.0):
    """The oracle on the ensemble's members, all host cores, member-parallel:
    about 10-15 s of CPU work (every member each step, or a round-robin
    share when the steps would exceed budget_s)."""
    v, _, desc, threads = oracle_ensemble(cases, 2, steps, budget_s)
    return {'value': v, 'unit': 'cell-steps/s', 'cores': threads, 'kind': 'port',
            'sample': '%d timed steps of the %d-member ensemble (%s); FP64 C restatement of the reference '
                      'loops' % (steps, len(cases), desc)}


def reference(args, rank, ws):
    """The CPU restatement of the reference's loops on the headline ensemble,
    timed on the host cores (rank 0 alone; the other ranks exit)."""
    if rank != 0:
        return None
    cases = ensemble_cases(args.members, args.warmup + args.steps + 10)
    v, ms, sample, threads = oracle_ensemble(cases, args.warmup, args.steps, budget_s=90.0)
    return {'metric': METRIC, 'value': v, 'unit': 'cell-steps/s', 'n_gpus': ws, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'impl': 'reference',
            'config': {'workload': 'ensemble_%d_uneven_basins_laplacian' % args.members},
            'cpu_baseline': {'value': v, 'unit': 'cell-steps/s', 'cores': threads, 'kind': 'port',
                             'sample': sample},
            'e2e': {'value': v, 'unit': 'cell-steps/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}


def sor_measurement(args, cells=4096, eps=1e-4):
    """The reference's own solver (main_ElSolv_SOR: masked spherical
    Laplacian, fixed Chebyshev relaxation schedule, absolute stop on the
    correction norm, eps = 1e-4 as calc_lib.h) on the 4096^2 basin (chi, B,
    the five coefficients and the reciprocal diagonal, 1.3 GB, exceed L2).  The right-hand side is a
    smooth random field of the size of a flow divergence (1e-9 /s), as
    computeVelocityPotential passes one.  A call after the first (first_guess
    false, as every call but the first from the diagnostics) is capped by the
    reference at max_count = 10 max(Nx, Ny) iterations; from chi = 0 it may
    end there unconverged, which is reported.  Roofline: 10 words per point and iteration (chi read
    and written, B, the five coefficients, the reciprocal diagonal)."""
    import torch
    from swm_gb300.host import synthetic
    from swm_gb300.host.driver import Driver
    from swm_gb300.model import GpuModel
    case = synthetic.double_gyre(cells, biharmonic=False, nsteps=10, ah=500.0)
    g = GpuModel('plain_fp64')
    Driver(case, g).init(with_diag=False)
    g.sor_init()
    ny, nx = case['config']['ny'], case['config']['nx']
    rng = np.random.default_rng(7)
    # a smooth random field (scales of a few hundred km) of divergence size
    k = np.fft.fftfreq(nx)[None, :] ** 2 + np.fft.fftfreq(ny)[:, None] ** 2
    B = np.fft.ifft2(np.fft.fft2(rng.standard_normal((ny, nx))) * np.exp(-k * (nx / 16.0) ** 2)).real
    B *= 1e-9 / max(np.abs(B).max(), 1e-300) * g.ocean('eta')
    chi0 = np.zeros_like(B)
    g.sor_solve(B, chi0, 1e30, False)  # set-up and one iteration
    st = torch.cuda.ExternalStream(g.stream())
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = g.launch_count()
    t0 = time.perf_counter()
    a.record(st)
    chi, iters, anorm = g.sor_solve(B, chi0, eps, False)
    b.record(st)
    g.synchronize()
    wall = time.perf_counter() - t0
    dev = a.elapsed_time(b) * 1e-3
    launches = g.launch_count() - l0
    it = abs(iters)
    pts = nx * ny
    peak, kind = peaks()
    ach = 10 * 8 * pts * it / dev / 1e9
    g.close()
    return {'workload': 'elsolv_sor_%dx%d' % (cells, cells), 'points': pts, 'eps': eps,
            'iterations': it, 'converged': iters > 0, 'anorm': anorm, 'max_count': 10 * max(nx, ny),
            'time_s': wall, 'device_s': dev, 'ms_per_iteration': dev / max(it, 1) * 1e3,
            'gpu_launches': launches,
            'roofline': {'bound': 'hbm', 'achieved': ach, 'peak': peak, 'unit': 'GB/s', 'frac': ach / peak,
                         'peak_kind': kind, 'bytes_per_point_iteration': 80,
                         'note': 'one iteration = a red and a black half-sweep over all points; the half-sweep '
                                 "is bound by GB300's FP64 pipe: the reference's update is FP64 arithmetic, "
                                 'its division formed from the reciprocal diagonal by Markstein corrections'}}


def main():
    args = parse()
    if args.impl == 'ours' and args.workload not in ('ensemble', 'double_gyre'):
        import torch
        torch.cuda.set_device(0)
        if args.workload == 'tracer':
            out = tracer_measurement(args, cells=args.cells if args.cells != 1024 else 2048, steps=args.steps,
                                     err_steps=0 if args.device_only else 1000)
        elif args.workload == 'helmholtz':
            out = helmholtz_measurement(args, cells=args.cells if args.cells != 1024 else 4096)
        elif args.workload == 'output':
            out = output_measurement(args)
        elif args.workload == 'sor':
            out = sor_measurement(args, cells=args.cells if args.cells != 1024 else 4096)
        else:
            out = linear_rg_measurement(args)
        print(json.dumps(out))
        return
    rank, ws = dist_setup(args)
    if args.impl == 'reference':
        line = reference(args, rank, ws)
    elif args.workload == 'double_gyre':
        import torch
        torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', '0')))
        line = double_gyre_line(args, rank, ws, args.steps, args.warmup, side=not args.quick and not args.device_only)
    elif args.device_only:
        import torch
        torch.cuda.set_device(0)
        line = ensemble_device_only(args)
    else:
        line = ensemble_line(args, rank, ws)
    if rank == 0 and line is not None:
        print(json.dumps(line))


if __name__ == '__main__':
    main()
