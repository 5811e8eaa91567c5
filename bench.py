"""Benchmark of the SWM time step on GB300 (one JSON line on stdout).

Workload: the nonlinear wind-driven double gyre on 1024 x 1024 cells
(dx = 5 km, beta-plane f0 = 1e-4, beta = 2e-11, H = 500 m, tau = 0.1 cos(2 pi
y/L), biharmonic viscosity 1e10 m^4/s, bottom drag 1e-7 /s, seeded coastline,
rest start), synthetic seeded inputs.  One bench step = one model time step
(swm_gpu_step + swm_gpu_advance) of the whole basin.

value: cell-steps/s of the selected path (default fused_fp32c, the FP32
compensated path) with the state resident in HBM; the L2 cache (129 MB; the
per-step working set is ~85 MB) is flushed by a 512 MB device write before
every timed step, and each step is timed with CUDA events on the library's
stream.  e2e: the same metric through the C ABI with host buffers: every step
takes that step's wind-stress rows from host memory (H2D) and returns the
FP64 domain integrals of its result to host memory (D2H), wall clock.  --impl reference times the CPU restatement of
the reference's loops (the Fortran reference cannot be built here: no Fortran
compiler) on the host cores.
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
BYTES_PER_POINT = {'fused_fp32c': 89, 'fused_fp64': 129, 'plain_fp64': 129}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=2000)
    ap.add_argument('--warmup', type=int, default=20)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--path', default='fused_fp32c', choices=['fused_fp32c', 'fused_fp64', 'plain_fp64'])
    ap.add_argument('--cells', type=int, default=1024)
    ap.add_argument('--error-steps', type=int, default=1000)
    ap.add_argument('--quick', action='store_true', help='skip the side measurements')
    ap.add_argument('--device-only', action='store_true',
                    help='only the warm-up and timed device steps (the form to run under ncu)')
    ap.add_argument('--workload', default='double_gyre',
                    choices=['double_gyre', 'ensemble', 'tracer', 'helmholtz', 'linear_rg'],
                    help='ensemble / tracer: print that measurement alone (profiling)')
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


def ours(args, rank, ws):
    import torch
    torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', '0')))
    cells = args.cells
    npts = (cells + 1) * (cells + 1)  # array points (Nx, Ny) = cells + 1: the bytes moved
    ncell = cells * cells              # cells: the unit of the metric
    case, g, drv = build_model(args.path, cells, args.warmup + args.steps)
    stream = torch.cuda.ExternalStream(g.stream())
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device='cuda')
    itt = 0
    g.run(itt, args.warmup)
    itt += args.warmup
    g.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    l0 = g.launch_count()
    t0 = time.perf_counter()
    with ClockSampler(int(os.environ.get('LOCAL_RANK', '0'))) as clk:
        ms = timed_steps(g, itt, args.steps, flush, stream)
    wall = time.perf_counter() - t0
    launches = g.launch_count() - l0
    itt += args.steps
    barrier(ws)
    step_ms = allmax(ws, float(ms.mean()))
    value = ncell * ws / (step_ms * 1e-3)
    line = {'metric': METRIC, 'value': value, 'unit': 'cell-steps/s', 'n_gpus': ws, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': step_ms, 'higher_is_better': True, 'scaling': 'weak',
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
    traffic = profiled_traffic(args.path, cells)
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
    k_e2e = min(args.steps, 1000)
    ny = case['config']['ny']
    rows_pin = torch.empty((k_e2e, ny), dtype=torch.float64).pin_memory().numpy()
    prof = case['streams'][0]['rec1'][0][:, 0]
    rows_pin[:] = prof[None, :] * (1.0 + 1e-3 * np.cos(np.arange(k_e2e) * 2e-3))[:, None]
    outs = torch.empty((k_e2e, 3), dtype=torch.float64).pin_memory().numpy()
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
                               'issued by swm_gpu_run_monitor; wall clock including the final wait; no L2 flush'}
    if rank == 0 and not args.quick:
        line.update(side_measurements(args, case, g, stream, flush, ncell))
        line['speedup_vs_fp64_plain'] = line['plain_fp64']['ms_per_step'] / step_ms
        line['ensemble'] = ensemble_measurement(args)
        line['tracer'] = tracer_measurement(args)
        line['helmholtz'] = helmholtz_measurement(args)
        line['linear_rg'] = linear_rg_measurement(args)
    if rank == 0 and ws == 1 and not args.quick:
        line['cpu_baseline'] = cpu_baseline(cells)
    g.close()
    return line


def profiled_traffic(path, cells):
    """DRAM bytes per launch of the step kernel from the committed ncu summary."""
    name = {'fused_fp32c': 'k_march', 'fused_fp64': 'k_fused'}.get(path)
    f = os.path.join(ROOT, 'profiles', '%s_double_gyre_%d.md' % (name, cells))
    if name is None or not os.path.exists(f):
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


def ensemble_measurement(args, n_members=256, steps=200, one_by_one=True, err_members=8):
    """The batched FP32 path on 256 basins of uneven sizes (Nx, Ny
    log-uniform in 64-512, Laplacian Ah = 500), against the same members
    stepped one by one on the FP64 plain path; with one_by_one, also the
    batched members' error against the FP64 plain path after
    args.error_steps steps, on err_members members spread over the sizes."""
    import torch
    from swm_gb300.host import synthetic
    from swm_gb300.host.driver import Driver
    from swm_gb300.model import GpuEnsemble, GpuModel
    err_steps = max(getattr(args, 'error_steps', 0), 12 + steps) if one_by_one else 0
    cases = synthetic.ensemble_members(n=n_members, nsteps=max(steps + 100, err_steps + 10))
    cells = sum((c['config']['nx'] - 1) * (c['config']['ny'] - 1) for c in cases)
    pts = sum(c['config']['nx'] * c['config']['ny'] for c in cases)
    ms = []
    for c in cases:
        g = GpuModel('fused_fp32c')
        Driver(c, g).init(with_diag=False)
        ms.append(g)
    ens = GpuEnsemble(ms)
    st = torch.cuda.ExternalStream(ens.stream())
    ens.run(0, 12)
    ens.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = ens.launch_count()
    a.record(st)
    ens.run(12, steps)
    b.record(st)
    ens.synchronize()
    launches = ens.launch_count() - l0
    ms_step = a.elapsed_time(b) / steps
    ints = ens.integrals()
    err = None
    if one_by_one:
        # continue the batched run to err_steps, then compare members spread
        # over the sizes with the FP64 plain path from the same start
        ens.run(12 + steps, err_steps - 12 - steps)
        ens.synchronize()
        order = sorted(range(n_members), key=lambda i: cases[i]['config']['nx'] * cases[i]['config']['ny'])
        pick = [order[round(q * (n_members - 1) / (err_members - 1))] for q in range(err_members)]
        worst = {f: {'rel_l2': 0.0, 'rel_max': 0.0} for f in ('u', 'v', 'eta')}
        for i in pick:
            ref = GpuModel('plain_fp64')
            Driver(cases[i], ref).init(with_diag=False)
            ref.run(0, err_steps)
            for f in ('u', 'v', 'eta'):
                m = ref.ocean(f).astype(bool)
                a, b = ms[i].field(f)[m], ref.field(f)[m]
                den = max(float(np.linalg.norm(b)), 1e-300)
                worst[f]['rel_l2'] = max(worst[f]['rel_l2'], float(np.linalg.norm(a - b)) / den)
                worst[f]['rel_max'] = max(worst[f]['rel_max'],
                                          float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)))
            ref.close()
        err = {'steps': err_steps, 'members': len(pick),
               'sizes': [[cases[i]['config']['nx'], cases[i]['config']['ny']] for i in pick],
               'worst_over_members': worst}
    out = {'members': n_members, 'cells': cells, 'array_points': pts, 'steps': steps,
           'ms_per_step': ms_step, 'value': cells / (ms_step * 1e-3), 'unit': 'cell-steps/s',
           'rows_per_strip': ens.rows(), 'gpu_launches': launches,
           'l2': 'not flushed: the ensemble state (%.2f GB) is larger than L2' % (89 * pts / 1e9),
           'finite_integrals': bool(np.isfinite(ints).all())}
    if err is not None:
        out['fp32c_error_vs_fp64'] = err
    peak, kind = peaks()
    ach = 89 * pts / (ms_step * 1e-3) / 1e9
    out['roofline'] = {'bound': 'hbm', 'achieved': ach, 'peak': peak, 'unit': 'GB/s', 'frac': ach / peak,
                       'peak_kind': kind, 'kernel': 'k_march_ens<1>', 'bytes_per_point': 89}
    ens.close()
    for g in ms:
        g.close()
    if not one_by_one:
        return out
    # the same members one by one on the FP64 plain path (3 steps each, after start-up)
    tot = 0.0
    for c in cases:
        g = GpuModel('plain_fp64')
        Driver(c, g).init(with_diag=False)
        g.run(0, 3)
        g.synchronize()
        t0 = time.perf_counter()
        g.run(3, 3)
        g.synchronize()
        tot += (time.perf_counter() - t0) / 3
        g.close()
    out['plain_fp64_one_by_one'] = {'ms_per_step': tot * 1e3, 'value': cells / tot, 'unit': 'cell-steps/s',
                                    'timing': 'wall clock per member, summed'}
    out['speedup_vs_plain_fp64_one_by_one'] = tot * 1e3 / ms_step
    return out


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


def cpu_baseline(cells, budget_s=15.0):
    """The FP64 CPU restatement (oracle) on the same basin, all host cores."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    from oracle import OracleBackend
    from swm_gb300.host import synthetic
    from swm_gb300.host.driver import Driver
    case = synthetic.double_gyre(cells, biharmonic=True, nsteps=100)
    o = OracleBackend()
    Driver(case, o).init(with_diag=False)
    o.run_steady(2)
    n, t = 0, 0.0
    t0 = time.perf_counter()
    while t < budget_s and n < 200:
        o.run_steady(1)
        n += 1
        t = time.perf_counter() - t0
    return {'value': cells * cells * n / t, 'unit': 'cell-steps/s', 'cores': os.cpu_count(), 'kind': 'port',
            'sample': '%d model steps of the %dx%d basin (FP64 C restatement, OpenMP)' % (n, cells, cells)}


def reference(args, rank, ws):
    """CPU restatement of the reference loops, timed on the host cores."""
    if rank != 0:
        return None
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    from oracle import OracleBackend
    from swm_gb300.host import synthetic
    from swm_gb300.host.driver import Driver
    strip = 64
    case = synthetic.double_gyre((args.cells, strip), biharmonic=True, nsteps=args.warmup + args.steps)
    o = OracleBackend()
    Driver(case, o).init(with_diag=False)
    o.run_steady(args.warmup)
    t0 = time.perf_counter()
    o.run_steady(args.steps)
    t = time.perf_counter() - t0
    v = args.cells * strip * args.steps / t
    sample = 'one model step per bench step on a %dx%d-cell strip of the basin (same physics)' % (args.cells, strip)
    return {'metric': METRIC, 'value': v, 'unit': 'cell-steps/s', 'n_gpus': ws, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': t / args.steps * 1e3, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'impl': 'reference',
            'config': {'workload': 'double_gyre_%dx%d_biharmonic' % (args.cells, args.cells)},
            'cpu_baseline': {'value': v, 'unit': 'cell-steps/s', 'cores': os.cpu_count(), 'kind': 'port',
                             'sample': sample},
            'e2e': {'value': v, 'unit': 'cell-steps/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}


def main():
    args = parse()
    if args.workload != 'double_gyre':
        import torch
        torch.cuda.set_device(0)
        if args.workload == 'tracer':
            out = tracer_measurement(args, cells=args.cells, steps=args.steps,
                                     err_steps=0 if args.device_only else 1000)
        elif args.workload == 'helmholtz':
            out = helmholtz_measurement(args, cells=args.cells)
        elif args.workload == 'linear_rg':
            out = linear_rg_measurement(args)
        else:
            out = ensemble_measurement(args, steps=args.steps, one_by_one=not args.device_only)
        print(json.dumps(out))
        return
    rank, ws = dist_setup(args)
    line = reference(args, rank, ws) if args.impl == 'reference' else ours(args, rank, ws)
    if rank == 0 and line is not None:
        print(json.dumps(line))


if __name__ == '__main__':
    main()
