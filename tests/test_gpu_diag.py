"""Diagnostics formed on the device: the streamfunction (computeStreamfunction,
summed in the reference's order) bit for bit against the FP64 oracle, and the
device averaging buffers against the host averaging of the same snapshots."""
import numpy as np
import pytest

from harness import golden_case, run_case
from oracle import OracleBackend
from swm_gb300.host import synthetic
from swm_gb300.host.driver import Driver
from swm_gb300.model import GpuModel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('barotropic', [0, 1])
@pytest.mark.parametrize('path', ['plain_fp64', 'fused_fp32c'])
def test_streamfunction_bit_exact(barotropic, path):
    case = synthetic.double_gyre((48, 40), biharmonic=False, nsteps=100)
    case['config'].update(barotropic=barotropic)
    o, g = OracleBackend(), GpuModel(path)
    run_case(case, o, nsteps=100, with_diag=False)
    run_case(case, g, nsteps=100, with_diag=False)
    # the oracle's streamfunction of the GPU's own state: the same sums
    psi_g = g.streamfunction()
    psi_o = o.streamfunction(g.field('u'), g.field('v'))
    assert np.array_equal(psi_g, psi_o)
    assert np.abs(psi_g).max() > 0


def test_device_averages_equal_host_averages():
    case, _ = golden_case('test_fixed_length_output')
    outs = []
    for dev in (True, False):
        g = GpuModel('plain_fp64')
        d = Driver(case, g, device_averages=dev)
        d.init(with_diag=True)
        d.run(with_diag=True)
        outs.append(d.outputs())
    assert outs[0].keys() == outs[1].keys()
    n = 0
    for fn in outs[0]:
        ta, ra, _ = outs[0][fn]
        tb, rb, _ = outs[1][fn]
        assert np.array_equal(ta, tb), fn
        assert np.array_equal(ra, rb), fn
        n += len(ra)
    assert n > 0


def test_psi_average_on_device():
    case = synthetic.double_gyre((40, 32), biharmonic=False, nsteps=40)
    g = GpuModel('fused_fp32c')
    d = Driver(case, g)
    d.init(with_diag=False)
    acc = np.zeros((case['config']['ny'], case['config']['nx']))
    for s in range(1, 11):
        d.run(1, with_diag=False)
        g.diag_accumulate(3, 'psi', True, 2.0)
        p = g.streamfunction()
        acc = acc + 2.0 * (p * p)
    mean, cnt = g.diag_mean(3)
    assert cnt == 20.0
    assert np.array_equal(mean, acc / 20.0)


def test_async_field_copies_match_sync():
    """swm_gpu_get_field_async into pinned buffers, issued between steps and
    collected later, gives the fields get_field gives at the same points."""
    import torch
    case = synthetic.double_gyre((40, 32), biharmonic=True, nsteps=60)
    a, b = GpuModel('fused_fp32c'), GpuModel('fused_fp32c')
    for g in (a, b):
        Driver(case, g).init(with_diag=False)
    shape = (case['config']['ny'], case['config']['nx'])
    bufs, tickets, ref = [], [], []
    itt = 0
    for k in range(5):
        a.run(itt, 7)
        b.run(itt, 7)
        itt += 7
        for f in ('u', 'eta', 'psi'):
            buf = torch.empty(shape, dtype=torch.float64).pin_memory().numpy()
            bufs.append(buf)
            tickets.append(a.field_async(f, buf))
            ref.append(b.field(f))
    for t in tickets:
        a.wait(t)
        assert a.ready(t) == 1
    for buf, r in zip(bufs, ref):
        assert np.array_equal(buf, r)


def test_async_integrals_match_sync():
    import torch
    case = synthetic.double_gyre((40, 32), biharmonic=True, nsteps=60)
    a, b = GpuModel('fused_fp32c'), GpuModel('fused_fp32c')
    for g in (a, b):
        Driver(case, g).init(with_diag=False)
    bufs = [torch.empty(3, dtype=torch.float64).pin_memory().numpy() for _ in range(4)]
    tickets, ref = [], []
    for k in range(4):
        a.run(k * 5, 5)
        b.run(k * 5, 5)
        tickets.append(a.integrals_async(bufs[k]))
        ref.append(b.integrals())
    for t in tickets:
        a.wait(t)
    for buf, r in zip(bufs, ref):
        assert np.array_equal(buf, r)


@pytest.mark.parametrize('start', [0, 5])
@pytest.mark.parametrize('pinned', [True, False])
@pytest.mark.parametrize('path', ['fused_fp32c', 'plain_fp64'])
def test_run_monitor_matches_step_by_step(path, pinned, start):
    """swm_gpu_run_monitor (per-step row uploads and integrals, no host wait
    per step) gives the state of the same steps made one call at a time, bit
    for bit, and their integrals.  Pinned arrays are read and written in
    place by the kernels, pageable ones through staged copies.  On the FP32
    pair path the step kernel forms the integrals itself, in its own order:
    1e-12 of the sum's scale; elsewhere (and for a first step that prepares
    the pair path) they come from the same reduction as swm_gpu_integrals:
    bit for bit.  The rows change every step, so a step that read another
    step's rows would leave a different state."""
    import torch
    case = synthetic.double_gyre((40, 32), biharmonic=True, nsteps=60)
    a, b = GpuModel(path), GpuModel(path)
    for g in (a, b):
        Driver(case, g).init(with_diag=False)
    ny, n = case['config']['ny'], 20
    prof = case['streams'][0]['rec1'][0][:, 0]
    if pinned:
        rows = torch.empty((n, ny), dtype=torch.float64).pin_memory().numpy()
        out = torch.empty((n, 3), dtype=torch.float64).pin_memory().numpy()
    else:
        rows, out = np.empty((n, ny)), np.empty((n, 3))
    rows[:] = prof[None, :] * (1.0 + 0.1 * np.arange(n))[:, None]
    if start:
        a.run(0, start)
        b.run(0, start)
    a.run_monitor(start, n, 0, rows, out)
    for s in range(n):
        b.set_stream_rows(0, np.ascontiguousarray(rows[s]))
        b.step(start + 1 + s)
        b.advance(start + 1 + s)
        ref = b.integrals()
        if path == 'fused_fp32c' and start + s > 0:
            _, scale = _numpy_integrals(case, b)
            assert np.all(np.abs(out[s] - ref) <= 1e-12 * scale), (s, out[s], ref)
        else:
            assert np.array_equal(out[s], ref), s
    for f in ('u', 'v', 'eta'):
        assert np.array_equal(a.field(f), b.field(f))


def _numpy_integrals(case, g):
    """FP64 numpy sums of the three integrals of g's current fields, with the
    oracle's grid (cos of each point's latitude, ocean masks, dLambda,
    dTheta), and the scale of each sum's rounding error (the volume sum
    cancels: sum |eta| area)."""
    o = OracleBackend()
    Driver(case, o).init(with_diag=False)
    dl, dt = o.scalars()
    A, G = case['config']['A'], case['config']['G']
    area = {k: (A * A * o.lat('cos_' + k) * dl * dt)[:, None] for k in ('u', 'v', 'eta')}
    m = {k: o.ocean(k) == 1 for k in ('u', 'v', 'eta')}
    u, v, e = g.field('u'), g.field('v'), g.field('eta')
    vol = e * area['eta'] * m['eta']
    want = np.array([vol.sum(), (0.5 * G * e * e * area['eta'] * m['eta']).sum(),
                     (0.5 * u * u * area['u'] * m['u']).sum() + (0.5 * v * v * area['v'] * m['v']).sum()])
    return want, np.array([np.abs(vol).sum(), want[1], want[2]])


@pytest.mark.parametrize('path,cells', [('plain_fp64', (48, 40)), ('fused_fp64', (48, 40)),
                                        ('fused_fp32c', (48, 40)), ('fused_fp32c', (2100, 10)),
                                        ('plain_fp64', (2100, 10)), ('fused_fp32c', (1024, 24)),
                                        ('fused_fp32c', (5, 300))])
def test_integrals_against_numpy_sums(path, cells):
    """swm_gpu_integrals against FP64 numpy sums of the fields the library
    returns.  Rows of 2101 points take two chunks of the reduction; 6-point
    rows leave most of a warp idle."""
    case = synthetic.double_gyre(cells, biharmonic=True, nsteps=40)
    g = GpuModel(path)
    Driver(case, g).init(with_diag=False)
    g.run(0, 30)
    got = g.integrals()
    want, scale = _numpy_integrals(case, g)
    assert np.all(want[1:] > 0) and scale[0] > 0
    tol = 1e-13 if path != 'fused_fp32c' else 1e-12
    assert np.all(np.abs(got - want) <= tol * scale), (got, want, (got - want) / scale)


@pytest.mark.parametrize('cells', [(48, 40), (300, 17), (5, 300), (2100, 10)])
def test_step_kernel_integrals_against_numpy_sums(cells):
    """The integrals the FP32 step kernel forms of the state it writes
    (swm_gpu_run_monitor) against FP64 numpy sums of that state."""
    import torch
    case = synthetic.double_gyre(cells, biharmonic=True, nsteps=40)
    g = GpuModel('fused_fp32c')
    Driver(case, g).init(with_diag=False)
    g.run(0, 10)
    out = torch.empty((3, 3), dtype=torch.float64).pin_memory().numpy()
    g.run_monitor(10, 3, 0, None, out)
    want, scale = _numpy_integrals(case, g)
    assert np.all(np.abs(out[-1] - want) <= 1e-12 * scale), (out[-1], want, (out[-1] - want) / scale)


@pytest.mark.parametrize('variant', ['laplace', 'laplace_qbf', 'linear_rg', 'no_mode', 'no_mixing', 'tracer'])
def test_run_monitor_variants(variant):
    """swm_gpu_run_monitor on the FP32 pair path across the step kernel's
    variants (Laplacian, Laplacian with quadratic drag and barotropic
    division, linear reduced gravity, no linearisation, no mixing) and on
    prescribed flow with tracers (the general route): the same state, bit
    for bit, as the same steps made one call at a time, and integrals equal
    to FP64 numpy sums of that state within 1e-12 of each sum's scale."""
    import torch
    from test_gpu_fused import _case
    if variant == 'no_mixing':
        case = synthetic.double_gyre((40, 32), biharmonic=False, nsteps=60)
        case['config'].update(lateral_mixing=0)
    elif variant == 'tracer':
        case = synthetic.tracer_flow(48, dx=5e3, nsteps=60)
    else:
        case = _case(variant, 60)
    a, b = GpuModel('fused_fp32c'), GpuModel('fused_fp32c')
    for g in (a, b):
        Driver(case, g).init(with_diag=False)
    ny, n = case['config']['ny'], 12
    s0 = case['streams'][0] if case['streams'] else None
    use_rows = s0 is not None and 'rec1' in s0 and s0['rec1'] is not None and not s0.get('is_const', False)
    rows = None
    if use_rows:
        prof = np.asarray(s0['rec1'][0])[:, 0]
        rows = torch.empty((n, ny), dtype=torch.float64).pin_memory().numpy()
        rows[:] = prof[None, :] * (1.0 + 0.05 * np.arange(n))[:, None]
    out = torch.empty((n, 3), dtype=torch.float64).pin_memory().numpy()
    a.run(0, 4)
    b.run(0, 4)
    a.run_monitor(4, n, 0, rows, out)
    for s in range(n):
        if use_rows:
            b.set_stream_rows(0, np.ascontiguousarray(rows[s]))
        b.step(5 + s)
        b.advance(5 + s)
    for f in ('u', 'v', 'eta'):
        assert np.array_equal(a.field(f), b.field(f)), f
    want, scale = _numpy_integrals(case, b)
    assert np.all(np.abs(out[-1] - want) <= 1e-12 * np.maximum(scale, 1e-300)), (out[-1], want)


@pytest.mark.parametrize('nsteps', [1, 2, 3])
def test_run_monitor_short_runs(nsteps):
    """Monitored runs of one to three steps: the first step of a run has no
    previous step for the side-job block to finish and the last is finished
    by its own kernel; state and integrals as the same steps one at a time,
    and a second run continues from the first."""
    import torch
    case = synthetic.double_gyre((40, 32), biharmonic=True, nsteps=60)
    a, b = GpuModel('fused_fp32c'), GpuModel('fused_fp32c')
    for g in (a, b):
        Driver(case, g).init(with_diag=False)
    ny = case['config']['ny']
    prof = case['streams'][0]['rec1'][0][:, 0]
    a.run(0, 5)
    b.run(0, 5)
    itt = 5
    for rep in range(2):
        rows = torch.empty((nsteps, ny), dtype=torch.float64).pin_memory().numpy()
        rows[:] = prof[None, :] * (1.0 + 0.2 * (rep + 1) + 0.1 * np.arange(nsteps))[:, None]
        out = torch.empty((nsteps, 3), dtype=torch.float64).pin_memory().numpy()
        out[:] = np.nan
        a.run_monitor(itt, nsteps, 0, rows, out)
        for s in range(nsteps):
            b.set_stream_rows(0, np.ascontiguousarray(rows[s]))
            b.step(itt + 1 + s)
            b.advance(itt + 1 + s)
            _, scale = _numpy_integrals(case, b)
            ref = b.integrals()
            assert np.all(np.abs(out[s] - ref) <= 1e-12 * scale), (rep, s, out[s], ref)
        itt += nsteps
        for f in ('u', 'v', 'eta'):
            assert np.array_equal(a.field(f), b.field(f)), (rep, f)
    # plain steps after the monitored runs read the last rows set
    a.run(itt, 3)
    b.run(itt, 3)
    for f in ('u', 'v', 'eta'):
        assert np.array_equal(a.field(f), b.field(f)), f
