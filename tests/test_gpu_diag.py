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


def test_run_monitor_matches_step_by_step():
    """swm_gpu_run_monitor (per-step row uploads and integrals, no host wait
    per step) gives the state and per-step integrals of the same steps made
    one call at a time."""
    import torch
    case = synthetic.double_gyre((40, 32), biharmonic=True, nsteps=60)
    a, b = GpuModel('fused_fp32c'), GpuModel('fused_fp32c')
    for g in (a, b):
        Driver(case, g).init(with_diag=False)
    ny, n = case['config']['ny'], 20
    prof = case['streams'][0]['rec1'][0][:, 0]
    rows = torch.empty((n, ny), dtype=torch.float64).pin_memory().numpy()
    rows[:] = prof[None, :] * (1.0 + 0.1 * np.arange(n))[:, None]
    out = torch.empty((n, 3), dtype=torch.float64).pin_memory().numpy()
    a.run(0, 5)
    b.run(0, 5)
    a.run_monitor(5, n, 0, rows, out)
    for s in range(n):
        b.set_stream_rows(0, np.ascontiguousarray(rows[s]))
        b.step(6 + s)
        b.advance(6 + s)
        assert np.array_equal(out[s], b.integrals()), s
    for f in ('u', 'v', 'eta'):
        assert np.array_equal(a.field(f), b.field(f))
