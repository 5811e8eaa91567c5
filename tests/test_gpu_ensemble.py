"""Batched ensemble of uneven basins (swm_gpu_ensemble_*): the persistent
queue kernel against the same members stepped one at a time on the
single-basin FP32 path, and against the FP64 oracle.

The batched kernel reads each member's parameters from shared memory, the
single-basin kernel from its launch parameters; the two are compiled
separately and the compiler may fuse different multiply-adds, so they agree
to binary32 rounding (about 1e-7 relative after tens of steps), not bit for
bit.  The strip length does not change either kernel's results."""
import math

import numpy as np
import pytest

from harness import rel_l2
from oracle import OracleBackend
from swm_gb300 import SwmGpuError
from swm_gb300.host import synthetic
from swm_gb300.host.driver import Driver
from swm_gb300.model import GpuEnsemble, GpuModel

pytestmark = pytest.mark.gpu


def _cases(n, biharmonic=False, lo=20, hi=90, seed=11):
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n):
        cx = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        cy = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        dx = rng.uniform(5e3, 20e3)
        out.append(synthetic.double_gyre((cx, cy), biharmonic=biharmonic, dx=dx, amp=rng.uniform(0.05, 0.2),
                                         ah=500.0, rng=rng, nsteps=500, dt=15.0 * dx / 5e3))
    return out


def _models(cases, path='fused_fp32c'):
    ms = []
    for c in cases:
        g = GpuModel(path)
        Driver(c, g).init(with_diag=False)
        ms.append(g)
    return ms


@pytest.mark.parametrize('biharmonic', [False, True])
def test_ensemble_matches_members_stepped_alone(biharmonic):
    cases = _cases(12, biharmonic=biharmonic)
    batched, alone = _models(cases), _models(cases)
    ens = GpuEnsemble(batched)
    assert ens.rows() in (16, 24, 32, 48)
    itt = 0
    for n in (40, 17, 12):  # start-up steps, graph blocks and single steps
        ens.run(itt, n)
        for g in alone:
            g.run(itt, n)
        itt += n
        for a, b in zip(batched, alone):
            for f in ('u', 'v', 'eta'):
                x, y = a.field(f), b.field(f)
                assert np.isfinite(x).all()
                assert np.abs(x - y).max() <= 1e-6 * max(np.abs(y).max(), 1e-30), (n, f)
    ints = ens.integrals()
    for k, b in enumerate(alone):
        # potential and kinetic energy; the volume anomaly is a sum that
        # cancels to ~0 and has no relative precision
        np.testing.assert_allclose(ints[k][1:], b.integrals()[1:], rtol=1e-6)
    assert (ints[:, 1] > 0).all()
    ens.close()


def test_ensemble_tiles_do_not_change_results(monkeypatch):
    """The ensemble queue's tiles (rows per warp, masked-row cost, and so the
    order of the costliest-first queue) change which warp computes a point,
    not its value: four tilings agree bit for bit."""
    cases = _cases(6, biharmonic=True, seed=5)
    results = []
    for rows, slow in ((16, 1.0), (48, 1.0), (24, 2.0), (17.5, 1.4)):
        monkeypatch.setenv('SWM_GB300_MARCH_S', str(rows))
        monkeypatch.setenv('SWM_GB300_MARCH_SLOW', str(slow))
        ms = _models(cases)
        ens = GpuEnsemble(ms)
        ens.run(0, 23)
        results.append([[g.field(f) for f in ('u', 'v', 'eta')] for g in ms])
        ens.close()
        for g in ms:
            g.close()
    for other in results[1:]:
        for a, b in zip(results[0], other):
            for x, y in zip(a, b):
                assert np.array_equal(x, y)


def test_ensemble_against_fp64_oracle():
    cases = _cases(3, lo=30, hi=60, seed=5)
    ms = _models(cases)
    ens = GpuEnsemble(ms)
    ens.run(0, 200)
    for c, g in zip(cases, ms):
        o = OracleBackend()
        d = Driver(c, o)
        d.init(with_diag=False)
        d.run(200, with_diag=False)
        for f in ('u', 'v', 'eta'):
            m = o.ocean(f).astype(bool)
            assert rel_l2(g.field(f), o.field(f), m) <= 1e-5, f


def test_ensemble_one_launch_per_step():
    ms = _models(_cases(5))
    ens = GpuEnsemble(ms)
    ens.run(0, 5)
    l0 = ens.launch_count()
    ens.run(5, 24)
    ens.synchronize()
    assert ens.launch_count() - l0 == 24


def test_ensemble_rejects_other_paths():
    cases = _cases(2)
    ms = _models(cases[:1]) + _models(cases[1:], path='plain_fp64')
    with pytest.raises(SwmGpuError):
        GpuEnsemble(ms)


def test_ensemble_rejects_members_with_per_step_forcing():
    """A custom forcing stream with records that change in time makes the
    member's forcing fields change every step, which the batched step does
    not recompute: such a member is refused."""
    cases = _cases(2)
    ny, nx = cases[1]['config']['ny'], cases[1]['config']['nx']
    recs = np.stack([np.full((ny, nx), 1e-7), np.full((ny, nx), 2e-7)])
    cases[1]['streams'].append(dict(type=2, comp=0, omega=0.0, rec1=recs, dt1=900.0, chunksize=2, rec2=None,
                                    dt2=0.0))
    ms = _models(cases)
    with pytest.raises(SwmGpuError, match='time-dependent forcing'):
        GpuEnsemble(ms)


def test_ensemble_monitor_pageable_buffers():
    """swm_gpu_ensemble_run_monitor with ordinary (pageable) host arrays: the
    rows are staged through a device buffer and the integrals copied back
    after every step, where pinned arrays are read and written in place by
    the kernels.  Both give the same integrals and state bit for bit."""
    import torch
    cases = _cases(5, seed=31)
    ny = [c['config']['ny'] for c in cases]
    off = np.concatenate([[0], np.cumsum(ny)])
    nsteps = 14
    rows = np.empty((nsteps, off[-1]))
    for i, c in enumerate(cases):
        prof = c['streams'][0]['rec1'][0][:, 0]
        rows[:, off[i]:off[i + 1]] = prof[None, :] * (1.0 + 0.05 * np.sin(0.9 * np.arange(nsteps) + i))[:, None]
    results = []
    for pinned in (True, False):
        ms = _models(cases)
        ens = GpuEnsemble(ms)
        if pinned:
            r = torch.empty(rows.shape, dtype=torch.float64).pin_memory().numpy()
            r[:] = rows
            out = torch.empty((nsteps, len(cases), 3), dtype=torch.float64).pin_memory().numpy()
        else:
            r = rows.copy()
            out = np.empty((nsteps, len(cases), 3))
        ens.run_monitor(0, nsteps, r, out)
        results.append((out.copy(), [[g.field(f) for f in ('u', 'v', 'eta')] for g in ms]))
        ens.close()
        for g in ms:
            g.close()
    (oa, fa), (ob, fb) = results
    assert np.isfinite(oa).all() and np.all(oa[-1][:, 1:] > 0)
    assert np.array_equal(oa, ob)
    for x, y in zip(fa, fb):
        for a, b in zip(x, y):
            assert np.array_equal(a, b)


@pytest.mark.parametrize('biharmonic', [False, True])
def test_ensemble_monitor_matches_steps_and_integrals(biharmonic):
    """swm_gpu_ensemble_run_monitor (each step: every member's wind rows in,
    every member's integrals out, no host wait) against FP64 numpy sums of
    the fields it leaves (1e-11 of each sum's scale, after two calls that
    split the run), and against the same members given the same rows
    through swm_gpu_set_stream_rows and stepped one step at a time by
    swm_gpu_ensemble_run.  The monitored steps run a separately compiled
    instance of the step kernel, so the two runs agree to binary32 rounding
    (1e-6), not bit for bit."""
    import torch
    from test_gpu_diag import _numpy_integrals
    cases = _cases(6, biharmonic=biharmonic, seed=21)
    ma, mb = _models(cases), _models(cases)
    ea, eb = GpuEnsemble(ma), GpuEnsemble(mb)
    ny = [c['config']['ny'] for c in cases]
    off = np.concatenate([[0], np.cumsum(ny)])
    nsteps = 17
    rows = torch.empty((nsteps, off[-1]), dtype=torch.float64).pin_memory().numpy()
    for i, c in enumerate(cases):
        prof = c['streams'][0]['rec1'][0][:, 0]
        rows[:, off[i]:off[i + 1]] = prof[None, :] * (1.0 + 0.05 * np.cos(0.7 * np.arange(nsteps) + i))[:, None]
    out = torch.empty((nsteps, len(cases), 3), dtype=torch.float64).pin_memory().numpy()
    for s0, s1 in ((0, 9), (9, nsteps)):
        part = torch.empty((s1 - s0, len(cases), 3), dtype=torch.float64).pin_memory().numpy()
        ea.run_monitor(s0, s1 - s0, np.ascontiguousarray(rows[s0:s1]), part)
        out[s0:s1] = part
        for k, (c, a) in enumerate(zip(cases, ma)):
            want, scale = _numpy_integrals(c, a)
            assert np.all(want[1:] > 0)
            assert np.all(np.abs(out[s1 - 1][k] - want) <= 1e-11 * scale), (s1, k, out[s1 - 1][k], want)
    for s in range(nsteps):
        for i, g in enumerate(mb):
            g.set_stream_rows(0, np.ascontiguousarray(rows[s, off[i]:off[i + 1]]))
        eb.run(s, 1)
        ref = eb.integrals()
        assert np.isfinite(out[s]).all()
        np.testing.assert_allclose(out[s][:, 1:], ref[:, 1:], rtol=1e-6, atol=0, err_msg='step %d' % s)
    for a, b in zip(ma, mb):
        for f in ('u', 'v', 'eta'):
            x, y = a.field(f), b.field(f)
            assert np.abs(x - y).max() <= 1e-6 * np.abs(y).max(), f
    # rows=None: no wind update, the steps go on with the last rows
    out2 = torch.empty((3, len(cases), 3), dtype=torch.float64).pin_memory().numpy()
    ea.run_monitor(nsteps, 3, None, out2)
    eb.run(nsteps, 3)
    np.testing.assert_allclose(out2[-1][:, 1:], eb.integrals()[:, 1:], rtol=1e-6, atol=0)
    ea.close()
    eb.close()
