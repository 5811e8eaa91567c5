"""Tracer paths on the GPU against the FP64 oracle: the plain FP64 kernels
bit for bit (reference centred flux, upwind-biased extension, frozen flow),
and the FP32 compensated tracer kernel of the fused_fp32c path to 1e-5
relative L2 on ocean cells (that path always uses the guarded 0/0
coefficients, so the oracle runs with tracer_nan_guard)."""
import numpy as np
import pytest

from harness import rel_l2, run_case
from oracle import OracleBackend
from swm_gb300.host import synthetic
from swm_gb300.host.driver import Driver
from swm_gb300.model import GpuModel

pytestmark = pytest.mark.gpu


def _gyre_with_tracers(flux, nsteps=120):
    case = synthetic.double_gyre((48, 40), biharmonic=False, nsteps=nsteps)
    case['config'].update(tracer_flux=flux)
    rng = np.random.default_rng(5)
    ny, nx = case['config']['ny'], case['config']['nx']
    for kap in (50.0, 5e3):
        case['tracers'].append(dict(varid='C', kappa_h=kap, cons=1e-7, gamma_c=1.0 / (30 * 86400.0),
                                    field_C=rng.uniform(0, 1, (ny, nx)), field_C0=rng.uniform(0, 1, (ny, nx)),
                                    field_gamma_C=None, field_cons=None))
    return case


def _pair(case, nsteps, path, guard=True):
    o, g = OracleBackend(tracer_nan_guard=guard), GpuModel(path, tracer_nan_guard=guard)
    run_case(case, o, nsteps=nsteps, with_diag=False)
    run_case(case, g, nsteps=nsteps, with_diag=False)
    return o, g


@pytest.mark.parametrize('guard', [False, True])
def test_plain_upwind_biased_bit_exact(guard):
    o, g = _pair(_gyre_with_tracers(1), 120, 'plain_fp64', guard)
    for t in range(2):
        for f in ('CH', 'C', 'diff'):
            of = o.tracer_field(t, 'CH0' if f == 'CH' else f)
            assert np.array_equal(of, g.tracer_field(t, f), equal_nan=True), (t, f)


@pytest.mark.parametrize('flux', [0, 1])
def test_plain_frozen_flow_bit_exact(flux):
    case = synthetic.tracer_flow(48, nsteps=80, flux=flux)
    o, g = _pair(case, 80, 'plain_fp64')
    for t in range(2):
        assert np.array_equal(o.tracer_field(t, 'CH0'), g.tracer_field(t, 'CH')), t
    np.testing.assert_array_equal(g.field('u'), o.field('u'))


@pytest.mark.parametrize('flux', [0, 1])
@pytest.mark.parametrize('frozen', [False, True])
def test_fp32_tracers_against_oracle(flux, frozen):
    nsteps = 200
    case = synthetic.tracer_flow(64, nsteps=nsteps, flux=flux) if frozen else _gyre_with_tracers(flux, nsteps)
    o, g = _pair(case, nsteps, 'fused_fp32c')
    m = o.ocean('eta').astype(bool)
    for t in range(2):
        for f in ('CH', 'C'):
            a = g.tracer_field(t, f)
            b = o.tracer_field(t, 'CH0' if f == 'CH' else f)
            assert np.isfinite(a[m]).all()
            assert rel_l2(a, b, m) <= 1e-5, (t, f, rel_l2(a, b, m))


def test_fp32_tracers_graph_replay_and_launches():
    case = synthetic.tracer_flow(40, nsteps=100)
    a, b = GpuModel('fused_fp32c', tracer_nan_guard=True), GpuModel('fused_fp32c', tracer_nan_guard=True)
    Driver(case, a).init(with_diag=False)
    Driver(case, b).init(with_diag=False)
    a.run(0, 5)
    l0 = a.launch_count()
    a.run(5, 37)
    a.synchronize()
    assert a.launch_count() - l0 == 37  # frozen flow: one tracer kernel per step
    for s in range(1, 43):
        b.step(s)
        b.advance(s)
    for t in range(2):
        assert np.array_equal(a.tracer_field(t, 'CH'), b.tracer_field(t, 'CH')), t


@pytest.mark.parametrize('flux,ntr', [(0, 2), (1, 2), (1, 3)])
def test_fp32_tracer_rows_per_warp_do_not_change_results(flux, ntr, monkeypatch):
    """Each tracer point is computed from the same inputs whatever the rows
    per warp strip: the results agree bit for bit (three tracers: the
    instance that reloads the updated row's CH pair)."""
    case = synthetic.tracer_flow(72, nsteps=30, flux=flux)
    while len(case['tracers']) < ntr:
        case['tracers'].append(dict(case['tracers'][0], kappa_h=500.0))
    out = []
    for rows in ('5', '16', '23'):
        monkeypatch.setenv('SWM_GB300_TRC_ROWS', rows)
        g = GpuModel('fused_fp32c', tracer_nan_guard=True)
        Driver(case, g).init(with_diag=False)
        g.run(0, 25)
        out.append([g.tracer_field(t, 'CH') for t in range(ntr)])
        g.close()
    for other in out[1:]:
        for a, b in zip(out[0], other):
            assert np.array_equal(a, b)


@pytest.mark.parametrize('flux', [0, 1])
def test_fp32_tracer_prefetch_level_does_not_change_results(flux, monkeypatch):
    """The L2 prefetches of the tracer kernel write no register: both levels
    give the same fields bit for bit."""
    case = synthetic.tracer_flow(72, nsteps=30, flux=flux)
    out = []
    for pf in ('0', '1'):
        monkeypatch.setenv('SWM_GB300_TRC_PREFETCH', pf)
        monkeypatch.setenv('SWM_GB300_TRC_ROWS', '7')
        g = GpuModel('fused_fp32c', tracer_nan_guard=True)
        Driver(case, g).init(with_diag=False)
        g.run(0, 25)
        out.append([g.tracer_field(t, 'CH') for t in range(2)])
        g.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


def _gyre_with_n_tracers(n, flux, nsteps):
    """The gyre with n tracers of different diffusivities; the odd ones relax
    with a per-cell rate field and the last decays with a per-cell rate."""
    case = synthetic.double_gyre((48, 40), biharmonic=False, nsteps=nsteps)
    case['config'].update(tracer_flux=flux)
    rng = np.random.default_rng(11)
    ny, nx = case['config']['ny'], case['config']['nx']
    for q in range(n):
        gam = rng.uniform(0.5, 2.0, (ny, nx)) / (30 * 86400.0) if q % 2 else None
        cons = rng.uniform(0.5, 2.0, (ny, nx)) * 1e-7 if q == n - 1 and n > 1 else None
        case['tracers'].append(dict(varid='C', kappa_h=(50.0, 5e3, 500.0, 20.0, 1e3)[q % 5], cons=1e-7,
                                    gamma_c=1.0 / (30 * 86400.0), field_C=rng.uniform(0, 1, (ny, nx)),
                                    field_C0=rng.uniform(0, 1, (ny, nx)), field_gamma_C=gam, field_cons=cons))
    return case


@pytest.mark.parametrize('n', [1, 3, 5])
def test_fp32_tracer_counts_against_oracle(n):
    """The tracer kernel's instances for 1 to 4 tracers per launch, and more
    tracers than one launch takes (5 = 4 + 1), with per-cell relaxation and
    decay fields, against the oracle."""
    nsteps = 150
    case = _gyre_with_n_tracers(n, 1, nsteps)
    o, g = _pair(case, nsteps, 'fused_fp32c')
    m = o.ocean('eta').astype(bool)
    for t in range(n):
        a, b = g.tracer_field(t, 'CH'), o.tracer_field(t, 'CH0')
        assert np.isfinite(a[m]).all()
        assert rel_l2(a, b, m) <= 1e-5, (t, rel_l2(a, b, m))


def test_plain_tracer_fields_bit_exact():
    """Three tracers with per-cell relaxation and decay fields on the FP64
    tracer kernels: bit for bit with the oracle."""
    case = _gyre_with_n_tracers(3, 1, 80)
    o, g = _pair(case, 80, 'plain_fp64')
    for t in range(3):
        assert np.array_equal(o.tracer_field(t, 'CH0'), g.tracer_field(t, 'CH'), equal_nan=True), t
