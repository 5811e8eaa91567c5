"""Every GPU path on the reference's own spherical configurations.

selfcheck/test_nonlinear and selfcheck/test_nl_tracer are the reference's
configurations of the nonlinear path and of the tracer: FULLY_NONLINEAR +
LATERAL_MIXING + BAROTROPIC, 201 x 101 points from 25S to 25N on a sphere of
radius 6371 km (cos(lat) 0.91-1, tan(lat)/A up to 7e-8 /m), dt = 3500 s,
wind stress scaled by TAU_SCALE = 5e-2, north/south sponges (test_nonlinear)
and two tracers with kappa 5e3 and 1e2 (test_nl_tracer).  There the metric
terms of the stress tensor (pll_coeff/plt_coeff,
swm_lateralmixing_module.f90:115-146), the cos-weighted flux divergences
(swm_nonlinear_timestep_module.f90:353-368) and the tracer coefficients
(tracer_module.f90:291-342) all differ from their flat-grid values, so a
slip in any of them shows here.

Tolerances: the plain FP64 path bit for bit; fused_fp64 1e-11 relative L2;
the FP32 pair paths (single basin, batched ensemble, tracer kernel) 1e-5
relative L2 on ocean points, after 400 steps (16 days of model time).
"""
import numpy as np
import pytest

from harness import golden_case, rel_l2, run_case
from oracle import OracleBackend
from swm_gb300.host.driver import Driver
from swm_gb300.model import GpuEnsemble, GpuModel

pytestmark = pytest.mark.gpu

NSTEPS = 400
STATE = ['u', 'v', 'eta']
DIAG = ['D', 'Dh', 'Du', 'Dv', 'edens', 'pot', 'zeta', 'mu', 'mv', 'F_x', 'F_y', 'F_eta', 'latmix_u', 'latmix_v']
TOL = {'fused_fp64': 1e-11, 'fused_fp32c': 1e-5}


def _case(name, biharmonic=False):
    case, _ = golden_case(name)
    if biharmonic:
        # the biharmonic extension on the same sphere (about 55 km spacing)
        case['config'].update(mixing_kind=1, bih=1e13)
    return case


def _oracle(case, guard=False, nsteps=NSTEPS):
    o = OracleBackend(tracer_nan_guard=guard)
    run_case(case, o, nsteps=nsteps, with_diag=False)
    return o


def _tracer_mass(backend, case, name, t):
    """FP64 sum of CH times the cell area over ocean eta points."""
    o = OracleBackend()
    Driver(case, o).init(with_diag=False)
    dl, dt = o.scalars()
    A = case['config']['A']
    area = (A * A * o.lat('cos_eta') * dl * dt)[:, None]
    m = o.ocean('eta') == 1
    return float((backend.tracer_field(t, name) * area)[m].sum())


@pytest.mark.parametrize('name,guard', [('test_nonlinear', False), ('test_nl_tracer', False),
                                        ('test_nl_tracer', True)])
def test_plain_bit_exact_on_sphere(name, guard):
    case = _case(name)
    o = _oracle(case, guard)
    g = GpuModel('plain_fp64', tracer_nan_guard=guard)
    run_case(case, g, nsteps=NSTEPS, with_diag=False)
    for f in STATE + DIAG:
        assert np.array_equal(o.field(f), g.field(f), equal_nan=True), f
    assert np.abs(g.field('u')).max() > 0.1
    for t in range(len(case['tracers'])):
        for f in ('CH', 'C', 'uhc', 'vhc', 'diff'):
            of = o.tracer_field(t, 'CH0' if f == 'CH' else f)
            assert np.array_equal(of, g.tracer_field(t, f), equal_nan=True), (t, f)
    if case['tracers'] and not guard:
        # the reference's 0/0 tracer coefficients (land-land pairs) fill the
        # basin with NaN; the guarded form keeps every point finite
        assert np.isnan(g.tracer_field(0, 'CH')).any()


def test_sor_and_nondivergent_flow_on_sphere():
    """The drop-in main_ElSolv_SOR and the non-divergent correction on the
    spherical test_nonlinear grid (cos(lat) 0.91-1 in the coefficients) from
    the state after NSTEPS steps: chi bit for bit with the oracle when the
    iteration counts agree (they agree or differ by one: the correction norm
    is a parallel sum on the GPU)."""
    case = _case('test_nonlinear')
    o = _oracle(case)
    g = GpuModel('plain_fp64')
    run_case(case, g, nsteps=NSTEPS, with_diag=False)
    o.sor_init()
    g.sor_init()
    B = o.divergence(o.field('u'), o.field('v'))
    assert np.abs(B).max() > 0
    xo, io, _ = o.sor_solve(B, np.zeros_like(B), 1e-4, True)
    xg, ig, _ = g.sor_solve(B, np.zeros_like(B), 1e-4, True)
    assert io > 0 and abs(ig - io) <= 1, (io, ig)
    if ig == io:
        assert np.array_equal(xo, xg)
    assert np.abs(xo - xg).max() <= 1e-6 * np.abs(xo).max()
    uo, vo, co, io2 = o.nondivergent(o.field('u'), o.field('v'), np.zeros_like(B), True)
    ug, vg, cg, ig2, rc = g.nondivergent(True)
    assert rc == 0 and io2 > 0 and abs(ig2 - io2) <= 1, (io2, ig2)
    if ig2 == io2:
        assert np.array_equal(cg, co) and np.array_equal(ug, uo) and np.array_equal(vg, vo)
    assert np.abs(ug - uo).max() <= 1e-6 * np.abs(uo).max()
    g.close()


@pytest.mark.parametrize('path', ['fused_fp64', 'fused_fp32c'])
@pytest.mark.parametrize('name,biharmonic', [('test_nonlinear', False), ('test_nonlinear', True),
                                             ('test_nl_tracer', False), ('test_fixed_length_output', False)])
def test_fused_paths_on_sphere(path, name, biharmonic):
    """test_fixed_length_output is the reference's linear state-of-rest case
    with oscillating forcing (added to the forcing fields every step on the
    fused paths) and a bathymetry file, 61 x 41 points on the sphere."""
    case = _case(name, biharmonic)
    guard = bool(case['tracers'])
    o = _oracle(case, guard)
    g = GpuModel(path, tracer_nan_guard=guard)
    run_case(case, g, nsteps=NSTEPS, with_diag=False)
    for f in STATE:
        m = o.ocean(f).astype(bool)
        a = g.field(f)
        assert np.isfinite(a).all(), f
        err = rel_l2(a, o.field(f), m)
        assert err <= TOL[path], (f, err)
    for f in ('D', 'zeta', 'mu', 'mv', 'pot'):
        a, b = g.field(f), o.field(f)
        m = np.isfinite(b)
        assert np.abs(a - b)[m].max() <= 100 * TOL[path] * np.abs(b[m]).max(), f
    for t in range(len(case['tracers'])):
        m = o.ocean('eta').astype(bool)
        for f in ('CH', 'C'):
            a, b = g.tracer_field(t, f), o.tracer_field(t, 'CH0' if f == 'CH' else f)
            assert np.isfinite(a[m]).all(), (t, f)
            assert rel_l2(a, b, m) <= TOL[path], (t, f, rel_l2(a, b, m))


def test_fp32_tracer_mass_on_sphere():
    """Tracer mass (sum of CH times cell area) in the closed spherical basin
    of test_nl_tracer, which has no sources (gamma_C = 0, cons = 0, F_eta =
    0): the FP64 oracle keeps it to rounding, the FP32 pair kernel to 1e-6
    relative after 400 steps."""
    case = _case('test_nl_tracer')
    g = GpuModel('fused_fp32c', tracer_nan_guard=True)
    Driver(case, g).init(with_diag=False)
    m0 = [_tracer_mass(g, case, 'CH', t) for t in range(2)]
    g.run(0, NSTEPS)
    m1 = [_tracer_mass(g, case, 'CH', t) for t in range(2)]
    o = _oracle(case, guard=True)
    mo = [_tracer_mass(o, case, 'CH0', t) for t in range(2)]
    for t in range(2):
        assert m0[t] > 0
        assert abs(mo[t] - m0[t]) <= 1e-12 * m0[t], (t, mo[t], m0[t])
        assert abs(m1[t] - m0[t]) <= 1e-6 * m0[t], (t, m1[t], m0[t])


@pytest.mark.parametrize('biharmonic', [False, True])
def test_ensemble_on_sphere(biharmonic):
    """The batched kernel with the spherical test_nonlinear basin as a member,
    beside a second copy of it (two members, so the member tables and the
    queue both carry more than one entry), against the oracle."""
    case = _case('test_nonlinear', biharmonic)
    o = _oracle(case)
    ms = []
    for _ in range(2):
        g = GpuModel('fused_fp32c')
        Driver(case, g).init(with_diag=False)
        ms.append(g)
    ens = GpuEnsemble(ms)
    ens.run(0, NSTEPS)
    ens.synchronize()
    for g in ms:
        for f in STATE:
            m = o.ocean(f).astype(bool)
            err = rel_l2(g.field(f), o.field(f), m)
            assert err <= 1e-5, (f, err)
    ens.close()
    for g in ms:
        g.close()


def test_monitored_integrals_on_sphere():
    """The integrals the monitored step forms inside the step kernel weight
    each point by its own row's cell area; on the sphere the rows differ by
    cos(lat).  Against FP64 numpy sums of the fields the library returns."""
    import torch
    from test_gpu_diag import _numpy_integrals
    case = _case('test_nonlinear')
    g = GpuModel('fused_fp32c')
    Driver(case, g).init(with_diag=False)
    g.run(0, 50)
    out = torch.empty((10, 3), dtype=torch.float64).pin_memory().numpy()
    g.run_monitor(50, 10, 0, None, out)
    want, scale = _numpy_integrals(case, g)
    assert np.all(want[1:] > 0)
    assert np.all(np.abs(out[-1] - want) <= 1e-12 * scale), (out[-1], want)
    got = g.integrals()
    assert np.all(np.abs(got - want) <= 1e-12 * scale), (got, want)
