"""GPU plain-FP64 path against the FP64 CPU oracle.

The plain path runs the reference's loop nests with the reference's
evaluation order and no FMA contraction, so the comparison is bit-for-bit
(tolerance 0) on every field the time step touches.
"""
import numpy as np
import pytest

from harness import golden_case, run_case, compare_outputs
from oracle import OracleBackend
from swm_gb300.host import synthetic
from swm_gb300.model import GpuModel

pytestmark = pytest.mark.gpu

STATE = ['u', 'v', 'eta']
DIAG = ['D', 'Dh', 'Du', 'Dv', 'edens', 'pot', 'zeta', 'mu', 'mv', 'F_x', 'F_y', 'F_eta']


def _same(a, b):
    return np.array_equal(a, b, equal_nan=True)


def _pair(case, nsteps, path='plain_fp64', nan_guard=False):
    o, g = OracleBackend(tracer_nan_guard=nan_guard), GpuModel(path, tracer_nan_guard=nan_guard)
    run_case(case, o, nsteps=nsteps, with_diag=False)
    run_case(case, g, nsteps=nsteps, with_diag=False)
    return o, g


@pytest.mark.parametrize('name,nsteps', [('test_fixed_length_output', None), ('test_oscfrc', 700),
                                         ('test_diaglist', 700)])
def test_selfcheck_cases_bit_exact(name, nsteps):
    case, _ = golden_case(name)
    o, g = _pair(case, nsteps)
    for f in STATE + DIAG + ['H', 'H_u', 'H_v', 'H_eta', 'impl_u', 'impl_v', 'impl_eta']:
        assert _same(o.field(f), g.field(f)), f


def test_fixed_length_output_goldens_on_gpu():
    case, extra = golden_case('test_fixed_length_output')
    g = GpuModel('plain_fp64')
    drv = run_case(case, g)
    res = compare_outputs(drv, g, extra)
    for fn, (rel, bits, n) in res.items():
        assert rel <= 5e-16, (fn, rel)


@pytest.mark.parametrize('variant', ['biharmonic', 'laplace_qbf', 'linear_rg'])
def test_synthetic_bit_exact(variant):
    if variant == 'linear_rg':
        case = synthetic.linear_rg(40, 24, nsteps=200)
    else:
        case = synthetic.double_gyre((48, 40), biharmonic=(variant == 'biharmonic'), nsteps=200)
        if variant == 'laplace_qbf':
            case['config'].update(quadratic_friction=1, barotropic=1)
            case['damping'] += [dict(term=3, type=0, value=2e-3, sl_length=1.0, sl_cutoff=15.0, loc=0, file_data=None),
                                dict(term=4, type=1, value=3e-3, sl_length=0.02, sl_cutoff=15.0, loc=15,
                                     file_data=None)]
    o, g = _pair(case, 200)
    for f in STATE + DIAG + ['latmix_u', 'latmix_v']:
        assert _same(o.field(f), g.field(f)), f
    assert np.abs(g.field('u')).max() > 0


@pytest.mark.parametrize('nan_guard', [False, True])
def test_tracer_bit_exact(nan_guard):
    case = synthetic.double_gyre((48, 40), biharmonic=False, nsteps=120)
    rng = np.random.default_rng(5)
    ny, nx = case['config']['ny'], case['config']['nx']
    for kap in (50.0, 5e3):
        case['tracers'].append(dict(varid='C', kappa_h=kap, cons=1e-7, gamma_c=1.0 / (30 * 86400.0),
                                    field_C=rng.uniform(0, 1, (ny, nx)), field_C0=rng.uniform(0, 1, (ny, nx)),
                                    field_gamma_C=None, field_cons=None))
    o, g = _pair(case, 120, nan_guard=nan_guard)
    for t in range(2):
        for f in ('CH1', 'C', 'uhc', 'vhc', 'diff'):
            of = o.tracer_field(t, 'CH0' if f == 'CH1' else f)
            gf = g.tracer_field(t, 'CH' if f == 'CH1' else f)
            assert _same(of, gf), (t, f)
    if not nan_guard:
        # the reference's 0/0 tracer coefficients on land-land pairs spread
        # NaN into the basin after two steps
        assert np.isnan(g.tracer_field(0, 'CH')).any()
    else:
        assert np.isfinite(g.tracer_field(0, 'CH')).all()


@pytest.mark.parametrize('shape', [(40, 32), (41, 33)])
def test_sor_matches_oracle(shape):
    """Odd Nx pads one colour's rows in the colour-split layout."""
    case = synthetic.double_gyre(shape, biharmonic=False, nsteps=10)
    o, g = _pair(case, 10)
    o.sor_init()
    g.sor_init()
    rng = np.random.default_rng(3)
    # a compatible right-hand side (the divergence of a random flow), as the
    # reference's caller computeVelocityPotential passes (calc_lib.f90:519-521)
    u = rng.standard_normal((case['config']['ny'], case['config']['nx'])) * o.ocean('u')
    v = rng.standard_normal(u.shape) * o.ocean('v')
    B = o.divergence(u, v)
    chi0 = np.zeros_like(B)
    xo, io, ao = o.sor_solve(B, chi0, 1e-4, True)
    xg, ig, ag = g.sor_solve(B, chi0, 1e-4, True)
    assert io > 0 and abs(ig - io) <= 1, (io, ig)
    if ig == io:
        # same sweeps in the same colour order: identical iterates
        assert np.array_equal(xo, xg)
    assert np.abs(xo - xg).max() <= 1e-6 * np.abs(xo).max()
    # a non-converging call (max_count = 10*max(Nx,Ny)) reports it
    xg2, ig2, _ = g.sor_solve(B, chi0, 1e-40, False)
    assert ig2 < 0


def test_sor_division_is_correctly_rounded():
    """The SOR half-sweep and the plain path divide by fixed divisors through
    their reciprocals and two Markstein corrections (div_fast); on 2^26 pairs
    per seed (divisors over the exponent range it serves, all-ones and
    power-of-two significands among them; one numerator in eight zero,
    subnormal, tiny, huge, infinite or NaN) the quotient equals the division
    operator's in every bit."""
    from swm_gb300 import _lib
    import ctypes
    lib = _lib.lib()
    for seed in (1, 2):
        bad = ctypes.c_int64(-1)
        assert lib.swm_gpu_check_division(1 << 26, seed, ctypes.byref(bad)) == 0
        assert bad.value == 0


def test_nondivergent_flow_matches_oracle():
    """computeNonDivergentFlowField on the GPU (divergence, SOR, gradient on
    the device) against the oracle pipeline from the same state, for a first
    call (first_guess) and a second one starting from the kept chi."""
    case = synthetic.double_gyre((40, 32), biharmonic=False, nsteps=60)
    o, g = _pair(case, 60)
    o.sor_init()
    g.sor_init()
    chi = np.zeros((case['config']['ny'], case['config']['nx']))
    for first in (True, False):
        uo, vo, chi, io = o.nondivergent(o.field('u'), o.field('v'), chi, first)
        ug, vg, cg, ig, rc = g.nondivergent(first)
        if io < 0:
            # max_count (10 max(Nx, Ny) after the first call) reached
            # unconverged, as the reference allows with a warning
            assert rc == 4 and ig == -io, (io, ig)
            io = -io
        else:
            assert rc == 0 and abs(ig - io) <= 1, (io, ig)
        if ig == io:
            assert np.array_equal(cg, chi)
            assert np.array_equal(ug, uo) and np.array_equal(vg, vo)
        assert np.abs(ug - uo).max() <= 1e-6 * np.abs(uo).max()
        chi = cg
        o.run_steady(5)
        g.run(60 + (0 if first else 5), 5)
    # a converged correction (the first-call iteration budget) removes the
    # divergence of cells away from the coast (next to it the reference's
    # gradient, masked with the eta masks and the land boundary factor, puts
    # velocity on land faces, which the divergence then reads)
    oe, ou, ov = g.ocean('eta'), g.ocean('u'), g.ocean('v')
    inner = (oe == 1) & (ou == 1) & (np.roll(ou, -1, 1) == 1) & (ov == 1) & (np.roll(ov, -1, 0) == 1)
    inner &= (np.roll(oe, 1, 1) == 1) & (np.roll(oe, -1, 1) == 1) & (np.roll(oe, 1, 0) == 1) & (np.roll(oe, -1, 0) == 1)
    d0 = np.abs(o.divergence(g.field('u'), g.field('v'))[inner]).sum()
    ug, vg, _, _, rc = g.nondivergent(True)
    assert rc == 0
    assert np.abs(o.divergence(ug, vg)[inner]).sum() < 0.5 * d0


def test_damping_factors_set_during_a_run():
    """impl_u set between steps: the plain path forms the reciprocals of its
    damping factors again (and drops its step graph), so the run stays bit
    for bit with the oracle given the same field; the fused paths, which
    keep their own copies, refuse static fields once they have stepped."""
    from swm_gb300 import SwmGpuError
    case = synthetic.double_gyre((40, 32), biharmonic=False, nsteps=60)
    o, g = _pair(case, 20)
    impl = o.field('impl_u') * 1.5
    o.set_field('impl_u', impl)
    g.set_field('impl_u', impl)
    o.run_steady(15)
    g.run(20, 15)  # long enough for a graph replay
    for f in STATE:
        assert np.array_equal(o.field(f), g.field(f)), f
    f32 = GpuModel('fused_fp32c')
    run_case(case, f32, nsteps=3, with_diag=False)
    with pytest.raises(SwmGpuError, match='before the first step'):
        f32.set_field('impl_u', impl)
    f32.close()
    g.close()
