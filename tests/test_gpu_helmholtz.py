"""GPU Helmholtz SOR (swm_helm_*) against the FP64 oracle: FP64 sweeps bit
for bit (same colour order, same arithmetic without FMA, same check
cadence), the operator bit for bit, the mixed-precision solver to the same
1e-10 relative residual, and the autotuner's choices."""
import numpy as np
import pytest

from oracle import helmholtz_apply, helmholtz_coeffs, helmholtz_sor
from swm_gb300 import SwmGpuError
from swm_gb300.host import synthetic
from swm_gb300.model import GpuHelmholtz

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def case():
    return synthetic.helmholtz_case(96, dx=20e3)


def _oracle(case):
    cx, cy, cc = helmholtz_coeffs(1.0 / case['H'], case['lam'], case['dx'], case['dy'])
    return cx, cy, cc


def test_apply_bit_exact(case):
    g = GpuHelmholtz(case['H'], case['ocean'], case['dx'], case['dy'], case['lam'])
    psi = np.random.default_rng(1).standard_normal(case['H'].shape)
    cx, cy, cc = _oracle(case)
    assert np.array_equal(g.apply(psi), helmholtz_apply(cx, cy, cc, case['ocean'], psi))


def test_fp64_solve_bit_exact(case):
    g = GpuHelmholtz(case['H'], case['ocean'], case['dx'], case['dy'], case['lam'])
    cx, cy, cc = _oracle(case)
    po, so, ro = helmholtz_sor(cx, cy, cc, case['ocean'], case['rhs'], np.zeros_like(case['H']), 1.9, 1e-10, 5000)
    pg, sg, _, rg, rc = g.solve(case['rhs'], omega=1.9, rtol=1e-10, max_sweeps=5000)
    assert rc == 0 and ro < 1e-10 and rg < 1e-10
    assert sg == so
    assert np.array_equal(pg, po)


def test_mixed_solve_reaches_fp64_accuracy(case):
    g = GpuHelmholtz(case['H'], case['ocean'], case['dx'], case['dy'], case['lam'])
    cx, cy, cc = _oracle(case)
    po, _, _ = helmholtz_sor(cx, cy, cc, case['ocean'], case['rhs'], np.zeros_like(case['H']), 1.9, 1e-13, 20000)
    pm, sm, outer, rm, rc = g.solve(case['rhs'], omega=1.9, rtol=1e-10, mixed=True)
    assert rc == 0 and rm < 1e-10 and outer >= 2
    r = case['rhs'] - helmholtz_apply(cx, cy, cc, case['ocean'], pm)
    m = case['ocean'] == 1
    assert np.linalg.norm(r[m]) < 1e-10 * np.linalg.norm(case['rhs'][m])
    assert np.abs(pm - po).max() <= 1e-7 * np.abs(po).max()


def test_not_converged_is_reported(case):
    g = GpuHelmholtz(case['H'], case['ocean'], case['dx'], case['dy'], case['lam'])
    _, sw, _, rel, rc = g.solve(case['rhs'], omega=1.9, rtol=1e-14, max_sweeps=32, raise_on_fail=False)
    assert rc == 4 and sw == 32 and rel > 1e-14
    with pytest.raises(SwmGpuError):
        g.solve(case['rhs'], omega=1.9, rtol=1e-14, max_sweeps=32)


def test_autotune_choices(case):
    g = GpuHelmholtz(case['H'], case['ocean'], case['dx'], case['dy'], case['lam'])
    om, blk = g.autotune(case['rhs'], 1.8, 1.99, 12, 64)
    assert 1.8 <= om <= 1.99
    assert blk in ((32, 8), (64, 4), (128, 2), (256, 1))
    # the chosen factor converges at least as fast as the range's ends
    counts = {}
    for w in (1.8, om, 1.99):
        counts[w] = g.solve(case['rhs'], omega=w, rtol=1e-10, max_sweeps=20000)[1]
    assert counts[om] <= max(counts[1.8], counts[1.99])


def test_temporal_blocking_does_not_change_results(case, monkeypatch):
    """K sweeps per launch on shared-memory tiles with a 2K halo give the
    same iterates as K global sweeps: the mixed solve is identical with global
    sweeps only (K = 0) and for K = 1, 2, 3, 4 (3 leaves 2 of every 32
    sweeps to the global kernel)."""
    res = []
    for k in ('0', '1', '2', '3', '4'):
        monkeypatch.setenv('SWM_GB300_HELM_K', k)
        g = GpuHelmholtz(case['H'], case['ocean'], case['dx'], case['dy'], case['lam'])
        g.autotune(case['rhs'], 1.9, 1.9, 1, 16)
        res.append(g.solve(case['rhs'], omega=1.9, rtol=1e-10, mixed=True))
        g.close()
    for r in res[1:]:
        assert r[1] == res[0][1] and r[2] == res[0][2]
        assert np.array_equal(r[0], res[0][0])


@pytest.fixture(scope='module')
def edge_case(case):
    """A 13 x 21 slice of the basin whose edge cells are ocean (the other
    cases have a land frame), so the zero face coefficients at the grid's
    edge are exercised; smaller than one tiled region in both directions."""
    sl = (slice(30, 43), slice(40, 61))
    ocean = np.ones((13, 21), dtype=np.int8)
    ocean[5:7, 8:11] = 0
    rhs = 1e-10 * np.random.default_rng(4).standard_normal((13, 21)) * ocean
    return dict(H=case['H'][sl].copy(), ocean=ocean, rhs=rhs, dx=case['dx'], dy=case['dy'], lam=case['lam'])


def test_edge_ocean_fp64_solve_bit_exact(edge_case):
    c = edge_case
    g = GpuHelmholtz(c['H'], c['ocean'], c['dx'], c['dy'], c['lam'])
    cx, cy, cc = _oracle(c)
    po, so, ro = helmholtz_sor(cx, cy, cc, c['ocean'], c['rhs'], np.zeros_like(c['H']), 1.5, 1e-10, 5000)
    pg, sg, _, rg, rc = g.solve(c['rhs'], omega=1.5, rtol=1e-10, max_sweeps=5000)
    assert rc == 0 and sg == so and np.array_equal(pg, po)


def test_edge_ocean_tiles_equal_global_sweeps(edge_case, monkeypatch):
    """Mixed solves with global sweeps only and with K = 1 .. 4 sweeps per
    tiled launch agree bit for bit on the small edge-ocean grid."""
    c = edge_case
    res = []
    for k in ('0', '1', '2', '3', '4'):
        monkeypatch.setenv('SWM_GB300_HELM_K', k)
        g = GpuHelmholtz(c['H'], c['ocean'], c['dx'], c['dy'], c['lam'])
        g.autotune(c['rhs'], 1.5, 1.5, 1, 16)
        res.append(g.solve(c['rhs'], omega=1.5, rtol=1e-10, mixed=True))
        g.close()
    assert res[0][4] == 0
    for r in res[1:]:
        assert r[1] == res[0][1] and r[2] == res[0][2]
        assert np.array_equal(r[0], res[0][0])
