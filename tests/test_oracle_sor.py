"""Known-answer tests of the oracle's restatement of the reference SOR
(init_ElSolv_SOR and main_ElSolv_SOR, src/ElSolv_SOR.f90:44-66,150-222),
whose GPU counterpart (sor.cu) matches it bit for bit when the iteration
counts agree (tests/test_gpu_parity.py).

The reference ships no SOR fixture, so the restatement is pinned here by a
manufactured solution: on a closed flat basin and on the reference's own
spherical test_nonlinear grid, B = A chi* is formed in numpy from the
coefficients for a smooth random chi* on ocean cells, and SOR from chi = 0
must recover chi* up to the constant the masked operator cannot see (its
land faces carry no flux, so constants are in its null space): the
residual and every coupled face difference must match.  The coefficients
themselves are checked for the masked spherical Laplacian's structure:
zero row sums, and symmetry under the cos(lat)-weighted inner product."""
import numpy as np
import pytest

from harness import golden_case, run_case
from oracle import OracleBackend
from swm_gb300.host import synthetic


def _apply(c, chi):
    """The reference operator: c0 chi(i+1) + c1 chi(i-1) + c2 chi(j+1) +
    c3 chi(j-1) + c4 chi, periodic indices as ip1/im1/jp1/jm1."""
    return (c[0] * np.roll(chi, -1, axis=1) + c[1] * np.roll(chi, 1, axis=1) + c[2] * np.roll(chi, -1, axis=0) +
            c[3] * np.roll(chi, 1, axis=0) + c[4] * chi)


def _smooth(rng, shape, scale):
    ny, nx = shape
    k = np.fft.fftfreq(nx)[None, :] ** 2 + np.fft.fftfreq(ny)[:, None] ** 2
    f = np.fft.ifft2(np.fft.fft2(rng.standard_normal(shape)) * np.exp(-k * scale ** 2)).real
    return f / np.abs(f).max()


def _oracle(case):
    o = OracleBackend()
    run_case(case, o, nsteps=1, with_diag=False)
    o.sor_init()
    return o


CASES = {
    'flat_closed_basin': lambda: synthetic.double_gyre((41, 33), biharmonic=False, nsteps=10),
    'sphere_test_nonlinear': lambda: golden_case('test_nonlinear')[0],
}


@pytest.mark.parametrize('name', sorted(CASES))
def test_sor_coefficients_are_the_masked_laplacian(name):
    """ElSolvSOR_c(:,:,1..5) of init_ElSolv_SOR (ElSolv_SOR.f90:54-62),
    formed here in numpy from the grid (A, dLambda, dTheta, cos(lat) of the
    eta and v rows, u and v masks), against the oracle's; then the operator's
    structure: zero row sums, and symmetry of the meridional coupling under
    the cos(lat_eta)-weighted inner product."""
    case = CASES[name]()
    o = _oracle(case)
    c = o.sor_coeff()
    A = case['config']['A']
    dL, dT = o.scalars()
    cE, cV = o.lat('cos_eta')[:, None], o.lat('cos_v')[:, None]
    oU, oV = o.ocean('u').astype(float), o.ocean('v').astype(float)
    oUp, oVp, cVp = np.roll(oU, -1, axis=1), np.roll(oV, -1, axis=0), np.roll(cV, -1, axis=0)
    ax = (A * cE * dL) ** 2
    ay = A ** 2 * cE * dT ** 2
    want = np.stack([oUp / ax, oU / ax, cVp * oVp / ay, cV * oV / ay,
                     (-oUp - oU) / ax + (-cVp * oVp - cV * oV) / ay])
    want = np.broadcast_to(want, c.shape)
    assert np.all(np.abs(c - want) <= 4e-16 * np.abs(want)), np.abs(c - want).max()
    ocean = o.ocean('eta') == 1
    scale = np.abs(c[4][ocean]).max()
    assert np.abs(c.sum(axis=0)[ocean]).max() <= 1e-14 * scale
    # a zonal face couples (i, j) and (i+1, j) with one coefficient both ways
    assert np.array_equal(c[0], np.roll(c[1], -1, axis=1))
    # a meridional face: cos_eta(j) c3(i, j) = cos_eta(j+1) c4(i, j+1)
    lhs, rhs = cE * c[2], np.roll(cE * c[3], -1, axis=0)
    assert np.all(np.abs(lhs - rhs) <= 1e-15 * np.abs(lhs).max())


@pytest.mark.parametrize('name', sorted(CASES))
def test_sor_recovers_a_manufactured_solution(name):
    o = _oracle(CASES[name]())
    c = o.sor_coeff()
    ocean = o.ocean('eta') == 1
    rng = np.random.default_rng(5)
    chi_star = np.where(ocean, _smooth(rng, ocean.shape, ocean.shape[1] / 6.0), 0.0)
    B = np.where(ocean, _apply(c, chi_star), 0.0)
    x, iters, anorm = o.sor_solve(B, np.zeros_like(B), 1e-13, True)
    assert iters > 0, (iters, anorm)
    r = np.where(ocean, _apply(c, x) - B, 0.0)
    assert np.abs(r).max() <= 1e-9 * np.abs(B).max()
    # every face the operator couples: differences agree, constants cancel
    for axis, cf in ((1, c[0]), (0, c[2])):
        coupled = ocean & (cf != 0)
        dx = (np.roll(x, -1, axis=axis) - x)[coupled]
        ds = (np.roll(chi_star, -1, axis=axis) - chi_star)[coupled]
        assert np.abs(dx - ds).max() <= 1e-7 * np.abs(ds).max()
