"""CPU oracle of the Helmholtz extension: the SOR iteration converges to
the solution of the assembled sparse system (scipy direct solve), and the
workload generator meets its stated ranges."""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle import helmholtz_apply, helmholtz_coeffs, helmholtz_sor
from swm_gb300.host import synthetic


def _matrix(cx, cy, cc, mask):
    ny, nx = mask.shape
    n = nx * ny
    idx = np.arange(n).reshape(ny, nx)
    rows, cols, vals = [], [], []
    for (di, dj, c) in ((-1, 0, cx), (1, 0, np.roll(cx, -1, axis=1)), (0, -1, cy), (0, 1, np.roll(cy, -1, axis=0))):
        for j in range(ny):
            for i in range(nx):
                ii, jj = i + di, j + dj
                if 0 <= ii < nx and 0 <= jj < ny and mask[j, i] and mask[jj, ii]:
                    rows.append(idx[j, i]); cols.append(idx[jj, ii]); vals.append(c[j, i])
    diag = np.where(mask.ravel() == 1, cc.ravel(), 1.0)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n)) + sp.diags(diag)
    return A


def test_sor_matches_direct_solve():
    case = synthetic.helmholtz_case(40, dx=50e3)
    hinv = 1.0 / case['H']
    cx, cy, cc = helmholtz_coeffs(hinv, case['lam'], case['dx'], case['dy'])
    mask = case['ocean']
    psi, sweeps, rel = helmholtz_sor(cx, cy, cc, mask, case['rhs'], np.zeros_like(hinv), 1.9, 1e-12, 20000)
    assert rel < 1e-12 and sweeps < 20000
    A = _matrix(cx, cy, cc, mask)
    x = spla.spsolve(A.tocsc(), np.where(mask == 1, case['rhs'], 0.0).ravel()).reshape(mask.shape)
    assert np.abs(psi - x).max() <= 1e-9 * np.abs(x).max()
    r = case['rhs'] - helmholtz_apply(cx, cy, cc, mask, psi)
    assert np.linalg.norm(r[mask == 1]) <= 1e-12 * np.linalg.norm(case['rhs'][mask == 1])


def test_symmetric_operator():
    case = synthetic.helmholtz_case(24, dx=50e3)
    cx, cy, cc = helmholtz_coeffs(1.0 / case['H'], case['lam'], case['dx'], case['dy'])
    A = _matrix(cx, cy, cc, case['ocean'])
    assert abs(A - A.T).max() == 0.0


def test_generator_ranges():
    case = synthetic.helmholtz_case(128, dx=20e3)
    assert case['H'].min() >= 50.0 and case['H'].max() <= 5000.0
    frac = 1.0 - case['ocean'].mean()
    assert 0.1 < frac < 0.3
    rhs = case['rhs'][case['ocean'] == 1]
    assert 0.3e-10 < rhs.std() < 3e-10
    assert (case['rhs'][case['ocean'] == 0] == 0).all()
