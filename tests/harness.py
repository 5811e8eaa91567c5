"""Shared helpers for the parity tests (test infrastructure)."""
import os
import numpy as np

from swm_gb300.host.caseio import load_case
from swm_gb300.host.driver import Driver

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
# the test_diaglist fixtures were written by an older build: damping records
# add up and the basic-state psi is zero on land (see oracle/swm_oracle.c)
COMPAT = {'test_diaglist': dict(damping_additive=1, mask_psi_bs=1)}


def golden_case(name):
    case, extra = load_case(os.path.join(GOLDEN, name + '.npz'))
    case['config'].update(COMPAT.get(name, {}))
    return case, extra


def run_case(case, backend, nsteps=None, with_diag=True):
    drv = Driver(case, backend)
    drv.init(with_diag=with_diag)
    drv.run(nsteps, with_diag=with_diag)
    return drv


def compare_outputs(drv, backend, extra, partial=False):
    """Per golden file: (max relative error over ocean points, number of
    bit-identical records, number of records compared).  partial=True
    compares only the records a shortened run produced."""
    res = {}
    for fn, (times, recs, grid) in drv.outputs().items():
        key = 'data__' + fn
        if key not in extra or recs is None:
            continue
        gold, gt = extra[key], extra['time__' + fn]
        m = backend.ocean(grid).astype(bool)
        n = min(len(gold), len(recs))
        assert partial or n == len(gold), (fn, n, len(gold))
        assert np.allclose(times[:n], gt[:n]), fn
        scale = max(np.abs(gold[k][m]).max() for k in range(n))
        err = max(np.abs(recs[k][m] - gold[k][m]).max() for k in range(n))
        bits = sum(np.array_equal(recs[k][m], gold[k][m]) for k in range(n))
        res[fn] = (err / scale if scale > 0 else err, bits, n)
    return res


def rel_l2(a, b, mask):
    d = np.linalg.norm((a - b)[mask])
    r = np.linalg.norm(b[mask])
    return d / r if r > 0 else d
