"""swm_gpu_integrals_noalloc, the allocation-free domain integrals, against
swm_gpu_integrals through the C ABI.

Both run the same reduction kernels with the same block count and cell areas,
so the tolerance is tight (1e-13 relative); two calls in a row check that the
fixed scratch is reused cleanly.  Kept in a file that is collected last, so
that it runs both alone in a fresh process and after every other GPU test.
"""
import ctypes

import numpy as np
import pytest

from swm_gb300 import _lib
from swm_gb300.host import synthetic
from swm_gb300.host.driver import Driver
from swm_gb300.model import GpuModel

pytestmark = pytest.mark.gpu

RTOL = 1e-13


def _noalloc(g):
    out = np.zeros(3)
    _lib.check(_lib.lib().swm_gpu_integrals_noalloc(g.ctx, out.ctypes.data_as(ctypes.c_void_p)))
    return out


@pytest.mark.parametrize('path', ['plain_fp64', 'fused_fp32c'])
def test_noalloc_integrals_match_allocating_entry(path):
    case = synthetic.double_gyre((48, 40), biharmonic=True, nsteps=60)
    g = GpuModel(path)
    Driver(case, g).init(with_diag=False)
    g.run(0, 40)
    ref = g.integrals()
    first, second = _noalloc(g), _noalloc(g)
    assert np.all(ref[1:] > 0), ref
    np.testing.assert_allclose(first, ref, rtol=RTOL, atol=0)
    np.testing.assert_allclose(second, ref, rtol=RTOL, atol=0)
    # the state moves on: the next pair of calls follows it
    g.run(40, 20)
    ref2 = g.integrals()
    assert not np.array_equal(ref2, ref)
    np.testing.assert_allclose(_noalloc(g), ref2, rtol=RTOL, atol=0)
    np.testing.assert_allclose(_noalloc(g), ref2, rtol=RTOL, atol=0)


def test_noalloc_rejects_grids_beyond_scratch():
    case = synthetic.linear_rg(6, 8200, nsteps=2)
    g = GpuModel('plain_fp64')
    Driver(case, g).init(with_diag=False)
    with pytest.raises(_lib.SwmGpuError, match='at most 8192'):
        _noalloc(g)
    # the allocating entry point still serves the same context
    assert np.isfinite(g.integrals()).all()
