"""swm_gpu_integrals_noalloc, the allocation-free domain integrals, against
swm_gpu_integrals through the C ABI.

Some hosts cannot allocate inside their time loop: a model whose device
memory is reserved in full by its own pool, or one that runs other streams
that an implicit device synchronisation of cudaMalloc/cudaFree would stall.
The entry point serves them from one fixed array compiled into the library.
Both entry points run the same reduction kernels with the same block count
and cell areas, so the results must agree bit for bit; two calls in a row
check that the shared scratch is reused cleanly, and the device's free
memory must not move across calls.  Kept in a file that is collected last,
so that it runs both alone in a fresh process and after every other GPU
test.
"""
import ctypes

import numpy as np
import pytest

from swm_gb300 import _lib
from swm_gb300.host import synthetic
from swm_gb300.host.driver import Driver
from swm_gb300.model import GpuModel

pytestmark = pytest.mark.gpu


def _noalloc(g):
    out = np.zeros(3)
    _lib.check(_lib.lib().swm_gpu_integrals_noalloc(g.ctx, out.ctypes.data_as(ctypes.c_void_p)))
    return out


def _free_bytes():
    import torch
    return torch.cuda.mem_get_info()[0]


@pytest.mark.parametrize('path', ['plain_fp64', 'fused_fp32c'])
def test_noalloc_integrals_match_allocating_entry(path):
    case = synthetic.double_gyre((48, 40), biharmonic=True, nsteps=60)
    g = GpuModel(path)
    Driver(case, g).init(with_diag=False)
    g.run(0, 40)
    ref = g.integrals()
    first = _noalloc(g)          # the first call may load kernels and look up the array
    _free_bytes()
    before = _free_bytes()
    second = _noalloc(g)
    third = _noalloc(g)
    assert _free_bytes() == before
    assert np.all(ref[1:] > 0), ref
    for got in (first, second, third):
        np.testing.assert_array_equal(got, ref)
    # the state moves on: the next pair of calls follows it
    g.run(40, 20)
    ref2 = g.integrals()
    assert not np.array_equal(ref2, ref)
    np.testing.assert_array_equal(_noalloc(g), ref2)
    np.testing.assert_array_equal(_noalloc(g), ref2)


def test_noalloc_serves_the_largest_grid():
    """A grid of exactly SWM_NOALLOC_MAX_NY = 8192 rows fits the scratch."""
    case = synthetic.linear_rg(6, 8191, nsteps=4)
    g = GpuModel('plain_fp64')
    Driver(case, g).init(with_diag=False)
    assert case['config']['ny'] == 8192
    g.run(0, 3)
    ref = g.integrals()
    np.testing.assert_array_equal(_noalloc(g), ref)
    np.testing.assert_array_equal(_noalloc(g), ref)


def test_noalloc_rejects_grids_beyond_scratch():
    case = synthetic.linear_rg(6, 8200, nsteps=2)
    g = GpuModel('plain_fp64')
    Driver(case, g).init(with_diag=False)
    with pytest.raises(_lib.SwmGpuError, match='at most 8192'):
        _noalloc(g)
    # the allocating entry point still serves the same context
    assert np.isfinite(g.integrals()).all()
