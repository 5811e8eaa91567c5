"""The asynchronous diagnostics writer on the GPU: snapshots leave the
device as asynchronous copies into pinned buffers (swm_gpu_get_field_async
into arrays pinned by swm_gpu_host_register) while the host thread steps on,
and the files hold what the oracle's synchronous run writes: bit for bit on
the plain FP64 path (test_fixed_length_output, the reference's own
configuration), to the path's tolerance on the FP32 pair path."""
import numpy as np
import pytest

from harness import golden_case
from oracle import OracleBackend
from swm_gb300.host.driver import Driver
from swm_gb300.host.writer import MISS_VAL_DEF, AsyncWriter
from swm_gb300.model import GpuModel

pytestmark = pytest.mark.gpu

FILES = ('u_snapshot.nc', 'u_average.nc')


def _records(path, var):
    from scipy.io import netcdf_file
    nc = netcdf_file(path, 'r', mmap=False)
    out = np.array(nc.variables[var].data), np.array(nc.variables['TIME'].data)
    nc.close()
    return out


def _write(backend, outdir):
    case, extra = golden_case('test_fixed_length_output')
    w = AsyncWriter(str(outdir), buffers=2)
    drv = Driver(case, backend, writer=w)
    drv.init()
    drv.run()
    drv.finish()
    return w, extra


@pytest.mark.parametrize('path,tol', [('plain_fp64', 0.0), ('fused_fp32c', 1e-5)])
def test_async_writer_files_match_the_oracle(tmp_path, path, tol):
    wo, extra = _write(OracleBackend(), tmp_path / 'oracle')
    g = GpuModel(path)
    wg, _ = _write(g, tmp_path / 'gpu')
    assert wg.from_device > 0 and wg.written == wg.submitted
    for fn in FILES:
        var = str(extra['var__' + fn])
        a, ta = _records(str(tmp_path / 'oracle' / fn), var)
        b, tb = _records(str(tmp_path / 'gpu' / fn), var)
        assert np.array_equal(ta, tb) and a.shape == b.shape == extra['data__' + fn].shape
        land = a == MISS_VAL_DEF
        assert np.array_equal(land, b == MISS_VAL_DEF)
        if tol == 0.0:
            assert np.array_equal(a, b), fn
        else:
            assert np.abs(a[~land] - b[~land]).max() <= tol * np.abs(a[~land]).max(), fn
    g.close()
