"""Time-dependent forcing records kept on the device and interpolated there
(swm_gpu_stream_records / swm_gpu_stream_interp) against the host
interpolation that uploads each step's field."""
import numpy as np
import pytest

from harness import golden_case, rel_l2, run_case
from oracle import OracleBackend
from swm_gb300.host import synthetic
from swm_gb300.host.driver import Driver
from swm_gb300.model import GpuModel

pytestmark = pytest.mark.gpu


def _run(case, path, nsteps, device_streams):
    g = GpuModel(path)
    d = Driver(case, g, device_streams=device_streams)
    d.init(with_diag=False)
    d.run(nsteps, with_diag=False)
    return g


def test_device_interpolation_equals_host_upload():
    case, _ = golden_case('test_oscfrc')
    a = _run(case, 'plain_fp64', 300, True)
    b = _run(case, 'plain_fp64', 300, False)
    for f in ('u', 'v', 'eta', 'F_x', 'F_y', 'F_eta'):
        assert np.array_equal(a.field(f), b.field(f)), f


def _varying_wind_case(nsteps):
    case = synthetic.double_gyre((48, 40), biharmonic=True, nsteps=nsteps)
    s = case['streams'][0]
    rec = s['rec1'][0]
    s.update(rec1=np.stack([rec, 0.3 * rec, 1.7 * rec]), dt1=900.0, chunksize=2)
    return case


@pytest.mark.parametrize('path', ['plain_fp64', 'fused_fp32c'])
def test_time_dependent_wind_on_device(path):
    nsteps = 200
    case = _varying_wind_case(nsteps)
    o = OracleBackend()
    run_case(case, o, nsteps=nsteps, with_diag=False)
    g = _run(case, path, nsteps, True)
    for f in ('u', 'v', 'eta'):
        m = o.ocean(f).astype(bool)
        if path == 'plain_fp64':
            assert np.array_equal(g.field(f), o.field(f)), f
        else:
            assert rel_l2(g.field(f), o.field(f), m) <= 1e-5, f
