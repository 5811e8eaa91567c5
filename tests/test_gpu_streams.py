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


def _emf_case(nsteps, comps):
    """The double gyre with time-dependent eddy momentum flux streams
    (processEddyMomentumFlux, swm_forcing_module.f90:451-523): smooth random
    flux records of 0.5 m^2/s^2 on the H points, three records 900 s apart."""
    case = synthetic.double_gyre((48, 40), biharmonic=True, nsteps=nsteps)
    ny, nx = case['config']['ny'], case['config']['nx']
    rng = np.random.default_rng(17)
    k = np.fft.fftfreq(nx)[None, :] ** 2 + np.fft.fftfreq(ny)[:, None] ** 2
    for comp in comps:
        recs = []
        for _ in range(3):
            f = np.fft.ifft2(np.fft.fft2(rng.standard_normal((ny, nx))) * np.exp(-k * 36.0)).real
            recs.append(0.5 * f / np.abs(f).max())
        case['streams'].append(dict(type=4, comp=comp, omega=0.0, rec1=np.stack(recs), dt1=900.0, chunksize=2,
                                    rec2=None, dt2=0.0))
    return case


@pytest.mark.parametrize('path', ['plain_fp64', 'fused_fp64', 'fused_fp32c'])
def test_eddy_momentum_flux_forcing(path):
    """U2, V2 and REY eddy momentum flux streams: the plain path bit for bit
    with the oracle, the fused paths (the flux divergence added to their
    forcing fields every step) to their tolerances."""
    nsteps = 120
    case = _emf_case(nsteps, (3, 4, 5))
    o = OracleBackend()
    run_case(case, o, nsteps=nsteps, with_diag=False)
    g = _run(case, path, nsteps, True)
    for f in ('u', 'v', 'eta'):
        m = o.ocean(f).astype(bool)
        if path == 'plain_fp64':
            assert np.array_equal(g.field(f), o.field(f)), f
        else:
            assert rel_l2(g.field(f), o.field(f), m) <= (1e-11 if path == 'fused_fp64' else 1e-5), f
    if path == 'plain_fp64':
        for f in ('F_x', 'F_y'):
            assert np.array_equal(g.field(f), o.field(f)), f
            assert np.abs(o.field(f)).max() > 0
