"""The asynchronous diagnostics writer (swm_gb300/host/writer.py) against
the reference's own output files (selfcheck/test_fixed_length_output and
test_diaglist, their layout kept in the golden fixtures): the datasets it
writes have the reference's dimensions, coordinates, variable names,
missing value and times, and records equal to the reference's (to the
oracle's agreement with them), with the missing value on land."""
import numpy as np
import pytest

from harness import golden_case, run_case
from oracle import OracleBackend
from swm_gb300.host.driver import Driver
from swm_gb300.host.writer import MISS_VAL_DEF, AsyncWriter, grid_coords


def _read(path):
    from scipy.io import netcdf_file
    nc = netcdf_file(path, 'r', mmap=False)
    out = {'dims': dict(nc.dimensions), 'vars': {k: (v.dimensions, dict(v._attributes), np.array(v.data))
                                                  for k, v in nc.variables.items()}}
    nc.close()
    return out


def _run(name, backend, outdir, nsteps=None):
    case, extra = golden_case(name)
    w = AsyncWriter(str(outdir))
    drv = Driver(case, backend, writer=w)
    drv.init()
    drv.run(nsteps)
    drv.finish()
    return case, extra, drv, w


def test_writer_reproduces_the_reference_files(tmp_path):
    b = OracleBackend()
    case, extra, drv, w = _run('test_fixed_length_output', b, tmp_path)
    assert w.written == w.submitted > 0
    for fn in ('u_snapshot.nc', 'u_average.nc'):
        f = _read(str(tmp_path / fn))
        var = str(extra['var__' + fn])
        assert f['dims'] == {'LONGITUDE': 61, 'LATITUDE': 41, 'TIME': None}
        dims, attrs, data = f['vars'][var]
        assert dims == ('TIME', 'LATITUDE', 'LONGITUDE')
        assert attrs['missing_value'] == extra['missval__' + fn][0] == MISS_VAL_DEF
        assert np.array_equal(f['vars']['LONGITUDE'][2], extra['lon__' + fn])
        assert np.array_equal(f['vars']['LATITUDE'][2], extra['lat__' + fn])
        assert np.array_equal(f['vars']['TIME'][2], extra['time__' + fn])
        gold = extra['data__' + fn]
        assert data.shape == gold.shape
        land = gold == MISS_VAL_DEF
        assert np.array_equal(data == MISS_VAL_DEF, land)
        scale = np.abs(gold[~land]).max()
        assert np.abs(data[~land] - gold[~land]).max() <= 5e-16 * scale, fn
    # the in-memory records equal those of a run without the writer
    ref = run_case(golden_case('test_fixed_length_output')[0], OracleBackend())
    for fn, (t, recs, _) in ref.outputs().items():
        t2, recs2, _ = drv.outputs()[fn]
        assert np.array_equal(t, t2) and np.array_equal(recs, recs2), fn


def test_writer_layout_on_every_grid(tmp_path):
    """test_diaglist writes fields of all four grids (H: psi, relvort,
    potvort; u; v; eta): names and coordinates as the reference's files; the
    set-up field H_out.nc record for record."""
    case, extra = golden_case('test_diaglist')
    b = OracleBackend()
    w = AsyncWriter(str(tmp_path))
    drv = Driver(case, b, writer=w)
    drv.init()
    drv.run(3468)
    drv.finish()
    for fn in [k[len('var__'):] for k in extra if k.startswith('var__')]:
        f = _read(str(tmp_path / fn))
        var = str(extra['var__' + fn])
        assert var in f['vars'], (fn, var)
        assert np.array_equal(f['vars']['LONGITUDE'][2], extra['lon__' + fn]), fn
        assert np.array_equal(f['vars']['LATITUDE'][2], extra['lat__' + fn]), fn
    h = _read(str(tmp_path / 'H_out.nc'))['vars'][str(extra['var__H_out.nc'])][2]
    gold = extra['data__H_out.nc']
    assert np.array_equal(h[0], gold[0])


@pytest.mark.parametrize('grid', ['H', 'u', 'v', 'eta'])
def test_grid_coords_follow_domain_module(grid):
    cfg = dict(nx=5, ny=3, lon_s=-30.0, lon_e=0.0, lat_s=-10.0, lat_e=10.0)
    lon, lat = grid_coords(cfg, grid)
    assert np.allclose(lon, np.linspace(-30, 0, 5) + (3.75 if grid in ('v', 'eta') else 0))
    assert np.allclose(lat, np.linspace(-10, 10, 3) + (5.0 if grid in ('u', 'eta') else 0))
