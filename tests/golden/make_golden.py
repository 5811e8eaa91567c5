"""Packs the reference's selfcheck runs into self-contained fixtures.

Reads <reference>/selfcheck/<case>/{model.h, model.namelist, input/*.nc,
output/reference_*.nc} and writes tests/golden/<case>.npz with the resolved
configuration, the input fields and the reference's FP64 output records
(the goldens the oracle is pinned against).

selfcheck/test_nonlinear and selfcheck/test_nl_tracer ship their
configuration and inputs but not their outputs (the reference tree lists
those as missing large files), so they are packed as inputs only: they are
the reference's own configurations of the nonlinear and tracer paths on the
real sphere (A = 6371 km, 25S-25N), which the GPU paths are checked on
against the oracle.

Run once where the reference tree is mounted:
    python tests/golden/make_golden.py <path of the swm source tree>
"""
import os
import sys
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from swm_gb300.host.case import load_case          # noqa: E402
from swm_gb300.host.caseio import save_case        # noqa: E402

CASES = {
    'test_fixed_length_output': ['u_snapshot.nc', 'u_average.nc'],
    'test_oscfrc': ['taux.nc'],
    'test_diaglist': ['u_out.nc', 'v_out.nc', 'eta_out.nc', 'psi_out.nc', 'u_mean_out.nc', 'eta2_mean_out.nc',
                      'H_out.nc', 'impl_u.nc', 'impl_v.nc', 'impl_n.nc', 'gamma_u.nc', 'gamma_v.nc', 'gamma_n.nc',
                      'edens.nc', 'potvort.nc', 'relvort.nc', 'mu.nc', 'mv.nc', 'd.nc'],
    # inputs only: the outputs of these two runs are not in the source tree
    'test_nonlinear': [],
    'test_nl_tracer': [],
}


def read_output(path):
    """Records, times and the dataset's layout: coordinates, variable name
    and missing value (what the asynchronous writer must reproduce)."""
    from scipy.io import netcdf_file
    nc = netcdf_file(path, 'r', mmap=False)
    var = [k for k in nc.variables if k not in ('LONGITUDE', 'LATITUDE', 'TIME')][0]
    data = np.array(nc.variables[var].data, dtype=np.float64)
    t = np.array(nc.variables['TIME'].data, dtype=np.float64)
    layout = {'lon': np.array(nc.variables['LONGITUDE'].data, dtype=np.float64),
              'lat': np.array(nc.variables['LATITUDE'].data, dtype=np.float64),
              'var': np.array(var),
              'missval': np.array([float(np.asarray(nc.variables[var]._attributes['missing_value']).ravel()[0])])}
    nc.close()
    return t, data, layout


def main(ref):
    for name, outs in CASES.items():
        d = os.path.join(ref, 'selfcheck', name)
        case = load_case(d)
        # only the diag tasks whose outputs are kept
        case['diag'] = [t for t in case['diag'] if t['filename'] in outs]
        extra = {}
        for fn in outs:
            t, data, layout = read_output(os.path.join(d, 'output', 'reference_000000000001_' + fn))
            extra['time__' + fn] = t
            extra['data__' + fn] = data
            for k, v in layout.items():
                extra[k + '__' + fn] = v
        save_case(os.path.join(HERE, name + '.npz'), case, extra)
        print(name, os.path.getsize(os.path.join(HERE, name + '.npz')))


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: make_golden.py <path of the swm source tree>')
    main(sys.argv[1])
