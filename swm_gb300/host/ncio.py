"""netCDF-3 input reading for the host mirror (restates the parts of
io_module.f90 the configuration path needs: last-record reads with missing
value masks, :198-204 and :596-617, and the record time spacing used by
memchunk_module getDt :259-277)."""
import re
import numpy as np

_UNITS = {'second': 1.0, 'seconds': 1.0, 'sec': 1.0, 's': 1.0, 'minute': 60.0, 'minutes': 60.0,
          'hour': 3600.0, 'hours': 3600.0, 'day': 86400.0, 'days': 86400.0}


def _open(path):
    from scipy.io import netcdf_file
    return netcdf_file(path, 'r', mmap=False)


def _time_var(nc, var):
    for d in var.dimensions:
        if d in nc.variables and d not in ('LATITUDE', 'LONGITUDE') and nc.dimensions.get(d, 1) != 0:
            v = nc.variables[d]
            if len(v.dimensions) == 1 and len(var.dimensions) == 3 and d == var.dimensions[0]:
                return v
    return None


def read_records(path, varname):
    """All records of a variable as float64 (nrec, ny, nx), the missing mask
    of the last record, and the record spacing in seconds."""
    nc = _open(path)
    try:
        v = nc.variables[varname]
        data = np.array(v.data, dtype=np.float64)
        if data.ndim == 2:
            data = data[None]
        miss = np.zeros(data.shape[1:], dtype=np.int8)
        for att in ('missing_value', '_FillValue'):
            if att in v._attributes:
                mv = float(np.asarray(v._attributes[att]).ravel()[0])
                miss[data[-1] == mv] = 1
        dt = 0.0
        tv = _time_var(nc, v)
        if tv is not None and data.shape[0] > 1:
            units = tv._attributes.get('units', b'seconds').decode()
            scale = _UNITS.get(units.split()[0].lower(), 1.0)
            t = np.array(tv.data, dtype=np.float64) * scale
            dt = (t[-1] - t[0]) / float(np.float32(data.shape[0] - 1))
        return data, miss, dt
    finally:
        nc.close()


def read_last(path, varname):
    data, miss, _ = read_records(path, varname)
    return data[-1].copy(), miss
