"""Asynchronous diagnostics output for the host mirror.

Restates the reference's netCDF output of a diagnostics task: the dataset
createDSEuler builds (io_module.f90:305-374: dimensions LONGITUDE, LATITUDE
and an unlimited TIME, the coordinate variables with their units, the
variable with its missing_value attribute) and the time slice putVarEuler
writes (io_module.f90:504-529: missing value on land of the variable's grid
and on non-finite values, the time coordinate, the record count), called
from writeTaskToFile (diagTask.f90:231-253).

The reference writes synchronously inside the time loop.  Here a snapshot
is a device-to-host copy into a pinned buffer issued on the model's stream
(swm_gpu_get_field_async), and one writer thread waits for the copy and
writes the record, so the host thread goes on stepping the model while the
copy and the file write are in flight.  Records reach each file in the
order they were submitted.  The files are netCDF-3 classic (CDF-1), written
here directly (no netCDF library on either machine).  A bounded pool of buffers per field shape keeps
the memory fixed: when every buffer is in flight, a submit waits for the
oldest write to finish.
"""
import os
import queue
import struct
import threading

import numpy as np

MISS_VAL_DEF = float(np.float32(1e37))  # default-real literal (include/io.h:32)
TUNIT = 'seconds since 0000-01-01 00:00:00'  # include/io.h:83


def grid_coords(cfg, grid):
    """(lon, lat) in degrees of one grid, as domain_module.f90:121-128 forms
    them from lon_s/lon_e/lat_s/lat_e: H and u on the corners in longitude,
    v and eta half a cell east; H and v on the corners in latitude, u and
    eta half a cell north."""
    nx, ny = cfg['nx'], cfg['ny']
    lon_s, lon_e, lat_s, lat_e = cfg['lon_s'], cfg['lon_e'], cfg['lat_s'], cfg['lat_e']
    lat = (np.arange(ny, dtype=np.float64) * (lat_e - lat_s)) / (ny - 1) + lat_s
    lon = (np.arange(nx, dtype=np.float64) * (lon_e - lon_s)) / (nx - 1) + lon_s
    if grid in ('u', 'eta'):
        lat = lat + (lat_e - lat_s) / (2. * (ny - 1))
    if grid in ('v', 'eta'):
        lon = lon + (lon_e - lon_s) / (2. * (nx - 1))
    return lon, lat


def _nc_name(name):
    b = name.encode()
    return struct.pack('>i', len(b)) + b + b'\0' * (-len(b) % 4)


def _nc_att_list(atts):
    """NC_ATTRIBUTE list of (name, value): str as NC_CHAR, float as NC_DOUBLE."""
    if not atts:
        return struct.pack('>ii', 0, 0)
    out = struct.pack('>ii', 0x0C, len(atts))
    for name, val in atts:
        out += _nc_name(name)
        if isinstance(val, str):
            b = val.encode()
            out += struct.pack('>ii', 2, len(b)) + b + b'\0' * (-len(b) % 4)
        else:
            out += struct.pack('>ii', 6, 1) + struct.pack('>d', float(val))
    return out


class EulerFile:
    """One output dataset of a 2-D variable (createDSEuler) and its records
    (putVarEuler), as a netCDF-3 classic file written here directly: the
    header and the coordinates at creation, then each record (TIME and the
    field, big-endian doubles) appended where the format puts it, and the
    record count in the header updated after every record, so the file is
    complete at any time.  Writing a record releases the interpreter lock
    for the copy to the file."""

    def __init__(self, path, varname, lon, lat, time_unit=TUNIT, missval=MISS_VAL_DEF):
        self.path, self.varname, self.missval = path, varname, missval
        self.nx, self.ny = len(lon), len(lat)
        dims = [('TIME', 0), ('LONGITUDE', self.nx), ('LATITUDE', self.ny)]
        head = b'CDF\x01' + struct.pack('>i', 0)  # magic, numrecs
        head += struct.pack('>ii', 0x0A, len(dims)) + b''.join(_nc_name(n) + struct.pack('>i', l) for n, l in dims)
        head += struct.pack('>ii', 0, 0)  # no global attributes
        # (name, dimension ids, attributes, bytes per record or in all)
        var_defs = [('LONGITUDE', [1], [('units', 'degrees_east'), ('long_name', 'LONGITUDE')], 8 * self.nx),
                    ('LATITUDE', [2], [('units', 'degrees_north'), ('long_name', 'LATITUDE')], 8 * self.ny),
                    ('TIME', [0], [('units', time_unit), ('long_name', 'TIME')], 8),
                    (varname, [0, 2, 1], [('missing_value', missval)], 8 * self.nx * self.ny)]

        def var_list(begins):
            out = struct.pack('>ii', 0x0B, len(var_defs))
            for (name, dimids, atts, vsize), begin in zip(var_defs, begins):
                out += _nc_name(name) + struct.pack('>i', len(dimids)) + b''.join(struct.pack('>i', d) for d in dimids)
                out += _nc_att_list(atts) + struct.pack('>iii', 6, vsize, begin)
            return out

        hlen = len(head) + len(var_list([0] * 4))
        begins = [hlen, hlen + 8 * self.nx]
        self.rec0 = begins[1] + 8 * self.ny
        begins += [self.rec0, self.rec0 + 8]
        self.recsize = 8 + 8 * self.nx * self.ny
        self.f = open(path, 'wb')
        self.f.write(head + var_list(begins))
        self.f.write(np.asarray(lon, dtype='>f8').tobytes())
        self.f.write(np.asarray(lat, dtype='>f8').tobytes())
        self.f.flush()
        self.nrec = 0
        self._land = None  # the land mask of the first record's grid

    def put(self, data, time, ocean=None, records=None):
        """One time slice: missing value where ocean != 1 and where the value
        is not finite; then the time coordinate; nrec + 1.  records: a list
        that also receives a copy of the data as given."""
        if records is not None:
            records.append(np.array(data, dtype=np.float64, copy=True))
        d = np.array(data, dtype=np.float64, copy=True)
        if ocean is not None:
            if self._land is None or self._land.shape != ocean.shape:
                self._land = ocean != 1
            np.copyto(d, self.missval, where=self._land)
        np.copyto(d, self.missval, where=~np.isfinite(d))
        self.f.seek(self.rec0 + self.nrec * self.recsize)
        self.f.write(struct.pack('>d', float(time)))
        self.f.write(d.astype('>f8').tobytes())
        self.nrec += 1
        self.f.seek(4)
        self.f.write(struct.pack('>i', self.nrec))
        self.f.flush()

    def close(self):
        if self.f is not None:
            self.f.close()
            self.f = None


PAGE = 4096


class _Pool:
    """Fixed buffers of one shape, pinned through the library when the
    backend can pin (swm_gpu_host_register).  Each buffer covers whole pages
    of its own allocation, so no two pinned ranges share a page."""

    def __init__(self, shape, n, pin):
        self.free = queue.Queue()
        self.pages, self.pin = [], pin
        nbytes = int(np.prod(shape)) * 8
        span = -(-nbytes // PAGE) * PAGE
        for _ in range(n):
            raw = np.empty(span + PAGE, dtype=np.uint8)
            off = (-raw.ctypes.data) % PAGE
            region = raw[off:off + span]
            if pin is not None:
                pin[0](region)
            self.pages.append((raw, region))
            self.free.put(region[:nbytes].view(np.float64).reshape(shape))

    def release(self):
        if self.pin is not None:
            for _, region in self.pages:
                self.pin[1](region)


class AsyncWriter:
    """Writer thread for the diagnostics files of one model.

    submit_field(backend, field, fh, time, ocean): the field's copy as of this
    point of the model's stream goes into a pooled (pinned) buffer; the
    writer thread waits for it and writes the record to fh.
    submit_host(data, fh, time, ocean): a host array (a device mean, the
    streamfunction) written the same way, after a copy.
    Both return at once unless every buffer of the shape is in flight.
    close() writes what is queued, joins the thread and closes the files."""

    def __init__(self, outdir, buffers=4, time_unit=TUNIT, inline=False):
        """inline: write in the calling thread with synchronous reads, as the
        reference does (for comparison)."""
        self.outdir, self.nbuf, self.time_unit, self.inline = outdir, buffers, time_unit, inline
        os.makedirs(outdir, exist_ok=True)
        self.files = {}
        self.pools = {}
        self.q = queue.Queue()
        self.error = None
        self.submitted = 0
        self.from_device = 0  # records submitted as asynchronous device copies
        self.written = 0
        self.thread = threading.Thread(target=self._run, name='swm-writer', daemon=True)
        self.thread.start()

    def file(self, filename, varname, lon, lat):
        if filename not in self.files:
            self.files[filename] = EulerFile(os.path.join(self.outdir, filename), varname, lon, lat, self.time_unit)
        return self.files[filename]

    def _pool(self, shape, backend):
        pin = None
        if backend is not None and hasattr(backend, 'host_register'):
            pin = (backend.host_register, backend.host_unregister)
        key = (shape, id(backend) if pin else None)
        if key not in self.pools:
            self.pools[key] = _Pool(shape, self.nbuf, pin)
        return self.pools[key]

    def submit_field(self, backend, field, fh, time, ocean=None, records=None):
        self._check()
        if self.inline:
            self.submitted += 1
            fh.put(backend.field(field), time, ocean, records)
            self.written += 1
            return
        pool = self._pool((backend.ny, backend.nx), backend)
        buf = pool.free.get()  # waits while every buffer of the shape is in flight
        try:
            ticket = backend.field_async(field, buf)
        except Exception:
            pool.free.put(buf)
            raise
        self.submitted += 1
        self.from_device += 1
        self.q.put((backend, ticket, buf, pool, fh, time, ocean, records))

    def submit_host(self, data, fh, time, ocean=None, records=None):
        self._check()
        if self.inline:
            self.submitted += 1
            fh.put(data, time, ocean, records)
            self.written += 1
            return
        self.submitted += 1
        self.q.put((None, None, np.array(data, dtype=np.float64, copy=True), None, fh, time, ocean, records))

    def _run(self):
        while True:
            item = self.q.get()
            if item is None:
                return
            backend, ticket, buf, pool, fh, time, ocean, records = item
            try:
                if backend is not None:
                    backend.wait(ticket)
                if self.error is None:
                    fh.put(buf, time, ocean, records)
                    self.written += 1
            except Exception as e:  # reported to the host thread at its next call
                self.error = e
            finally:
                if pool is not None:
                    pool.free.put(buf)

    def _check(self):
        if self.error is not None:
            raise RuntimeError('diagnostics writer failed: %r' % (self.error,))

    def close(self):
        if self.thread is not None:
            self.q.put(None)
            self.thread.join()
            self.thread = None
        for fh in self.files.values():
            fh.close()
        for p in self.pools.values():
            p.release()
        self.pools = {}
        self._check()
