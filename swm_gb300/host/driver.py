"""Host time loop and diagnostics (restates model.f90 initModel/timestepModel,
swm_forcing_module stream bookkeeping and diagTask.f90 processTask).

The driver is backend-agnostic: a backend implements the SWM/tracer entry
points (``setup_domain``, ``timestep_init``, ``add_damping``,
``finish_damping``, ``add_stream``, ``set_stream_data``, ``forcing_init``,
``initial_conditions``, ``add_tracer``, ``tracer_init``, ``step``,
``advance``, ``field``, ``streamfunction``) and the driver supplies what the
Fortran host would: time-interpolated input records and the diagnostics
cadence.  The GB300 path and the CPU oracle are both driven through it.
"""
import math
import numpy as np

from .memchunk import MemChunk
from .case import MODE_NONLINEAR

# registry name -> (backend field name, grid of the output mask)
DIAG_VARS = {
    'U': ('tot_u', 'u'), 'V': ('tot_v', 'v'), 'ETA': ('tot_eta', 'eta'),
    'SWM_U': ('u', 'u'), 'SWM_V': ('v', 'v'), 'SWM_ETA': ('eta', 'eta'),
    'PSI': ('psi', 'H'), 'H': ('H', 'H'), 'H_U': ('H_u', 'u'), 'H_V': ('H_v', 'v'), 'H_ETA': ('H_eta', 'eta'),
    'IMPL_U': ('impl_u', 'u'), 'IMPL_V': ('impl_v', 'v'), 'IMPL_ETA': ('impl_eta', 'eta'),
    'GAMMA_LIN_U': ('gamma_lin_u', 'u'), 'GAMMA_LIN_V': ('gamma_lin_v', 'v'),
    'GAMMA_LIN_ETA': ('gamma_lin_eta', 'eta'),
    'SWM_EDENS': ('edens', 'eta'), 'SWM_POT': ('pot', 'H'), 'SWM_RELVORT': ('zeta', 'H'),
    'SWM_MU': ('mu', 'u'), 'SWM_MV': ('mv', 'v'), 'SWM_D': ('D', 'eta'),
    'F_X': ('F_x', 'u'), 'F_Y': ('F_y', 'v'), 'F_ETA': ('F_eta', 'eta'),
}


class DiagTask:
    """One &diag_nl entry (diagTask.f90:266-335)."""

    def __init__(self, spec, Nt, dsi, dt, meant_out):
        self.spec = spec
        self.name = spec['varname'].upper()
        self.type = spec['type']
        self.period = spec['period']
        self.square = spec['process'] == 'S'
        self.dt, self.dsi, self.meant_out = dt, dsi, meant_out
        self.nstep = max(int((Nt - dsi) // spec['frequency']), 1) if self.type == 'S' and spec['frequency'] > 0 else 1
        self.buffer = None
        self.count = 0.0
        self.times, self.records = [], []

    def _add(self, data, dT):
        d = data * data if self.square else data
        if self.buffer is None:
            self.buffer = np.zeros_like(d)
        self.buffer = self.buffer + dT * d
        self.count = self.count + dT

    def process(self, itt, fetch, device=None, slot=None, emit=None):
        """device: a backend with diag_accumulate/diag_mean (the averaging
        buffer then lives on the GPU and one field crosses per period).
        emit(task, time, data): where a record goes (data None: the task's
        variable as of now); default: kept in self.times / self.records."""
        self._emit = emit or (lambda task, time, data: task._keep(time, fetch(task.name) if data is None else data))
        if device is not None and self.type == 'A':
            return self._process_device(itt, device, slot)
        return self._process_host(itt, fetch)

    def _keep(self, time, data):
        self.times.append(time)
        self.records.append(np.array(data, copy=True))

    def _process_device(self, itt, dev, slot):
        k = itt - self.dsi
        if math.fmod(k, self.nstep) != 0:
            return
        per = self.period if self.period != 2.628e6 else self.meant_out
        dT = min(math.fmod(self.dt * k, per), self.dt)
        field = DIAG_VARS[self.name][0]
        if dT < self.dt and k != 0:
            dev.diag_accumulate(slot, field, self.square, self.dt - dT)
            mean, _ = dev.diag_mean(slot)
            self._emit(self, self.dt * itt - dT, mean)
        dev.diag_accumulate(slot, field, self.square, dT)

    def _process_host(self, itt, fetch):
        k = itt - self.dsi
        if math.fmod(k, self.nstep) != 0:
            return
        if self.type == 'S':
            self._emit(self, itt * self.dt, None)
        elif self.type == 'A':
            per = self.period if self.period != 2.628e6 else self.meant_out
            dT = min(math.fmod(self.dt * k, per), self.dt)
            data = fetch(self.name)
            if dT < self.dt and k != 0:
                self._add(data, self.dt - dT)
                self.buffer = self.buffer / self.count
                self._emit(self, self.dt * itt - dT, self.buffer.copy())
                self.buffer = np.zeros_like(self.buffer)
                self.count = 0.0
            self._add(data, dT)
        elif self.type == 'I':
            if itt == 0:
                self._emit(self, 0.0, None)


class Driver:
    def __init__(self, case, backend, device_averages=True, device_streams=True, writer=None):
        """writer: an AsyncWriter (host/writer.py); each diagnostics record
        then also goes to the task's netCDF file, snapshots as asynchronous
        device copies, so the time loop does not wait for them."""
        self.case, self.b = case, backend
        self.writer = writer
        self.device_averages = device_averages
        # time-dependent forcing records kept on the device, interpolated there
        self.device_streams = device_streams and hasattr(backend, 'stream_interp')
        self.cfg = case['config']
        self.itt = 0
        self.tasks = []
        self._psi_cache = None
        self._masks = {}

    # -- init sequence: model.f90 initModel :71-144 ---------------------
    def init(self, with_diag=True):
        c, b, case = self.cfg, self.b, self.case
        b.setup_domain(case)
        b.timestep_init(case.get('psi_bs'))
        for d in case['damping']:
            b.add_damping(d)
        b.finish_damping()
        self.chunks = []
        for s in case['streams']:
            mc1 = MemChunk(s['rec1'], s['dt1'], s['chunksize'])
            mc2 = MemChunk(s['rec2'], s['dt2'], s['chunksize']) if s['rec2'] is not None else None
            tdf = (s['type'] == 1) or (s['type'] == 0 and c['mode'] == MODE_NONLINEAR) or not mc1.is_constant
            self.chunks.append((mc1, mc2, tdf))
            d1 = mc1.get(0.0) if not tdf else np.zeros_like(mc1.rec[0])
            d2 = (mc2.get(0.0) if (mc2 is not None and not tdf) else None)
            sid = b.add_stream(s, not tdf, d1, d2)
            if tdf and self.device_streams:
                b.stream_records(sid, 1, mc1.rec)
                if mc2 is not None:
                    b.stream_records(sid, 2, mc2.rec)
        self._feed_streams(0)
        b.forcing_init()
        self._feed_streams(0)
        ic = case['ic']
        b.initial_conditions(ic.get('eta'), ic.get('u'), ic.get('v'))
        for t in case.get('tracers', []):
            b.add_tracer(t)
        if case.get('tracers'):
            b.tracer_init()
        if with_diag:
            self.tasks = [DiagTask(s, c['Nt'], c['diag_start_ind'], c['dt'], c['meant_out'])
                          for s in case['diag']]
            if self.writer is not None:  # createTaskDS (diagTask.f90:344-371) at task set-up
                for t in self.tasks:
                    self._task_file(t)
            self.diag()

    def _feed_streams(self, itt):
        t = itt * self.cfg['dt']
        for sid, (mc1, mc2, tdf) in enumerate(self.chunks):
            if not tdf:
                continue
            if self.device_streams:
                self.b.stream_interp(sid, 1, mc1.bracket(t))
                if mc2 is not None:
                    self.b.stream_interp(sid, 2, mc2.bracket(t))
            else:
                self.b.set_stream_data(sid, mc1.get(t), mc2.get(t) if mc2 is not None else None)

    def fetch(self, name):
        if name == 'PSI':
            if self._psi_cache is None:
                self._psi_cache = self.b.streamfunction()
            return self._psi_cache
        return self.b.field(DIAG_VARS[name][0])

    def diag(self):
        if self.itt < self.cfg['diag_start_ind']:
            return
        self._psi_cache = None
        dev = self.b if self.device_averages and hasattr(self.b, 'diag_accumulate') else None
        emit = self._emit if self.writer is not None else None
        for slot, t in enumerate(self.tasks):
            t.process(self.itt, self.fetch, dev, slot, emit)

    def _emit(self, task, time, data):
        """A record to the task's file through the writer (writeTaskToFile,
        diagTask.f90:231-253): a snapshot of a state field as an asynchronous
        device copy, anything else (means, PSI) from the host.  The writer
        thread appends the record to task.records after writing it."""
        field, grid = DIAG_VARS[task.name]
        fh = self._task_file(task)
        if grid not in self._masks:
            self._masks[grid] = self.b.ocean(grid)
        task.times.append(time)
        if data is None and task.name != 'PSI' and hasattr(self.b, 'field_async'):
            self.writer.submit_field(self.b, field, fh, time, self._masks[grid], records=task.records)
        else:
            self.writer.submit_host(self.fetch(task.name) if data is None else data, fh, time, self._masks[grid],
                                    records=task.records)

    def _task_file(self, task):
        from .writer import grid_coords
        fn = task.spec['filename']
        if fn not in self.writer.files:
            lon, lat = grid_coords(self.cfg, DIAG_VARS[task.name][1])
            self.writer.file(fn, task.spec.get('ovarname') or task.spec['varname'], lon, lat)
        return self.writer.files[fn]

    def finish(self):
        """Writes the records still in flight and closes the output files."""
        if self.writer is not None:
            self.writer.close()

    # -- time loop: model.f90 timestepModel :153-197 ---------------------
    def run(self, nsteps=None, with_diag=True):
        n = self.cfg['Nt'] if nsteps is None else nsteps
        for _ in range(n):
            self.itt += 1
            self.b.step(self.itt)
            self._feed_streams(self.itt)
            self.b.advance(self.itt)
            if with_diag:
                self.diag()

    def outputs(self):
        out = {}
        for t in self.tasks:
            out[t.spec['filename']] = (np.array(t.times), np.array(t.records) if t.records else None,
                                       DIAG_VARS[t.name][1])
        return out
