"""Python view of one GPU model instance (the Fortran module entry points of
swm_module / swm_timestep_module / tracer_module / ElSolv_SOR, bound through
the C ABI).  Also the GPU backend of ``host.driver.Driver``.
"""
import ctypes as C
import numpy as np

from ._lib import lib, check, Config, CONFIG_INT, CONFIG_DBL, FIELD_ID, PATHS

TRC_FIELD = {'CH': 0, 'C': 1, 'G': 2, 'uhc': 3, 'vhc': 4, 'diff': 5, 'impl': 6}


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class GpuModel:
    """One SWM model on the GPU.  ``path`` selects plain_fp64 (drop-in),
    fused_fp64 or fused_fp32c."""

    def __init__(self, path='plain_fp64', tracer_nan_guard=False):
        self.L = lib()
        self.path = PATHS[path] if isinstance(path, str) else int(path)
        self.ctx = None
        self.nan_guard = tracer_nan_guard

    def close(self):
        if self.ctx:
            self.L.swm_gpu_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- init sequence -------------------------------------------------
    def setup_domain(self, case):
        cfg = case['config']
        c = Config()
        for n in CONFIG_INT:
            setattr(c, n, int(cfg.get(n, 0)))
        for n in CONFIG_DBL:
            setattr(c, n, float(cfg.get(n, 0.0)))
        if self.nan_guard:
            c.tracer_nan_guard = 1
        c.path = self.path
        self._cfg = c
        self.nx, self.ny = cfg['nx'], cfg['ny']
        ctx = C.c_void_p()
        check(self.L.swm_gpu_create(C.byref(c), C.byref(ctx)))
        self.ctx = ctx
        H = _f64(case.get('H'))
        miss = None if case.get('H_missing') is None else np.ascontiguousarray(case['H_missing'], np.int8)
        check(self.L.swm_gpu_domain(self.ctx, _p(H), _p(miss)))

    def timestep_init(self, psi_bs):
        p = _f64(psi_bs)
        check(self.L.swm_gpu_timestep_init(self.ctx, _p(p)))

    def add_damping(self, d):
        fd = _f64(d['file_data'])
        check(self.L.swm_gpu_add_damping(self.ctx, d['term'], d['type'], d['value'], d['sl_length'],
                                         d['sl_cutoff'], d['loc'], _p(fd)))

    def finish_damping(self):
        check(self.L.swm_gpu_finish_damping(self.ctx))

    def add_stream(self, s, is_const, d1, d2):
        a, b = _f64(d1), _f64(d2)
        sid = C.c_int()
        check(self.L.swm_gpu_add_stream(self.ctx, s['type'], s['comp'], s['omega'], int(is_const),
                                        _p(a), _p(b), C.byref(sid)))
        return sid.value

    def set_stream_data(self, sid, d1, d2):
        a, b = _f64(d1), _f64(d2)
        check(self.L.swm_gpu_set_stream_data(self.ctx, sid, _p(a), _p(b)))

    def stream_records(self, sid, part, records):
        r = np.ascontiguousarray(records, dtype=np.float64)
        check(self.L.swm_gpu_stream_records(self.ctx, sid, part, r.shape[0], _p(r)))

    def stream_interp(self, sid, part, bracket):
        r0, r1, t, t0, t1 = bracket
        check(self.L.swm_gpu_stream_interp(self.ctx, sid, part, r0, r1, t, t0, t1))

    def set_stream_rows(self, sid, r1, r2=None):
        a, b = _f64(r1), _f64(r2)
        check(self.L.swm_gpu_set_stream_rows(self.ctx, sid, _p(a), _p(b)))

    def integrals(self):
        out = np.zeros(3)
        check(self.L.swm_gpu_integrals(self.ctx, _p(out)))
        return out

    def integrals_async(self, out3):
        """Start the domain integrals into out3 (3 float64, ideally pinned);
        returns a ticket for wait()."""
        t = C.c_int64()
        check(self.L.swm_gpu_integrals_async(self.ctx, _p(out3), C.byref(t)))
        return t.value

    def forcing_init(self):
        check(self.L.swm_gpu_forcing_init(self.ctx))

    def initial_conditions(self, eta, u, v):
        e, uu, vv = _f64(eta), _f64(u), _f64(v)
        check(self.L.swm_gpu_initial_conditions(self.ctx, _p(e), _p(uu), _p(vv)))

    def add_tracer(self, t):
        arrs = [_f64(t.get('field_C')), _f64(t.get('field_C0')), _f64(t.get('field_gamma_C')),
                _f64(t.get('field_cons'))]
        tid = C.c_int()
        check(self.L.trc_gpu_add(self.ctx, t['kappa_h'], t['cons'], t['gamma_c'], *[_p(a) for a in arrs],
                                 C.byref(tid)))
        return tid.value

    def tracer_init(self):
        check(self.L.trc_gpu_init(self.ctx))

    # -- time loop -----------------------------------------------------
    def step(self, itt):
        check(self.L.swm_gpu_step(self.ctx, itt))

    def advance(self, itt):
        check(self.L.swm_gpu_advance(self.ctx, itt))

    def run(self, itt0, nsteps):
        check(self.L.swm_gpu_run(self.ctx, itt0, nsteps))

    def run_monitor(self, itt0, nsteps, sid, rows1, out3, rows2=None):
        """swm_gpu_run_monitor: rows1 (nsteps, Ny) per-step row profiles of
        stream sid (or None), out3 (nsteps, 3) receives each step's integrals."""
        assert out3.shape == (nsteps, 3) and out3.flags.c_contiguous and out3.dtype == np.float64
        for r in (rows1, rows2):
            assert r is None or (r.shape == (nsteps, self.ny) and r.flags.c_contiguous and r.dtype == np.float64)
        check(self.L.swm_gpu_run_monitor(self.ctx, itt0, nsteps, sid, _p(rows1), _p(rows2), _p(out3)))

    def synchronize(self):
        check(self.L.swm_gpu_synchronize(self.ctx))

    def launch_count(self):
        return self.L.swm_gpu_launch_count(self.ctx)

    def step_shape(self):
        """(rows per warp strip, masked-row cost, blocks) of the FP32 step
        kernel's tiles, zeros before the first step."""
        rows, cost, blocks = C.c_double(), C.c_double(), C.c_int()
        check(self.L.swm_gpu_step_shape(self.ctx, C.byref(rows), C.byref(cost), C.byref(blocks)))
        return rows.value, cost.value, blocks.value

    def stream(self):
        return self.L.swm_gpu_stream(self.ctx)

    # -- host access ---------------------------------------------------
    _ALIAS = {'tot_u': 'u', 'tot_v': 'v', 'tot_eta': 'eta'}

    def field(self, name):
        name = self._ALIAS.get(name, name)
        out = np.empty((self.ny, self.nx))
        check(self.L.swm_gpu_get_field(self.ctx, FIELD_ID[name], _p(out)))
        return out

    def field_async(self, name, out):
        """Start the copy of a field into out (a C-contiguous float64 array,
        ideally in pinned memory); returns a ticket for wait()/ready()."""
        name = self._ALIAS.get(name, name)
        assert out.flags.c_contiguous and out.dtype == np.float64 and out.size == self.nx * self.ny
        t = C.c_int64()
        check(self.L.swm_gpu_get_field_async(self.ctx, FIELD_ID[name], _p(out), C.byref(t)))
        return t.value

    def wait(self, ticket):
        check(self.L.swm_gpu_wait(self.ctx, ticket))

    def ready(self, ticket):
        return self.L.swm_gpu_ready(self.ctx, ticket)

    def host_register(self, arr):
        """Pin a host array (swm_gpu_host_register) for asynchronous copies."""
        check(self.L.swm_gpu_host_register(_p(arr), arr.nbytes))

    def host_unregister(self, arr):
        check(self.L.swm_gpu_host_unregister(_p(arr)))

    def set_field(self, name, arr):
        a = _f64(arr)
        check(self.L.swm_gpu_set_field(self.ctx, FIELD_ID[self._ALIAS.get(name, name)], _p(a)))

    def lat(self, name):
        which, grid = name.split('_')
        out = np.empty(self.ny)
        check(self.L.swm_gpu_get_metric(self.ctx, ['lat', 'cos', 'tan', 'f'].index(which),
                                        ['H', 'u', 'v', 'eta'].index(grid), _p(out)))
        return out

    def ocean(self, grid):
        out = np.empty((self.ny, self.nx), dtype=np.int8)
        check(self.L.swm_gpu_get_mask(self.ctx, ['H', 'u', 'v', 'eta'].index(grid), _p(out)))
        return out

    def diag_accumulate(self, slot, name, square, weight):
        """Device time-averaging buffer (swm_gpu_diag_accumulate)."""
        fid = FIELD_ID[self._ALIAS.get(name, name)]
        check(self.L.swm_gpu_diag_accumulate(self.ctx, slot, fid, int(bool(square)), float(weight)))

    def diag_mean(self, slot):
        out = np.empty((self.ny, self.nx))
        cnt = C.c_double()
        check(self.L.swm_gpu_diag_mean(self.ctx, slot, _p(out), C.byref(cnt)))
        return out, cnt.value

    def streamfunction(self):
        out = np.empty((self.ny, self.nx))
        check(self.L.swm_gpu_streamfunction(self.ctx, _p(out)))
        return out

    def tracer_field(self, t, name):
        out = np.empty((self.ny, self.nx))
        check(self.L.trc_gpu_get_field(self.ctx, t, TRC_FIELD[name], _p(out)))
        return out

    def nondivergent(self, first_guess, eps=1e-4):
        """computeNonDivergentFlowField of the current state: (u_nd, v_nd,
        chi, SOR iterations, status)."""
        u, v, chi = (np.empty((self.ny, self.nx)) for _ in range(3))
        it = C.c_int()
        rc = self.L.swm_gpu_nondivergent(self.ctx, int(bool(first_guess)), eps, _p(u), _p(v), _p(chi),
                                         C.byref(it))
        if rc not in (0, 4):
            check(rc)
        return u, v, chi, it.value, rc

    # -- SOR -----------------------------------------------------------
    def sor_init(self):
        check(self.L.elsolv_sor_gpu_init(self.ctx))

    def sor_solve(self, B, chi, eps, first_guess):
        b = _f64(B)
        x = np.ascontiguousarray(chi, np.float64).copy()
        it, an = C.c_int(), C.c_double()
        rc = self.L.elsolv_sor_gpu_solve(self.ctx, _p(b), _p(x), eps, int(first_guess), C.byref(it), C.byref(an))
        if rc not in (0, 4):
            check(rc)
        return x, (it.value if rc == 0 else -it.value), an.value


class GpuEnsemble:
    """Members (GpuModel, fused_fp32c, initialised) stepped together by one
    persistent launch per step (swm_gpu_ensemble_*)."""

    def __init__(self, members):
        self.L = lib()
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m.ctx for m in self.members])
        out = C.c_void_p()
        check(self.L.swm_gpu_ensemble_create(arr, len(self.members), C.byref(out)))
        self.ens = out

    def close(self):
        if self.ens:
            self.L.swm_gpu_ensemble_destroy(self.ens)
            self.ens = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, itt0, nsteps):
        check(self.L.swm_gpu_ensemble_run(self.ens, itt0, nsteps))

    def integrals(self):
        out = np.zeros((len(self.members), 3))
        check(self.L.swm_gpu_ensemble_integrals(self.ens, _p(out)))
        return out

    def run_monitor(self, itt0, nsteps, rows, out):
        """nsteps monitored steps: rows (nsteps x sum of the members' Ny,
        float64, C order; None: no wind update) feed each step's zonal wind
        rows, out (nsteps x members x 3, float64) receives each step's
        integrals.  Pinned arrays keep the copies asynchronous."""
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.shape == (nsteps, len(self.members), 3)
        if rows is not None:
            assert rows.dtype == np.float64 and rows.flags.c_contiguous and rows.shape[0] == nsteps
        check(self.L.swm_gpu_ensemble_run_monitor(self.ens, itt0, nsteps, None if rows is None else _p(rows),
                                                   _p(out)))

    def synchronize(self):
        check(self.L.swm_gpu_ensemble_synchronize(self.ens))

    def stream(self):
        return self.L.swm_gpu_ensemble_stream(self.ens)

    def launch_count(self):
        return self.L.swm_gpu_ensemble_launch_count(self.ens)

    def rows(self):
        return self.L.swm_gpu_ensemble_rows(self.ens)


class GpuHelmholtz:
    """div(H^-1 grad psi) - lam psi = rhs solved by red-black SOR on the GPU
    (swm_helm_*): FP64 sweeps or FP32 sweeps with FP64 refinement."""

    def __init__(self, H, ocean, dx, dy, lam):
        self.L = lib()
        self.shape = H.shape
        ny, nx = H.shape
        h = _f64(H)
        m = np.ascontiguousarray(ocean, dtype=np.int8)
        out = C.c_void_p()
        check(self.L.swm_helm_create(nx, ny, dx, dy, lam, _p(h), _p(m), C.byref(out)))
        self.h = out

    def close(self):
        if self.h:
            self.L.swm_helm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def apply(self, psi):
        out = np.zeros(self.shape)
        check(self.L.swm_helm_apply(self.h, _p(_f64(psi)), _p(out)))
        return out

    def solve(self, rhs, psi0=None, omega=1.9, rtol=1e-10, max_sweeps=100000, mixed=False, inner_tol=1e-4,
              raise_on_fail=True):
        psi = np.zeros(self.shape) if psi0 is None else np.array(psi0, dtype=np.float64)
        b = _f64(rhs)
        sw, outer, rel = C.c_int(), C.c_int(), C.c_double()
        if mixed:
            rc = self.L.swm_helm_solve_mixed(self.h, _p(b), _p(psi), omega, rtol, inner_tol, max_sweeps,
                                             C.byref(sw), C.byref(outer), C.byref(rel))
        else:
            rc = self.L.swm_helm_solve_fp64(self.h, _p(b), _p(psi), omega, rtol, max_sweeps, C.byref(sw),
                                            C.byref(rel))
        if raise_on_fail or rc not in (0, 4):
            check(rc)
        return psi, sw.value, outer.value, rel.value, rc

    def autotune(self, rhs, lo=1.8, hi=1.99, ngrid=12, trial_sweeps=64):
        om, bx, by = C.c_double(), C.c_int(), C.c_int()
        check(self.L.swm_helm_autotune(self.h, _p(_f64(rhs)), lo, hi, ngrid, trial_sweeps, C.byref(om),
                                       C.byref(bx), C.byref(by)))
        return om.value, (bx.value, by.value)

    def stream(self):
        return self.L.swm_helm_stream(self.h)

    def launch_count(self):
        return self.L.swm_helm_launch_count(self.h)
