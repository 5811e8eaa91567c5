"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, __graft_entry__.smoke() and the cpu_baseline leg of
bench.py to check the GB300 path; never by the product.  Builds
``oracle/_build/libswm_oracle.so`` on first use if it is missing.
"""
import ctypes as C
import os
import subprocess
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, '_build', 'libswm_oracle.so')

FIELDS = ['u0', 'u1', 'v0', 'v1', 'eta0', 'eta1', 'gu1', 'gu2', 'gu3', 'gv1', 'gv2', 'gv3',
          'geta1', 'geta2', 'geta3', 'D', 'Dh', 'Du', 'Dv', 'edens', 'pot', 'zeta', 'mu', 'mv',
          'H', 'H_u', 'H_v', 'H_eta', 'impl_u', 'impl_v', 'impl_eta', 'gamma_sq_u', 'gamma_sq_v',
          'gamma_lin_u', 'gamma_lin_v', 'gamma_lin_eta', 'F_x', 'F_y', 'F_eta', 'F_x_const',
          'F_y_const', 'F_eta_const', 'u_bs', 'v_bs', 'zeta_bs', 'psi_bs', 'latmix_u', 'latmix_v',
          'pll', 'plt', 'tot_u', 'tot_v', 'tot_eta', 'bc_H', 'bc_u', 'bc_v', 'bc_eta']
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}
FIELD_ID.update({'u': FIELD_ID['u0'], 'v': FIELD_ID['v0'], 'eta': FIELD_ID['eta0']})
LATS = ['lat_H', 'lat_u', 'lat_v', 'lat_eta', 'cos_H', 'cos_u', 'cos_v', 'cos_eta',
        'tan_H', 'tan_u', 'tan_v', 'tan_eta', 'f_H', 'f_u', 'f_v', 'f_eta']
TRC_FIELDS = ['CH0', 'CH1', 'G1', 'G2', 'G3', 'C', 'C0', 'gamma', 'impl', 'uhc', 'vhc', 'diff', 'forcing']


class Config(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ('nx', 'ny', 'mode', 'lateral_mixing', 'quadratic_friction',
                                          'barotropic', 'mixing_kind', 'coriolis_approx', 'tracer_nan_guard',
                                          'damping_additive', 'mask_psi_bs', 'tracer_flux',
                                          'frozen_flow')] + \
               [(n, C.c_double) for n in ('dt', 'G', 'Ah', 'A', 'OMEGA', 'RHO0', 'lbc', 'theta0', 'lon_s',
                                          'lon_e', 'lat_s', 'lat_e', 'H_overwrite', 'ab_chi', 'minD',
                                          'tau_scale', 'bih')]


def build():
    subprocess.run(['make', '-s', '-C', HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P, D, I, V = C.c_void_p, C.c_double, C.c_int, None
        sig = {
            'orc_create': (P, [P, P, P]), 'orc_destroy': (V, [P]),
            'orc_field': (P, [P, I]), 'orc_lat': (P, [P, I]), 'orc_ocean': (P, [P, I]),
            'orc_get_scalars': (V, [P, P, P]), 'orc_set_itt': (V, [P, C.c_int64]),
            'orc_set_psi_bs': (V, [P, P]), 'orc_timestep_init': (V, [P]),
            'orc_damping_add': (V, [P, I, I, D, D, D, I, P]), 'orc_damping_finalize': (V, [P]),
            'orc_forcing_add_stream': (I, [P, I, I, D, I, P, P]), 'orc_forcing_set_data': (V, [P, I, P, P]),
            'orc_forcing_init': (V, [P]), 'orc_forcing_update': (V, [P]),
            'orc_initial_conditions': (V, [P, P, P, P]), 'orc_swm_timestep': (V, [P]),
            'orc_swm_advance': (V, [P]), 'orc_model_advance': (V, [P]), 'orc_run': (V, [P, C.c_int64]),
            'orc_streamfunction': (V, [P, P, P, P]), 'orc_divergence': (V, [P, P, P, P]),
            'orc_tracer_add': (I, [P, D, D, D, P, P, P, P]), 'orc_tracer_init': (V, [P]),
            'orc_tracer_field': (P, [P, I, I]), 'orc_tracer_timestep': (V, [P]),
            'orc_tracer_advance': (V, [P]), 'orc_tracer_coeff': (P, [P]),
            'orc_sor_init': (V, [P]), 'orc_sor_solve': (I, [P, P, P, D, I, P]), 'orc_sor_coeff': (P, [P]),
            'orc_helmholtz_sor': (I, [I, I, P, P, P, P, P, P, D, D, I, P]),
            'orc_helmholtz_apply': (V, [I, I, P, P, P, P, P, P]),
            'orc_helmholtz_coeffs': (V, [I, I, P, D, D, D, P, P, P]),
            'orc_nondivergent_from_chi': (V, [P, P, P, P, P, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def make_config(cfg):
    c = Config()
    for name, _ in Config._fields_:
        setattr(c, name, cfg.get(name, 0))
    return c


class OracleBackend:
    """Driver backend running the CPU oracle."""

    def __init__(self, tracer_nan_guard=False):
        self.L = lib()
        self.m = None
        self.nan_guard = tracer_nan_guard
        self._keep = []

    def __del__(self):
        if self.m and self.L:
            self.L.orc_destroy(self.m)

    def setup_domain(self, case):
        cfg = dict(case['config'])
        if self.nan_guard:
            cfg['tracer_nan_guard'] = 1
        self.cfg = cfg
        self.nx, self.ny = cfg['nx'], cfg['ny']
        self._c = make_config(cfg)
        H = f64(case.get('H'))
        miss = None if case.get('H_missing') is None else np.ascontiguousarray(case['H_missing'], np.int8)
        self.m = self.L.orc_create(C.byref(self._c), ptr(H), ptr(miss))

    def timestep_init(self, psi_bs):
        if psi_bs is not None:
            p = f64(psi_bs)
            self.L.orc_set_psi_bs(self.m, ptr(p))
        self.L.orc_timestep_init(self.m)

    def add_damping(self, d):
        fd = f64(d['file_data'])
        self.L.orc_damping_add(self.m, d['term'], d['type'], d['value'], d['sl_length'],
                               d['sl_cutoff'], d['loc'], ptr(fd))

    def finish_damping(self):
        self.L.orc_damping_finalize(self.m)

    def add_stream(self, s, is_const, d1, d2):
        a, b = f64(d1), f64(d2)
        return self.L.orc_forcing_add_stream(self.m, s['type'], s['comp'], s['omega'], int(is_const),
                                             ptr(a), ptr(b))

    def set_stream_data(self, sid, d1, d2):
        a, b = f64(d1), f64(d2)
        self.L.orc_forcing_set_data(self.m, sid, ptr(a), ptr(b))

    def forcing_init(self):
        self.L.orc_forcing_init(self.m)

    def initial_conditions(self, eta, u, v):
        e, uu, vv = f64(eta), f64(u), f64(v)
        self.L.orc_initial_conditions(self.m, ptr(e), ptr(uu), ptr(vv))

    def add_tracer(self, t):
        arrs = [f64(t.get('field_C')), f64(t.get('field_C0')), f64(t.get('field_gamma_C')), f64(t.get('field_cons'))]
        return self.L.orc_tracer_add(self.m, t['kappa_h'], t['cons'], t['gamma_c'], *[ptr(a) for a in arrs])

    def tracer_init(self):
        self.L.orc_tracer_init(self.m)

    def step(self, itt):
        self.L.orc_set_itt(self.m, itt)
        self.L.orc_swm_timestep(self.m)
        self.L.orc_tracer_timestep(self.m)

    def advance(self, itt):
        self.L.orc_model_advance(self.m)

    def run_steady(self, nsteps):
        self.L.orc_run(self.m, nsteps)

    def _view(self, p, count=None):
        n = self.nx * self.ny if count is None else count
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_double)), shape=(n,))

    def field(self, name):
        return self._view(self.L.orc_field(self.m, FIELD_ID[name])).reshape(self.ny, self.nx).copy()

    def set_field(self, name, arr):
        self._view(self.L.orc_field(self.m, FIELD_ID[name]))[:] = np.ascontiguousarray(arr, np.float64).ravel()

    def lat(self, name):
        return self._view(self.L.orc_lat(self.m, LATS.index(name)), self.ny).copy()

    def ocean(self, g):
        p = self.L.orc_ocean(self.m, 'Huve'.index(g[0]) if g != 'eta' else 3)
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_int8)), shape=(self.nx * self.ny,)).reshape(self.ny, self.nx).copy()

    def scalars(self):
        a, b = C.c_double(), C.c_double()
        self.L.orc_get_scalars(self.m, C.byref(a), C.byref(b))
        return a.value, b.value

    def tracer_field(self, t, name):
        return self._view(self.L.orc_tracer_field(self.m, t, TRC_FIELDS.index(name))).reshape(self.ny, self.nx).copy()

    def streamfunction(self, u=None, v=None):
        uu = f64(self.field('tot_u') if u is None else u)
        vv = f64(self.field('tot_v') if v is None else v)
        out = np.zeros((self.ny, self.nx))
        self.L.orc_streamfunction(self.m, ptr(uu), ptr(vv), ptr(out))
        return out

    def divergence(self, u, v):
        uu, vv = f64(u), f64(v)
        out = np.zeros((self.ny, self.nx))
        self.L.orc_divergence(self.m, ptr(uu), ptr(vv), ptr(out))
        return out

    def nondivergent(self, u, v, chi0, first_guess, eps=1e-4):
        """computeNonDivergentFlowField: divergence, SOR for chi from chi0,
        gradient subtracted; returns (u_nd, v_nd, chi, iterations)."""
        div = self.divergence(u, v)
        chi, it, _ = self.sor_solve(div, chi0, eps, first_guess)
        uu, vv, cc = f64(u), f64(v), f64(chi)
        und, vnd = np.zeros_like(uu), np.zeros_like(vv)
        self.L.orc_nondivergent_from_chi(self.m, ptr(cc), ptr(uu), ptr(vv), ptr(und), ptr(vnd))
        return und, vnd, chi, it

    def sor_init(self):
        self.L.orc_sor_init(self.m)

    def sor_solve(self, B, chi, eps, first_guess):
        b = f64(B)
        x = np.ascontiguousarray(chi, np.float64).copy()
        an = C.c_double()
        it = self.L.orc_sor_solve(self.m, ptr(b), ptr(x), eps, int(first_guess), C.byref(an))
        return x, it, an.value

    def sor_coeff(self):
        n = self.nx * self.ny
        return self._view(self.L.orc_sor_coeff(self.m), 5 * n).reshape(5, self.ny, self.nx).copy()


def helmholtz_sor(cx, cy, cc, mask, rhs, psi0, omega, rtol, max_sweeps):
    L = lib()
    ny, nx = rhs.shape
    psi = np.ascontiguousarray(psi0, np.float64).copy()
    a = [f64(cx), f64(cy), f64(cc)]
    m = np.ascontiguousarray(mask, np.int8)
    r = f64(rhs)
    rel = C.c_double()
    it = L.orc_helmholtz_sor(nx, ny, ptr(a[0]), ptr(a[1]), ptr(a[2]), ptr(m), ptr(r), ptr(psi), omega, rtol,
                             max_sweeps, C.byref(rel))
    return psi, it, rel.value


def helmholtz_coeffs(hinv, lam, dx, dy):
    """cx, cy, cc of div(hinv grad psi) - lam psi (orc_helmholtz_coeffs)."""
    L = lib()
    ny, nx = hinv.shape
    h = f64(hinv)
    cx, cy, cc = np.zeros_like(h), np.zeros_like(h), np.zeros_like(h)
    L.orc_helmholtz_coeffs(nx, ny, ptr(h), lam, dx, dy, ptr(cx), ptr(cy), ptr(cc))
    return cx, cy, cc


def helmholtz_apply(cx, cy, cc, mask, psi):
    L = lib()
    ny, nx = psi.shape
    a = [f64(cx), f64(cy), f64(cc)]
    m = np.ascontiguousarray(mask, np.int8)
    p = f64(psi)
    out = np.zeros_like(p)
    L.orc_helmholtz_apply(nx, ny, ptr(a[0]), ptr(a[1]), ptr(a[2]), ptr(m), ptr(p), ptr(out))
    return out
