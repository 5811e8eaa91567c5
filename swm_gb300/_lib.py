"""ctypes binding of libswm_gb300.so (include/swm_gpu.h).

The library is built in-tree by swm_gb300.build; loading fails loudly when it
is missing -- there is no CPU fallback.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libswm_gb300.so')

CONFIG_INT = ('nx', 'ny', 'mode', 'lateral_mixing', 'quadratic_friction', 'barotropic', 'mixing_kind',
              'coriolis_approx', 'tracer_nan_guard', 'damping_additive', 'mask_psi_bs', 'tracer_flux',
              'frozen_flow')
CONFIG_DBL = ('dt', 'G', 'Ah', 'A', 'OMEGA', 'RHO0', 'lbc', 'theta0', 'lon_s', 'lon_e', 'lat_s', 'lat_e',
              'H_overwrite', 'ab_chi', 'minD', 'tau_scale', 'bih')


class Config(C.Structure):
    _fields_ = [(n, C.c_int32) for n in CONFIG_INT] + [(n, C.c_double) for n in CONFIG_DBL] + \
               [('path', C.c_int32), ('reserved', C.c_int32)]


FIELDS = ['u', 'v', 'eta', 'D', 'Dh', 'Du', 'Dv', 'edens', 'pot', 'zeta', 'mu', 'mv', 'H', 'H_u', 'H_v',
          'H_eta', 'impl_u', 'impl_v', 'impl_eta', 'gamma_lin_u', 'gamma_lin_v', 'gamma_lin_eta',
          'gamma_sq_u', 'gamma_sq_v', 'F_x', 'F_y', 'F_eta', 'u_bs', 'v_bs', 'zeta_bs', 'latmix_u',
          'latmix_v', 'G_u', 'G_v', 'G_eta', 'psi']
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}
PATHS = {'plain_fp64': 0, 'fused_fp64': 1, 'fused_fp32c': 2}

# exported symbols (every declaration of include/swm_gpu.h)
SIGNATURES = {}
_lib = None


def _sigs():
    P, D, I, I64 = C.c_void_p, C.c_double, C.c_int, C.c_int64
    PP = C.POINTER(C.c_void_p)
    return {
        'swm_gpu_last_error': (C.c_char_p, []),
        'swm_gpu_create': (I, [P, PP]), 'swm_gpu_destroy': (I, [P]), 'swm_gpu_synchronize': (I, [P]),
        'swm_gpu_stream': (P, [P]), 'swm_gpu_launch_count': (I64, [P]), 'swm_gpu_step_shape': (I, [P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int)]),
        'swm_gpu_plan_step_tiles': (I, [I, I, I, P, D, D, P, I]), 'swm_gpu_step_strip_columns': (I, [I]),
        'swm_gpu_domain': (I, [P, P, P]), 'swm_gpu_timestep_init': (I, [P, P]),
        'swm_gpu_add_damping': (I, [P, I, I, D, D, D, I, P]), 'swm_gpu_finish_damping': (I, [P]),
        'swm_gpu_add_stream': (I, [P, I, I, D, I, P, P, C.POINTER(C.c_int)]),
        'swm_gpu_set_stream_data': (I, [P, I, P, P]), 'swm_gpu_forcing_init': (I, [P]),
        'swm_gpu_stream_records': (I, [P, I, I, I, P]),
        'swm_gpu_stream_interp': (I, [P, I, I, I, I, D, D, D]),
        'swm_gpu_set_stream_rows': (I, [P, I, P, P]), 'swm_gpu_integrals': (I, [P, P]),
        'swm_gpu_integrals_noalloc': (I, [P, P]),
        'swm_gpu_integrals_async': (I, [P, P, C.POINTER(C.c_int64)]),
        'swm_gpu_initial_conditions': (I, [P, P, P, P]), 'swm_gpu_step': (I, [P, I64]),
        'swm_gpu_advance': (I, [P, I64]), 'swm_gpu_run': (I, [P, I64, I64]),
        'swm_gpu_run_monitor': (I, [P, I64, I64, I, P, P, P]),
        'swm_gpu_get_field': (I, [P, I, P]), 'swm_gpu_set_field': (I, [P, I, P]),
        'swm_gpu_get_field_async': (I, [P, I, P, C.POINTER(C.c_int64)]), 'swm_gpu_wait': (I, [P, I64]),
        'swm_gpu_ready': (I, [P, I64]),
        'swm_gpu_host_register': (I, [P, I64]), 'swm_gpu_host_unregister': (I, [P]),
        'swm_gpu_get_metric': (I, [P, I, I, P]), 'swm_gpu_get_mask': (I, [P, I, P]),
        'swm_gpu_streamfunction': (I, [P, P]),
        'swm_gpu_diag_accumulate': (I, [P, I, I, I, D]),
        'swm_gpu_diag_mean': (I, [P, I, P, C.POINTER(C.c_double)]),
        'trc_gpu_add': (I, [P, D, D, D, P, P, P, P, C.POINTER(C.c_int)]), 'trc_gpu_init': (I, [P]),
        'trc_gpu_get_field': (I, [P, I, I, P]),
        'swm_gpu_ensemble_create': (I, [P, I, PP]), 'swm_gpu_ensemble_destroy': (I, [P]),
        'swm_gpu_ensemble_run': (I, [P, I64, I64]), 'swm_gpu_ensemble_integrals': (I, [P, P]),
        'swm_gpu_ensemble_run_monitor': (I, [P, I64, I64, P, P]),
        'swm_gpu_ensemble_synchronize': (I, [P]), 'swm_gpu_ensemble_stream': (P, [P]),
        'swm_gpu_ensemble_launch_count': (I64, [P]), 'swm_gpu_ensemble_rows': (I, [P]),
        'swm_helm_create': (I, [I, I, D, D, D, P, P, PP]), 'swm_helm_destroy': (I, [P]),
        'swm_helm_stream': (P, [P]), 'swm_helm_launch_count': (I64, [P]), 'swm_helm_apply': (I, [P, P, P]),
        'swm_helm_solve_fp64': (I, [P, P, P, D, D, I, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
        'swm_helm_solve_mixed': (I, [P, P, P, D, D, D, I, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.POINTER(C.c_double)]),
        'swm_helm_autotune': (I, [P, P, D, D, I, I, C.POINTER(C.c_double), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int)]),
        'swm_gpu_nondivergent': (I, [P, I, D, P, P, P, C.POINTER(C.c_int)]),
        'elsolv_sor_gpu_init': (I, [P]),
        'elsolv_sor_gpu_solve': (I, [P, P, P, D, I, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
        'swm_gpu_check_division': (I, [I64, I64, C.POINTER(C.c_int64)]),
    }


SIGNATURES.update(_sigs())


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError('libswm_gb300.so is not built: run `python -m swm_gb300.build` '
                               '(or __graft_entry__.build()) first')
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class SwmGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__('swm_gpu error %d: %s' % (code, msg))
        self.code = code


def check(rc):
    if rc != 0:
        raise SwmGpuError(rc, lib().swm_gpu_last_error().decode())
    return rc
