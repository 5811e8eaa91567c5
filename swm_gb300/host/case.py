"""Turns a reference run directory (model.h + model.namelist + input/) into a
self-contained case description: resolved configuration scalars, input
fields, damping entries, forcing streams and diagnostic tasks.

Defaults follow the Fortran declarations they replace:
  &model_nl   vars_module.f90:27-36, 121-138
  &domain_nl  domain_module.f90:11-44, 59-64
  &tint_nl    time_integration_module.f90:20, 36
  &swm_damping_nl   swm_damping_module.f90:143-156, 209-229
  &swm_forcing_nl   swm_forcing_module.f90:83-121
  &trc_tracer_nl    tracer_vars.f90:71-113
  &diag_nl    diagTask.f90:180-222 with include/diag_module.h defaults
Default-real literals in the Fortran (G, OMEGA, TAU_SCALE, ...) are rounded
to binary32 before use, as the Fortran compiler does.
"""
import os
import re
import numpy as np

from . import namelist as nl
from .modelh import parse_defines
from . import ncio
from .memchunk import MemChunk

MODE_NONE, MODE_NONLINEAR, MODE_LIN_REST, MODE_LIN_MEAN = 0, 1, 2, 3
F32 = lambda x: float(np.float32(x))

TERMS = {'GAMMA_LIN_U': 0, 'GAMMA_LIN_V': 1, 'GAMMA_LIN_ETA': 2, 'GAMMA_SQ_U': 3, 'GAMMA_SQ_V': 4}
DAMP_TYPES = {'uniform': 0, 'sponge': 1, 'file': 2}
FRC_TYPES = {'W': 0, 'O': 1, 'C': 2, 'H': 3, 'E': 4}


def _cpp_real(txt):
    """Value of a CPP-substituted Fortran real literal (binary32 unless it
    carries a d exponent or a kind suffix)."""
    t = txt.strip()
    if re.search(r'[dD]', t) or '_' in t:
        return float(t.replace('d', 'e').replace('D', 'e').split('_')[0])
    return F32(float(t))


def sponge_flags(loc):
    f = 0
    for ch, bit in (('N', 1), ('S', 2), ('W', 4), ('E', 8)):
        if ch in loc.upper():
            f |= bit
    return f


def component_code(ftype, comp):
    c = comp[:1].upper()
    if ftype == 'E':
        return {'U': 3, 'V': 4, 'R': 5}[c]
    return {'Z': 0, 'M': 1, 'C': 2}.get(c, 2)


def load_case(run_dir):
    """Parse a run directory into a case dict (arrays are float64, row-major
    (Ny, Nx), i.e. Fortran (Nx, Ny) memory order)."""
    with open(os.path.join(run_dir, 'model.h')) as fh:
        defs = parse_defines(fh.read())
    with open(os.path.join(run_dir, 'model.namelist')) as fh:
        groups = nl.parse(fh.read())
    P = lambda rel: os.path.join(run_dir, rel)

    mnl = nl.group(groups, 'model_nl')
    dnl = nl.group(groups, 'domain_nl')
    tnl = nl.group(groups, 'tint_nl')

    if 'FULLY_NONLINEAR' in defs:
        mode = MODE_NONLINEAR
    elif 'LINEARISED_MEAN_STATE' in defs:
        mode = MODE_LIN_MEAN
    elif 'LINEARISED_STATE_OF_REST' in defs:
        mode = MODE_LIN_REST
    else:
        mode = MODE_NONE

    cfg = dict(
        nx=int(dnl.get('nx', 100)), ny=int(dnl.get('ny', 100)), mode=mode,
        lateral_mixing=int('LATERAL_MIXING' in defs),
        quadratic_friction=int('QUADRATIC_BOTTOM_FRICTION' in defs),
        barotropic=int('BAROTROPIC' in defs),
        mixing_kind=0,
        coriolis_approx=int(dnl.get('coriolis_approx', 3)),
        tracer_nan_guard=0,
        dt=float(mnl.get('dt', 10.0)),
        G=float(mnl['g']) if 'g' in mnl else F32(9.80665),
        Ah=float(mnl.get('ah', 0.0)),
        A=float(dnl.get('a', 6371000.0)),
        OMEGA=float(dnl['omega']) if 'omega' in dnl else F32(7.272205e-5),
        RHO0=float(dnl.get('rho0', 1024.0)),
        # domain_module declares lbc twice; the namelist fills the local one
        # (initDomain :53).  2.0 is the module default used when it is absent.
        lbc=float(dnl.get('lbc', 2.0)),
        theta0=float(dnl.get('theta0', 0.0)),
        lon_s=float(dnl.get('lon_s', -20.0)), lon_e=float(dnl.get('lon_e', 20.0)),
        lat_s=float(dnl.get('lat_s', -20.0)), lat_e=float(dnl.get('lat_e', 20.0)),
        H_overwrite=float(dnl.get('h_overwrite', 0.0)),
        ab_chi=float(tnl.get('ab_chi', 0.1)),
        minD=1.0,
        tau_scale=_cpp_real(defs['TAU_SCALE']) if 'TAU_SCALE' in defs else 1.0,
        bih=0.0,
    )
    run_length = float(mnl.get('run_length', 100000.0))
    cfg['Nt'] = int(run_length / cfg['dt'])
    cfg['diag_start_ind'] = int(float(mnl.get('diag_start', 0.0)) / cfg['dt'])
    cfg['meant_out'] = float(mnl.get('meant_out', 2.628e6))
    cfg['tracer'] = int('TRACER' in defs)

    case = {'config': cfg, 'dir': run_dir}

    # bathymetry
    fh = dnl.get('in_file_h', '')
    if fh:
        H, miss = ncio.read_last(P(fh), dnl.get('in_varname_h', 'H'))
        case['H'], case['H_missing'] = H, miss
    else:
        case['H'], case['H_missing'] = None, None

    # basic state for LINEARISED_MEAN_STATE (SWM_timestep_init :73-85)
    if mode == MODE_LIN_MEAN:
        snl = nl.group(groups, 'swm_timestep_nl')
        data, _, dtf = ncio.read_records(P(snl['filename']), snl['varname'])
        mc = MemChunk(data, dtf, int(snl.get('chunksize', 100)))
        case['psi_bs'] = mc.get(0.0)

    # damping entries, in namelist order
    damping = []
    for d in nl.groups_named(groups, 'swm_damping_nl'):
        term = str(d.get('term', '')).upper()
        if term not in TERMS:
            continue
        typ = str(d.get('type', ''))
        ent = dict(term=TERMS[term], type=DAMP_TYPES[typ], value=float(d.get('value', 0.0)),
                   sl_length=float(d.get('sl_length', 1.0)), sl_cutoff=float(d.get('sl_cutoff', 15.0)),
                   loc=sponge_flags(str(d.get('sl_location', ''))), file_data=None)
        if typ == 'file':
            data, _, dtf = ncio.read_records(P(d['filename']), d['varname'])
            ent['file_data'] = MemChunk(data, dtf, 1).get(0.0)
        damping.append(ent)
    case['damping'] = damping

    # forcing streams, in namelist order (list order is applied by the caller)
    streams = []
    for d in nl.groups_named(groups, 'swm_forcing_nl'):
        fn = d.get('filename', '')
        if not fn:
            continue
        ftype = str(d.get('forcingtype', ''))[:1].upper()
        comp = str(d.get('component', ''))
        cs = int(d.get('chunksize', 100))
        r1, _, dt1 = ncio.read_records(P(fn), d['varname'])
        st = dict(type=FRC_TYPES[ftype], comp=component_code(ftype, comp), omega=float(d.get('omega', 0.0)),
                  rec1=r1, dt1=dt1, chunksize=cs, rec2=None, dt2=0.0)
        fn2, vn2 = d.get('filename2', ''), d.get('varname2', '')
        if fn2 and vn2:
            r2, _, dt2 = ncio.read_records(P(fn2), vn2)
            st['rec2'], st['dt2'] = r2, dt2
        streams.append(st)
    case['streams'] = streams

    # initial conditions (vars_module.f90:114-119, swm_module.f90:156-181)
    ic = {}
    for key, fk, vk, dv in (('eta', 'file_eta_init', 'varname_eta_init', 'ETA'),
                            ('u', 'file_u_init', 'varname_u_init', 'U'),
                            ('v', 'file_v_init', 'varname_v_init', 'V')):
        f = mnl.get(fk, '')
        if f:
            ic[key] = ncio.read_last(P(f), mnl.get(vk, dv))[0]
    case['ic'] = ic

    # tracers
    tracers = []
    for d in nl.groups_named(groups, 'trc_tracer_nl'):
        t = dict(varid=d.get('varid', ''), kappa_h=float(d.get('kappa_h', 0.0)),
                 cons=float(d.get('cons', 0.0)), gamma_c=float(d.get('gamma_c', 0.0)))
        for fld in ('C', 'C0', 'gamma_C', 'cons'):
            fnm, vnm = d.get('filename_' + fld.lower(), ''), d.get('varname_' + fld.lower(), '')
            t['field_' + fld] = ncio.read_last(P(fnm), vnm)[0] if fnm and vnm else None
        tracers.append(t)
    case['tracers'] = tracers

    # diagnostic tasks
    diag = []
    for d in nl.groups_named(groups, 'diag_nl'):
        diag.append(dict(filename=d.get('filename', 'out.nc'), varname=str(d.get('varname', '')),
                         type=str(d.get('type', 'S'))[:1].upper(), frequency=int(d.get('frequency', 1)),
                         period=float(d.get('period', 2.628e6)), process=str(d.get('process', 'A'))[:1].upper()))
    case['diag'] = diag
    return case
