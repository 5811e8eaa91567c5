"""Save/load a case description (host.case.load_case output) as a single
.npz file without pickling: scalars and specs as JSON, arrays as entries."""
import json
import numpy as np

_ARRAY_KEYS = ('H', 'H_missing', 'psi_bs')


def save_case(path, case, extra_arrays=None):
    arrays, meta = {}, {'config': case['config'], 'damping': [], 'streams': [], 'tracers': [],
                        'diag': case.get('diag', []), 'ic': [], 'extra': []}
    for k in _ARRAY_KEYS:
        if case.get(k) is not None:
            arrays[k] = np.asarray(case[k])
    for q, d in enumerate(case['damping']):
        m = {k: v for k, v in d.items() if k != 'file_data'}
        if d['file_data'] is not None:
            arrays['damp%d' % q] = d['file_data']
            m['file'] = 'damp%d' % q
        meta['damping'].append(m)
    for q, s in enumerate(case['streams']):
        m = {k: v for k, v in s.items() if k not in ('rec1', 'rec2')}
        arrays['s%d_rec1' % q] = s['rec1']
        if s['rec2'] is not None:
            arrays['s%d_rec2' % q] = s['rec2']
        meta['streams'].append(m)
    for k, v in case['ic'].items():
        arrays['ic_' + k] = v
        meta['ic'].append(k)
    for q, t in enumerate(case.get('tracers', [])):
        m = {}
        for k, v in t.items():
            if k.startswith('field_'):
                if v is not None:
                    arrays['t%d_%s' % (q, k)] = v
                    m[k] = 't%d_%s' % (q, k)
            else:
                m[k] = v
        meta['tracers'].append(m)
    for k, v in (extra_arrays or {}).items():
        arrays['x_' + k] = np.asarray(v)
        meta['extra'].append(k)
    np.savez_compressed(path, meta=np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8), **arrays)


def load_case(path):
    z = np.load(path)
    meta = json.loads(bytes(z['meta']).decode())
    case = {'config': meta['config'], 'diag': meta['diag']}
    for k in _ARRAY_KEYS:
        case[k] = z[k] if k in z.files else None
    case['damping'] = []
    for m in meta['damping']:
        d = dict(m)
        d['file_data'] = z[m['file']] if 'file' in m else None
        d.pop('file', None)
        case['damping'].append(d)
    case['streams'] = []
    for q, m in enumerate(meta['streams']):
        s = dict(m)
        s['rec1'] = z['s%d_rec1' % q]
        s['rec2'] = z['s%d_rec2' % q] if ('s%d_rec2' % q) in z.files else None
        case['streams'].append(s)
    case['ic'] = {k: z['ic_' + k] for k in meta['ic']}
    case['tracers'] = []
    for m in meta['tracers']:
        t = {k: v for k, v in m.items() if not k.startswith('field_')}
        for fld in ('field_C', 'field_C0', 'field_gamma_C', 'field_cons'):
            t[fld] = z[m[fld]] if fld in m else None
        case['tracers'].append(t)
    extra = {k: z['x_' + k] for k in meta['extra']}
    return case, extra
