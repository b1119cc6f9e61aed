"""Loads the golden fixtures of tests/golden/ (made by make_golden.py from
the reference itself) back into configs.py specs."""
import glob
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, 'golden')


def case_names():
    """Force-field cases (the mc_* fixtures hold MC trial cases, md_* MD
    trajectories, big_* compact fixtures of the benchmark-sized systems)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, '*.npz'))
                  if not os.path.basename(p).startswith(('mc_', 'md_', 'big_')))


def mc_case_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, 'mc_*.npz')))


def load_mc(name):
    """(case, data) of an MC trial fixture: case in the layout of
    configs.mc_workload, data the raw arrays (chain, trials, reference
    energies, prefactor and structure-factor arrays)."""
    d = dict(np.load(os.path.join(GOLDEN, name + '.npz'), allow_pickle=False))
    case = {'framework': {'pos': d['frame_pos'], 'charges': d['frame_charges'], 'sigmas': d['frame_sigmas'],
                          'epsilons': d['frame_epsilons'], 'rvecs': d['rvecs']},
            'guest': {'pos': d['guest_pos'], 'charges': d['guest_charges'], 'sigmas': d['guest_sigmas'],
                      'epsilons': d['guest_epsilons']},
            'rcut': float(d['rcut']), 'alpha': float(d['alpha']), 'gcut': float(d['gcut']),
            'close_contact': float(d['close_contact'])}
    return case, d


def load(name):
    """(spec, data) for a golden case."""
    return load_path(os.path.join(GOLDEN, name + '.npz'))


def load_path(path):
    """(spec, data) for the force-field fixture at `path`."""
    data = dict(np.load(path, allow_pickle=False))
    spec = {'pair': [], 'ewald': None, 'tr': None, 'charges': None, 'bonds': None}
    i = 0
    while 'pair%d_kind' % i in data:
        p = {'kind': str(data['pair%d_kind' % i])}
        for k in list(data):
            pre = 'pair%d_' % i
            if k.startswith(pre) and k != pre + 'kind':
                p[k[len(pre):]] = data[k]
        spec['pair'].append(p)
        i += 1
    for k, v in data.items():
        if k.startswith('spec_'):
            key = k[5:]
            if v.ndim == 0:
                v = v.item()
            spec[key] = v
    if 'ewald_alpha' in data:
        spec['ewald'] = {'alpha': float(data['ewald_alpha']), 'gcut': float(data['ewald_gcut'])}
    if 'tr_kind' in data:
        spec['tr'] = (str(data['tr_kind']), float(data['tr_par']))
    spec['scalings'] = tuple(float(x) for x in spec['scalings'])
    spec['name'] = str(spec['name'])
    spec['nlow'] = int(spec.get('nlow', 0))
    spec['nhigh'] = int(spec.get('nhigh', -1))
    return spec, data


def pair_keys_from_rows(rows):
    keys = np.stack([rows['a'], rows['b'], rows['r0'], rows['r1'], rows['r2']], 1).astype(np.int64)
    order = np.lexsort(keys.T[::-1])
    vals = np.stack([rows['d'], rows['dx'], rows['dy'], rows['dz']], 1)[order]
    return keys[order], vals


def rel_rms(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    den = np.sqrt((b ** 2).mean())
    if den == 0:
        return np.sqrt((a ** 2).mean())
    return np.sqrt(((a - b) ** 2).mean()) / den
