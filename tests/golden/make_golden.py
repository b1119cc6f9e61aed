"""Generate the golden fixtures in tests/golden/ by running the reference.

Run in a container that holds the reference checkout, after
``sh oracle/build_ref.sh`` has built its extension (the checkout is
$YAFF_REFERENCE, else the one the recipe built from):

    python tests/golden/make_golden.py [case ...]
    python tests/golden/make_golden.py big_triclinic50000 big_water24000

For every case the script builds the reference's own ForceField (through the
import shim in oracle/ref_shim.py), calls ForceField.compute(gpos, vtens) one
or more times (rebuild and skin paths), and stores the inputs (the spec) and
the reference outputs: per-part energies, gradients and virials, and the
neighbour list (full rows for small cases, a SHA-256 of the sorted pair keys
for large ones).  Cases 'water32' and 'quartz' use the geometries of the
reference's own test fixtures (yaff/test/common.py), read from the reference
checkout at generation time.
"""
import hashlib
import os
import sys
import warnings

import numpy as np

warnings.filterwarnings('ignore')
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, 'oracle'))

from yaff_gb300 import configs  # noqa: E402
from yaff_gb300.units import angstrom, kjmol  # noqa: E402
import ref_shim  # noqa: E402
from ref_ff import build_reference_ff  # noqa: E402


def pair_keys(nl):
    nb = nl.neighs[:nl.nneigh]
    keys = np.stack([nb['a'], nb['b'], nb['r0'], nb['r1'], nb['r2']], 1).astype(np.int64)
    order = np.lexsort(keys.T[::-1])
    vals = np.stack([nb['d'], nb['dx'], nb['dy'], nb['dz']], 1)[order]
    return keys[order], vals


def keys_digest(keys):
    return hashlib.sha256(np.ascontiguousarray(keys, dtype='<i8').tobytes()).hexdigest()


def spec_arrays(spec):
    out = {}
    for k, v in spec.items():
        if k == 'pair':
            for i, p in enumerate(v):
                out['pair%d_kind' % i] = np.array(p['kind'])
                for kk, vv in p.items():
                    if kk != 'kind':
                        out['pair%d_%s' % (i, kk)] = np.asarray(vv)
        elif k == 'ewald':
            if v is not None:
                out['ewald_alpha'] = np.array(v['alpha'])
                out['ewald_gcut'] = np.array(v['gcut'])
        elif k == 'tr':
            if v is not None:
                out['tr_kind'] = np.array(v[0])
                out['tr_par'] = np.array(v[1])
        elif v is None:
            continue
        else:
            out['spec_' + k] = np.asarray(v)
    return out


ONLY = set()   # case names given on the command line: regenerate only those


def run_case(name, spec, displacements=(), full_rows=True):
    if ONLY and name not in ONLY:
        return
    ff = build_reference_ff(spec)
    natom = len(spec['pos'])
    data = spec_arrays(spec)
    data['case'] = np.array(name)
    data['nsteps'] = np.array(1 + len(displacements))
    pos = spec['pos'].copy()
    steps = [np.zeros_like(pos)] + list(displacements)
    for s, dpos in enumerate(steps):
        pos = pos + dpos
        ff.update_pos(pos)
        gpos = np.zeros((natom, 3))
        vtens = np.zeros((3, 3))
        e = ff.compute(gpos, vtens)
        data['step%d_pos' % s] = pos.copy()
        data['step%d_energy' % s] = np.array(e)
        data['step%d_gpos' % s] = gpos
        data['step%d_vtens' % s] = vtens
        data['step%d_parts' % s] = np.array([p.name for p in ff.parts])
        data['step%d_part_energy' % s] = np.array([p.energy for p in ff.parts])
        data['step%d_part_gpos' % s] = np.array([p.gpos for p in ff.parts])
        data['step%d_part_vtens' % s] = np.array([p.vtens for p in ff.parts])
        for p in ff.parts:
            if p.name.startswith('tailcorr_'):
                data['%s_ecorr' % p.name] = np.array(p.ecorr)
                data['%s_wcorr' % p.name] = np.array(p.wcorr)
        keys, vals = pair_keys(ff.nlist)
        data['step%d_nneigh' % s] = np.array(ff.nlist.nneigh)
        data['step%d_pairs_sha256' % s] = np.array(keys_digest(keys))
        if full_rows and s == 0:
            data['step%d_pair_keys' % s] = keys.astype(np.int32)
            data['step%d_pair_vals' % s] = vals
    data['rmax'] = np.asarray(ff.nlist.rmax)
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **data)
    print('%-14s natom %6d  nneigh %8d  E %.12e  rmax %s' % (
        name, natom, ff.nlist.nneigh, data['step0_energy'], ff.nlist.rmax))


def run_big_case(name, spec, displacements=()):
    """Compact fixture of a benchmark-sized system (file big_<name>.npz):
    positions, total energy / gradient / virial in FP64, per-part energies
    and virials in FP64, per-part gradients in FP32 (ample for the 1e-5
    relative RMS checks), and the neighbour list as its row count and the
    SHA-256 of the sorted pair keys.  Step 0 rebuilds the list; the later
    steps displace the atoms by less than half the skin, so the reference
    takes its skin (recompute) path."""
    if ONLY and ('big_' + name) not in ONLY:
        return
    ff = build_reference_ff(spec)
    natom = len(spec['pos'])
    data = spec_arrays(spec)
    data['case'] = np.array(name)
    data['nsteps'] = np.array(1 + len(displacements))
    pos = spec['pos'].copy()
    steps = [np.zeros_like(pos)] + list(displacements)
    for s, dpos in enumerate(steps):
        pos = pos + dpos
        ff.update_pos(pos)
        gpos = np.zeros((natom, 3))
        vtens = np.zeros((3, 3))
        e = ff.compute(gpos, vtens)
        if s > 0:
            data['step%d_pos' % s] = pos.copy()
        data['step%d_energy' % s] = np.array(e)
        data['step%d_gpos' % s] = gpos
        data['step%d_vtens' % s] = vtens
        data['step%d_parts' % s] = np.array([p.name for p in ff.parts])
        data['step%d_part_energy' % s] = np.array([p.energy for p in ff.parts])
        data['step%d_part_gpos32' % s] = np.array([p.gpos for p in ff.parts], dtype=np.float32)
        data['step%d_part_vtens' % s] = np.array([p.vtens for p in ff.parts])
        keys, _ = pair_keys(ff.nlist)
        data['step%d_nneigh' % s] = np.array(ff.nlist.nneigh)
        data['step%d_pairs_sha256' % s] = np.array(keys_digest(keys))
        data['step%d_rebuilt' % s] = np.array(s == 0)
        print('  %s step %d: E %.12e nneigh %d' % (name, s, e, ff.nlist.nneigh), flush=True)
    data['rmax'] = np.asarray(ff.nlist.rmax)
    np.savez_compressed(os.path.join(HERE, 'big_' + name + '.npz'), **data)
    print('%-14s natom %6d  nneigh %8d  E %.12e  rmax %s' % (
        name, natom, ff.nlist.nneigh, data['step0_energy'], ff.nlist.rmax))


def fixture_system(getter):
    ref_shim.import_reference()
    import importlib.util
    path = os.path.join(ref_shim.REF_ROOT, 'yaff', 'test', 'common.py')
    src = open(path).read()
    # the fixture module imports molmod/yaff wholesale; only the data getters
    # are needed, so evaluate it with the shimmed packages in place.
    mod = importlib.util.module_from_spec(importlib.util.spec_from_loader('ref_fixtures', loader=None))
    import yaff.system
    mod.__dict__.update({'np': np, 'System': _FixtureSystem, 'angstrom': angstrom})
    code = '\n'.join(l for l in src.splitlines()
                     if not l.startswith(('import ', 'from ')))
    exec(compile(code, path, 'exec'), mod.__dict__)
    return getattr(mod, getter)()


class _FixtureSystem(object):
    def __init__(self, **kw):
        self.kw = kw


def water32_spec():
    s = fixture_system('get_system_water32').kw
    pos = np.asarray(s['pos'], float)
    n = len(pos)
    spec = configs._base_spec('water32', pos, np.asarray(s['rvecs'], float))
    iso = np.array(s['numbers']) == 8
    spec['charges'] = np.asarray(s['charges'], float)
    spec['masses'] = np.where(iso, configs.MASS_O, configs.MASS_H)
    spec['bonds'] = np.asarray(s['bonds'], np.int64)
    spec['pair'] = [{'kind': 'lj', 'sigmas': np.where(iso, 3.15 * angstrom, 0.4 * angstrom),
                     'epsilons': np.where(iso, 0.64 * kjmol, 0.19 * kjmol)}, {'kind': 'ei'}]
    spec['rcut'] = 9.0 * angstrom
    spec['skin'] = 2.0 * angstrom
    spec['tr'] = ('switch3', 3.0 * angstrom)
    spec['scalings'] = (0.0, 0.5, 1.0, 1.0)
    spec['ewald'] = configs.ewald_params(spec['rcut'])
    o = np.arange(0, n, 3)
    spec['bond_terms'] = np.column_stack([spec['bonds'].astype(float), np.full(len(spec['bonds']), 4000 * kjmol / angstrom ** 2),
                                          np.full(len(spec['bonds']), 0.96 * angstrom)])
    spec['bend_terms'] = np.column_stack([(o + 1).astype(float), o.astype(float), (o + 2).astype(float),
                                          np.full(len(o), 300 * kjmol), np.full(len(o), 1.82)])
    return spec


def quartz_spec():
    s = fixture_system('get_system_quartz').kw
    pos = np.asarray(s['pos'], float)
    spec = configs._base_spec('quartz', pos, np.asarray(s['rvecs'], float))
    issi = np.array(s['numbers']) == 14
    spec['charges'] = np.asarray(s['charges'], float)
    spec['pair'] = [{'kind': 'mm3', 'sigmas': np.where(issi, 2.29, 1.82) * angstrom,
                     'epsilons': np.where(issi, 0.59, 0.25) * kjmol,
                     'onlypaulis': np.where(issi, 0, 1).astype(np.int32)}, {'kind': 'ei'}]
    spec['rcut'] = 8.0 * angstrom
    spec['skin'] = 0.0
    spec['tr'] = ('hammer', 0.5 * angstrom)
    spec['ewald'] = configs.ewald_params(spec['rcut'], 3.0, 1.3)
    return spec


def main():
    if not ref_shim.reference_available():
        raise SystemExit('reference not available: run oracle/build_ref.sh first')
    rng = np.random.default_rng(1234)

    lat = configs.lattice_lj_ei(nside=6, spacing=2.5, rcut=6.0, name='lat216')
    run_case('lat216', lat)

    w = configs.flexible_water(nside=4, box=12.42, rcut=5.0, skin=0.5, name='water64')
    n = len(w['pos'])
    small = rng.uniform(-0.02, 0.02, (n, 3)) * angstrom   # stays on the skin path
    large = rng.uniform(-0.6, 0.6, (n, 3)) * angstrom     # forces a rebuild
    run_case('water64', w, displacements=[small, small, large])

    t = configs.triclinic_mm3_ei(natom=600, rcut=6.0, skin=0.5, name='tric600')
    run_case('tric600', t, displacements=[rng.uniform(-0.05, 0.05, (600, 3)) * angstrom])

    ti = configs.triclinic_mm3_ei(natom=100, rcut=7.0, skin=0.3, name='tric100img')
    run_case('tric100img', ti)

    run_case('water32', water32_spec(), displacements=[rng.uniform(-0.05, 0.05, (96, 3)) * angstrom])
    run_case('quartz', quartz_spec())

    mc = configs.lattice_lj_ei(nside=6, spacing=2.5, rcut=6.0, name='lat216split')
    mc['nlow'] = 100
    mc['nhigh'] = 100
    run_case('lat216split', mc)

    big = configs.lattice_lj_ei(name='lattice1000')
    run_case('lattice1000', big, full_rows=False)

    t2 = configs.triclinic_mm3_ei(natom=2000, name='tric2000')
    run_case('tric2000', t2, full_rows=False)

    v = configs.valence_molecules(name='valence40')
    run_case('valence40', v, displacements=[rng.uniform(-0.08, 0.08, (40, 3)) * angstrom,
                                            rng.uniform(-0.08, 0.08, (40, 3)) * angstrom])

    for var in 'abc':
        pp = configs.pair_potentials(var)
        run_case(pp['name'], pp, displacements=[rng.uniform(-0.05, 0.05, (300, 3)) * angstrom])

    for var in ('a', 'b', 'c', 'lj', 'mm3'):
        tc = configs.tail_corrections(var)
        run_case(tc['name'], tc)

    # Gaussian charges (radii > 0) in both branches of the reference's EI
    # term (yaff/pes/pair_pot.c:724-748): screened by Ewald, and alone
    for name, ewald in (('gauss216', True), ('gauss216bare', False)):
        gs = configs.lattice_lj_ei(nside=6, spacing=2.5, rcut=6.0, name=name)
        gs['pair'][1]['radii'] = np.where(np.arange(216) % 2 == 0, 0.9, 1.2) * angstrom
        if not ewald:
            gs['ewald'] = None
        run_case(name, gs, displacements=[rng.uniform(-0.05, 0.05, (216, 3)) * angstrom])

    # benchmark-sized systems (minutes of reference CPU time each): only when
    # named on the command line, e.g. big_triclinic50000 big_water24000
    brng = np.random.default_rng(4321)
    if 'big_triclinic50000' in ONLY:
        t5 = configs.triclinic_50000()
        run_big_case('triclinic50000', t5, displacements=[brng.uniform(-0.05, 0.05, (50000, 3)) * angstrom])
    if 'big_water24000' in ONLY:
        w24 = configs.water_24000()
        run_big_case('water24000', w24, displacements=[brng.uniform(-0.05, 0.05, (24000, 3)) * angstrom])


if __name__ == '__main__':
    ONLY.update(sys.argv[1:])
    main()
