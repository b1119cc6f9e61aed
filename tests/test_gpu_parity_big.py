"""GPU: parity at the benchmark sizes, against fixtures made by the reference.

tests/golden/big_triclinic50000.npz (50,000-atom triclinic MM3 + EI + Ewald,
22.9 M list rows, 34,890 k-vectors) and big_water24000.npz (24,000-atom
flexible water with exclusions and valence) hold the reference's own
ForceField.compute results for a rebuild step and a skin-path step
(tests/golden/make_golden.py).  Checks, for the plain FP64 form and both
mixed forms:

* the pair set (a, b, r0, r1, r2) equals the reference's (row count and the
  SHA-256 of the sorted keys);
* energy: FP64 within 1e-10, mixed within 1e-6 relative to the total energy,
  and every part within the same bound relative to the largest part;
* gradient and virial: FP64 within 1e-9, mixed within 1e-5 relative RMS,
  per part and in total.
"""
import hashlib
import os

import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

TOL = {'fp64': (1e-10, 1e-9), 'mixed': (1e-6, 1e-5), 'mixed_kahan': (1e-6, 1e-5)}
BIG = ['triclinic50000', 'water24000']


def sorted_pair_digest(rows, natom):
    """SHA-256 of the (a, b, r0, r1, r2) keys in lexicographic order, as the
    fixture stores it; one int64 sort key instead of a five-key lexsort."""
    a = rows['a'].astype(np.int64)
    b = rows['b'].astype(np.int64)
    r = np.stack([rows['r0'], rows['r1'], rows['r2']], 1).astype(np.int64)
    rm = int(np.abs(r).max()) if len(r) else 0
    w = 2 * rm + 1
    key = a * natom + b
    for k in range(3):
        key = key * w + (r[:, k] + rm)
    order = np.argsort(key, kind='stable')
    keys = np.empty((len(a), 5), np.int64)
    keys[:, 0] = a[order]
    keys[:, 1] = b[order]
    keys[:, 2:] = r[order]
    return hashlib.sha256(np.ascontiguousarray(keys, dtype='<i8').tobytes()).hexdigest()


def load_big(name):
    path = os.path.join(gc.GOLDEN, 'big_%s.npz' % name)
    spec, data = gc.load_path(path)
    return spec, data


@pytest.mark.parametrize('precision', ['fp64', 'mixed', 'mixed_kahan'])
@pytest.mark.parametrize('name', BIG)
def test_big_case(name, precision):
    import yaff_gb300
    spec, data = load_big(name)
    natom = len(spec['pos'])
    ff = yaff_gb300.build_forcefield(spec, precision=precision)
    etol, gtol = TOL[precision]
    for s in range(int(data['nsteps'])):
        pos = spec['pos'] if s == 0 else data['step%d_pos' % s]
        ff.update_pos(pos)
        gpos = np.zeros((natom, 3))
        vtens = np.zeros((3, 3))
        e = ff.compute(gpos, vtens)
        assert ff.nlist.nneigh == int(data['step%d_nneigh' % s])
        if s == 0:
            assert sorted_pair_digest(ff.nlist.neighs, natom) == str(data['step0_pairs_sha256']), 'pair set differs'
        e_ref = float(data['step%d_energy' % s])
        assert abs(e - e_ref) <= etol * abs(e_ref), (s, e, e_ref)
        names = [str(x) for x in data['step%d_parts' % s]]
        pe = data['step%d_part_energy' % s]
        scale = abs(pe).max()
        for k, nm in enumerate(names):
            part = getattr(ff, 'part_' + nm)
            assert abs(part.energy - pe[k]) <= etol * scale, (s, nm, part.energy, pe[k])
            gref = data['step%d_part_gpos32' % s][k].astype(np.float64)
            if abs(gref).max() > 0:
                # the fixture's per-part gradients are FP32 copies (7 digits)
                assert gc.rel_rms(part.gpos, gref) <= max(gtol, 1e-6), (s, nm)
            vref = data['step%d_part_vtens' % s][k]
            if abs(vref).max() > 0:
                assert gc.rel_rms(part.vtens, vref) <= gtol, (s, nm)
        assert gc.rel_rms(gpos, data['step%d_gpos' % s]) <= gtol
        assert gc.rel_rms(vtens, data['step%d_vtens' % s]) <= gtol
