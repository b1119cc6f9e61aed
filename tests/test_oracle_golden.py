"""CPU: the oracle port reproduces the reference's golden fixtures exactly
(pair rows bit-identical, energies / gradients / virials to rounding)."""
import hashlib

import numpy as np
import pytest

import golden_cases as gc
from oracle import OracleForceField

CASES = gc.case_names()


def _digest(keys):
    return hashlib.sha256(np.ascontiguousarray(keys, dtype='<i8').tobytes()).hexdigest()


@pytest.mark.parametrize('name', CASES)
def test_oracle_matches_reference(name):
    spec, data = gc.load(name)
    orc = OracleForceField(spec)
    nsteps = int(data['nsteps'])
    for s in range(nsteps):
        orc.update_pos(data['step%d_pos' % s])
        gpos = np.zeros((len(spec['pos']), 3))
        vtens = np.zeros((3, 3))
        e = orc.compute(gpos, vtens)
        keys, rows = orc.pair_set()
        assert orc.nneigh == int(data['step%d_nneigh' % s])
        assert _digest(keys) == str(data['step%d_pairs_sha256' % s])
        if 'step%d_pair_keys' % s in data:
            assert np.array_equal(keys, data['step%d_pair_keys' % s].astype(np.int64))
            vals = np.stack([rows['d'], rows['dx'], rows['dy'], rows['dz']], 1)
            assert np.array_equal(vals, data['step%d_pair_vals' % s])
        names = [str(x) for x in data['step%d_parts' % s]]
        # tail corrections are host scalars of the product, checked against
        # the reference in test_tailcorr.py; the oracle covers the rest
        tail = [k for k, nm in enumerate(names) if nm.startswith('tailcorr_')]
        ref_e = float(data['step%d_energy' % s]) - sum(data['step%d_part_energy' % s][k] for k in tail)
        ref_v = data['step%d_vtens' % s] - sum((data['step%d_part_vtens' % s][k] for k in tail), np.zeros((3, 3)))
        assert abs(e - ref_e) <= 1e-13 * max(1.0, abs(ref_e))
        assert np.allclose(gpos, data['step%d_gpos' % s], rtol=0, atol=1e-13 * max(1, abs(data['step%d_gpos' % s]).max()))
        assert np.allclose(vtens, ref_v, rtol=0, atol=1e-13 * max(1, abs(data['step%d_vtens' % s]).max()))
        for k, nm in enumerate(names):
            if k not in tail:
                assert orc.part_energies[nm] == data['step%d_part_energy' % s][k], nm


def test_fixture_set_complete():
    for want in ('lat216', 'water64', 'tric600', 'tric100img', 'water32', 'quartz', 'lat216split', 'lattice1000',
                 'tric2000'):
        assert want in CASES
