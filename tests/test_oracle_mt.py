"""CPU: the threaded timing form of the oracle (oracle/yaff_oracle_mt.c)
evaluates the same thing as the single-thread oracle: an identical neighbour
list (same rows, same order) and energies, gradients and virials equal up to
the order of the final sums (1e-12 relative)."""
import numpy as np
import pytest

import golden_cases as gc
from oracle import OracleForceField


@pytest.mark.parametrize('name', ['tric2000', 'water64', 'lat216split', 'tric100img', 'quartz'])
def test_threaded_oracle_matches_single_thread(name):
    spec, data = gc.load(name)
    natom = len(spec['pos'])
    one = OracleForceField(spec)
    many = OracleForceField(spec, threads=4)
    for s in range(int(data['nsteps'])):
        for o in (one, many):
            o.update_pos(data['step%d_pos' % s])
        g1, v1 = np.zeros((natom, 3)), np.zeros((3, 3))
        g4, v4 = np.zeros((natom, 3)), np.zeros((3, 3))
        e1 = one.compute(g1, v1)
        e4 = many.compute(g4, v4)
        assert many.nneigh == one.nneigh
        assert np.array_equal(many.neighs[:many.nneigh], one.neighs[:one.nneigh])
        assert abs(e4 - e1) <= 1e-12 * max(abs(e1), max(abs(x) for x in one.part_energies.values()))
        assert np.abs(g4 - g1).max() <= 1e-12 * np.abs(g1).max()
        assert np.abs(v4 - v1).max() <= 1e-12 * np.abs(v1).max()
