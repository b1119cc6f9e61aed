"""GPU: neighbour rows split at the pair cutoff.

The build puts the entries within the largest pair cutoff at the front of an
atom's row and the skin shell (up to rcut + skin) at the back; on a list built
from the current coordinates the pair kernel reads only the front.  After a
skin-path recompute it reads both segments.  With the positions unchanged the
back entries lie beyond every pair cutoff, and the front entries keep their
order and lanes, so the pair parts must be bitwise the same either way, in
every precision form."""
import ctypes

import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu


def _pair_parts(ff):
    import yaff_gb300
    from yaff_gb300 import _lib
    from yaff_gb300.device import device_of
    dev = device_of(ff.system)
    parts = [p for p in ff.parts if isinstance(p, yaff_gb300.ForcePartPair)]
    mask = 0
    for p in parts:
        mask |= 1 << p._register()
    _lib.check(dev.lib.yg_pair_compute(dev.ctx, mask, 1), 'yg_pair_compute')
    out = []
    for p in parts:
        g, v = np.zeros((ff.system.natom, 3)), np.zeros((3, 3))
        e = dev.get_part(_lib.PART_PAIR0 + p._register(), g, v)
        out.append((e, g, v))
    return dev, out


@pytest.mark.parametrize('precision', ['fp64', 'mixed', 'mixed_kahan'])
@pytest.mark.parametrize('case', ['tric600', 'water64'])
def test_skin_shell_read_or_skipped_gives_the_same_pair_terms(case, precision):
    import yaff_gb300
    from yaff_gb300 import _lib
    spec, data = gc.load(case)
    ff = yaff_gb300.build_forcefield(spec, precision=precision)
    n = len(spec['pos'])
    ff.compute(np.zeros((n, 3)), np.zeros((3, 3)))   # registers the pair potentials
    ff.nlist.rebuild_next = True
    ff.update_pos(spec['pos'])
    ff.compute(np.zeros((n, 3)), np.zeros((3, 3)))   # a build with the potentials known
    dev, fresh = _pair_parts(ff)
    _lib.check(dev.lib.yg_nlist_recompute(dev.ctx), 'yg_nlist_recompute')   # same positions, skin path
    _, again = _pair_parts(ff)
    for (e0, g0, v0), (e1, g1, v1) in zip(fresh, again):
        assert e0 == e1
        np.testing.assert_array_equal(g0, g1)
        np.testing.assert_array_equal(v0, v1)
    e_ref = float(data['step0_energy'])
    g = np.zeros((n, 3))
    e = ff.compute(g, np.zeros((3, 3)))
    tol = 1e-10 if precision == 'fp64' else 1e-6
    assert abs(e - e_ref) <= tol * np.abs(data['step0_part_energy']).max()
