"""GPU: the device force path against the reference's golden fixtures.

Pair set: (a, b, r0, r1, r2) identical to the reference (SHA-256 of the
sorted keys), and on build steps d, dx, dy, dz bit-identical too.
Energies: FP64 within 1e-10 relative, mixed within 1e-6 relative; gradients
and virials: FP64 within 1e-9, mixed within 1e-5 relative RMS (the parity
tolerances of this path).  Energies are compared relative to the largest
part magnitude of the case, since the total can be a near-cancelling sum.
"""
import hashlib

import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

TOL = {'fp64': (1e-10, 1e-9), 'mixed': (1e-6, 1e-5), 'mixed_kahan': (1e-6, 1e-5)}
TAIL_TOL = 1e-8


def _digest(keys):
    return hashlib.sha256(np.ascontiguousarray(keys, dtype='<i8').tobytes()).hexdigest()


@pytest.fixture(scope='module')
def ygb():
    import yaff_gb300
    return yaff_gb300


@pytest.mark.parametrize('precision', ['fp64', 'mixed', 'mixed_kahan'])
@pytest.mark.parametrize('name', gc.case_names())
def test_golden_case(ygb, name, precision):
    spec, data = gc.load(name)
    ff = ygb.build_forcefield(spec, precision=precision)
    etol, gtol = TOL[precision]
    natom = len(spec['pos'])
    for s in range(int(data['nsteps'])):
        ff.update_pos(data['step%d_pos' % s])
        gpos = np.zeros((natom, 3))
        vtens = np.zeros((3, 3))
        e = ff.compute(gpos, vtens)
        # neighbour list: identical pair set
        assert ff.nlist.nneigh == int(data['step%d_nneigh' % s])
        keys, vals = gc.pair_keys_from_rows(ff.nlist.neighs)
        assert _digest(keys) == str(data['step%d_pairs_sha256' % s]), 'pair set differs at step %d' % s
        if ('step%d_pair_keys' % s) in data:
            assert np.array_equal(vals, data['step%d_pair_vals' % s]), 'row values differ at step %d' % s
        names = [str(x) for x in data['step%d_parts' % s]]
        pe = data['step%d_part_energy' % s]
        pv = data['step%d_part_vtens' % s]
        scale = max(abs(pe).max(), abs(float(data['step%d_energy' % s])), 1e-30)
        # tail corrections: host FP64 integrals within TAIL_TOL of the
        # reference's ten-digit closed forms (tests/test_tailcorr.py)
        tail = [k for k, nm in enumerate(names) if nm.startswith('tailcorr_')]
        allow = TAIL_TOL * sum(abs(pe[k]) for k in tail)
        assert abs(e - float(data['step%d_energy' % s])) <= etol * scale + allow
        vt_ref, vt = data['step%d_vtens' % s].copy(), vtens.copy()
        for k, nm in enumerate(names):
            part = getattr(ff, 'part_' + nm)
            if k in tail:
                assert abs(part.energy - pe[k]) <= TAIL_TOL * abs(pe[k]), nm
                assert np.allclose(part.vtens, pv[k], rtol=TAIL_TOL, atol=0), nm
                vt_ref -= pv[k]
                vt -= part.vtens
                continue
            assert abs(part.energy - pe[k]) <= etol * scale, nm
            gref = data['step%d_part_gpos' % s][k]
            if abs(gref).max() > 0:
                assert gc.rel_rms(part.gpos, gref) <= gtol, nm
        assert gc.rel_rms(gpos, data['step%d_gpos' % s]) <= gtol
        assert gc.rel_rms(vt, vt_ref) <= gtol


def test_nlist_bruteforce_check(ygb):
    spec, data = gc.load('tric100img')
    ff = ygb.build_forcefield(spec, precision='fp64')
    ff.compute()
    ff.nlist.check()


def test_standalone_parts_match_fused(ygb):
    spec, data = gc.load('water64')
    ff = ygb.build_forcefield(spec, precision='fp64')
    g1 = np.zeros((len(spec['pos']), 3))
    v1 = np.zeros((3, 3))
    e1 = ff.compute(g1, v1)
    parts_e = {p.name: p.energy for p in ff.parts}
    parts_g = {p.name: p.gpos.copy() for p in ff.parts}
    g2 = np.zeros_like(g1)
    v2 = np.zeros((3, 3))
    e2 = 0.0
    for p in ff.parts:
        e2 += p.compute(g2, v2)
        assert abs(p.energy - parts_e[p.name]) <= 1e-12 * max(1, abs(parts_e[p.name]))
        assert np.allclose(p.gpos, parts_g[p.name], atol=1e-12)
    assert abs(e1 - e2) < 1e-10
    assert np.allclose(g1, g2, atol=1e-10)


def test_nan_positions_raise(ygb):
    spec, data = gc.load('lat216')
    ff = ygb.build_forcefield(spec, precision='mixed')
    ff.compute()
    pos = spec['pos'].copy()
    pos[3, 1] = np.nan
    ff.update_pos(pos)
    with pytest.raises(ValueError):
        ff.compute(np.zeros((len(pos), 3)), np.zeros((3, 3)))


def test_nan_result_leaves_callers_arrays_untouched(ygb):
    """A NaN in the result raises ValueError before anything reaches the
    caller's gpos / vtens, as in the reference (yaff/pes/ff.py:156-168).
    Where the device adds the gradient into the caller's array itself
    (pageable host memory reached through the host's page tables) the
    result's status is checked on the device first.  A valid evaluation adds
    into the caller's arrays."""
    spec, data = gc.load('tric600')
    ff = ygb.build_forcefield(spec, precision='mixed')
    n = len(spec['pos'])
    g0, v0 = np.zeros((n, 3)), np.zeros((3, 3))
    e0 = ff.compute(g0, v0)
    g, v = np.full((n, 3), 7.0), np.full((3, 3), 7.0)
    assert ff.compute(g, v) == e0
    assert np.allclose(g - 7.0, g0, rtol=0, atol=1e-12) and np.allclose(v - 7.0, v0, rtol=0, atol=1e-12)
    ff.system.charges[5] = np.nan
    g, v = np.full((n, 3), 7.0), np.full((3, 3), 7.0)
    with pytest.raises(ValueError):
        ff.compute(g, v)
    assert (g == 7.0).all() and (v == 7.0).all()
