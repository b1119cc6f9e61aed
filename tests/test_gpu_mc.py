"""GPU: MC trial energies (yg_mc_*, yg_ewald_prefactors / structurefactors /
deltae) against the reference's own MC trial code (golden fixtures) and the
oracle.

Tolerances: FP64 trial energies 1e-9 relative (CUDA's sincos/erfc against
glibc's, different summation order); mixed 1e-6 relative to
max(|dE|, 1e-3 Ha); structure factors 1e-12 of the largest element;
prefactors bit-exact (same host code path and operation order).
"""
import numpy as np
import pytest

import golden_cases

pytestmark = pytest.mark.gpu

NAMES = golden_cases.mc_case_names()


def _engine(case, nchain=2, max_guests=64, precision='fp64'):
    from yaff_gb300.mc import MCTrials
    from yaff_gb300.system import Cell
    cell = Cell(case['framework']['rvecs'])
    return MCTrials(case['framework'], case['guest'], cell, case['rcut'], case['alpha'], case['gcut'], nchain,
                    max_guests, close_contact=case['close_contact'], precision=precision)


def _rel(e, ref, floor=1e-3):
    return np.abs(e - ref) / np.maximum(np.abs(ref), floor)


@pytest.mark.parametrize('name', NAMES)
def test_structure_factor_functions(name):
    from yaff_gb300.mc import compute_ewald_prefactors, compute_ewald_structurefactors, compute_ewald_deltae
    from yaff_gb300.system import Cell
    case, d = golden_cases.load_mc(name)
    cell = Cell(d['rvecs'])
    gmax = np.ascontiguousarray(d['gmax'], dtype=np.int64)
    pref = np.zeros(d['prefactors'].shape)
    compute_ewald_prefactors(cell, float(d['alpha']), gmax, float(d['gcut']), pref)
    np.testing.assert_array_equal(pref, d['prefactors'])
    allpos = np.ascontiguousarray(np.concatenate([d['frame_pos']] + list(d['chain'])))
    allq = np.ascontiguousarray(np.concatenate([d['frame_charges'], np.tile(d['guest_charges'], len(d['chain']))]))
    c, s = np.zeros(pref.shape), np.zeros(pref.shape)
    compute_ewald_structurefactors(allpos, allq, cell, float(d['alpha']), gmax, float(d['gcut']), c, s)
    scale = np.abs(d['cosfacs']).max()
    assert np.abs(c - d['cosfacs']).max() <= 1e-12 * scale
    assert np.abs(s - d['sinfacs']).max() <= 1e-12 * scale
    # ADDED, not overwritten
    c2 = c.copy()
    compute_ewald_structurefactors(allpos, allq, cell, float(d['alpha']), gmax, float(d['gcut']), c2, s.copy())
    assert np.abs(c2 - 2 * c).max() <= 1e-12 * scale
    de = compute_ewald_deltae(d['prefactors'], d['dcos'], d['cosfacs'], d['dsin'], d['sinfacs'])
    assert de == pytest.approx(float(d['deltae']), rel=1e-12)


@pytest.mark.parametrize('name', NAMES)
@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_trials_match_reference(name, precision):
    case, d = golden_cases.load_mc(name)
    eng = _engine(case, precision=precision)
    eng.set_chain(1, d['chain'])
    pos, cos, sin = eng.get_chain(1)
    np.testing.assert_array_equal(pos, d['chain'])
    scale = np.abs(d['cosfacs']).max()
    assert np.abs(cos - d['cosfacs']).max() <= 1e-12 * scale
    assert np.abs(sin - d['sinfacs']).max() <= 1e-12 * scale
    np.testing.assert_array_equal(eng.prefactors(), d['prefactors'])
    n = len(d['kind'])
    e = eng.trials(np.ones(n, np.int32), d['kind'], d['guest'], d['newpos'])
    tol = 1e-9 if precision == 'fp64' else 1e-6
    assert _rel(e, d['energy']).max() <= tol, (_rel(e, d['energy']).max(), precision)
    # chain 0 is empty: an insertion there sees the framework only
    e0 = eng.trials(np.zeros(1, np.int32), np.zeros(1, np.int32), -np.ones(1, np.int32), d['newpos'][:1])
    import mc_oracle
    ref0 = mc_oracle.trial_energy(case, [], 0, -1, d['newpos'][0])
    assert _rel(e0, np.array([ref0])).max() <= tol


def test_apply_updates_like_recompute():
    """Accepted insertion / deletion / translation: resident positions and
    structure factors equal a fresh set-up of the resulting chains, and a
    later trial agrees with the oracle on the new state."""
    import mc_oracle
    case, d = golden_cases.load_mc(NAMES[0])
    eng = _engine(case, nchain=3)
    chain = list(d['chain'])
    for c in range(3):
        eng.set_chain(c, chain)
    kinds = d['kind']
    ti = [int(np.where(kinds == k)[0][0]) for k in (0, 1, 2)]
    e = eng.trials(np.arange(3, dtype=np.int32), kinds[ti], d['guest'][ti], d['newpos'][ti])
    assert np.isfinite(e).all()
    eng.apply(np.arange(3, dtype=np.int32))
    expect = [chain + [d['newpos'][ti[0]]]]
    g = int(d['guest'][ti[1]])
    after_del = list(chain)
    after_del[g] = after_del[-1]
    expect.append(after_del[:-1])
    g = int(d['guest'][ti[2]])
    after_tr = list(chain)
    after_tr[g] = d['newpos'][ti[2]]
    expect.append(after_tr)
    fresh = _engine(case, nchain=3)
    for c in range(3):
        pos, cos, sin = eng.get_chain(c)
        np.testing.assert_array_equal(pos, np.array(expect[c]))
        fresh.set_chain(c, expect[c])
        _, cos2, sin2 = fresh.get_chain(c)
        scale = np.abs(cos2).max()
        assert np.abs(cos - cos2).max() <= 1e-11 * scale
        assert np.abs(sin - sin2).max() <= 1e-11 * scale
    # a trial on the updated chain 1 (after the deletion)
    g = 0
    newp = expect[1][g] + 0.3
    e = eng.trials(np.ones(1, np.int32), np.full(1, 2, np.int32), np.zeros(1, np.int32), newp[None])
    ref = mc_oracle.trial_energy(case, expect[1], 2, g, newp)
    assert _rel(e, np.array([ref])).max() <= 1e-9


def test_framework2000_trials_mixed_vs_fp64_and_oracle():
    """The 2,000-atom framework with a loaded chain: 64 mixed trials within
    1e-6 of the FP64 ones; a few FP64 trials against the oracle."""
    import mc_oracle
    from yaff_gb300 import configs
    work = configs.mc_workload(nchain=2, seed=7)
    work['chains'][1] = work['chains'][1][:150]
    case = {'framework': work['framework'], 'guest': work['guest'], 'rcut': work['rcut'], 'alpha': work['alpha'],
            'gcut': work['gcut'], 'close_contact': work['close_contact']}
    eng = _engine(case, nchain=2, max_guests=400, precision='fp64')
    for c in range(2):
        eng.set_chain(c, work['chains'][c])
    rng = np.random.default_rng(3)
    ch, kind, guest, newpos = configs.mc_trial_batch(rng, work, work['chains'], 32)
    e64 = eng.trials(ch, kind, guest, newpos)
    eng.set_precision('mixed')
    e32 = eng.trials(ch, kind, guest, newpos)
    finite = np.abs(e64) < 1e9
    assert finite.sum() >= 8
    assert _rel(e32[finite], e64[finite]).max() <= 1e-6
    assert (np.abs(e32[~finite]) >= 1e9).all()
    for t in np.where(finite)[0][:3]:
        ref = mc_oracle.trial_energy(case, list(work['chains'][ch[t]]), int(kind[t]), int(guest[t]), newpos[t])
        assert _rel(e64[t:t + 1], np.array([ref])).max() <= 1e-9
