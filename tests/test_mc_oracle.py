"""CPU: the MC trial-energy oracle against the reference's own MC trial
code (golden fixtures made by tests/golden/make_mc_golden.py)."""
import numpy as np
import pytest

import golden_cases

NAMES = golden_cases.mc_case_names()


@pytest.mark.parametrize('name', NAMES)
def test_mc_oracle_matches_reference(name):
    import mc_oracle
    case, d = golden_cases.load_mc(name)
    chain = list(d['chain'])
    for t in range(len(d['kind'])):
        e = mc_oracle.trial_energy(case, chain, int(d['kind'][t]), int(d['guest'][t]), d['newpos'][t])
        assert e == pytest.approx(d['energy'][t], rel=1e-12, abs=1e-12)
    ew = mc_oracle.EwaldInteraction(d['rvecs'], float(d['alpha']), float(d['gcut']))
    np.testing.assert_array_equal(ew.gmax, d['gmax'])
    np.testing.assert_array_equal(ew.pref[:-1], d['prefactors'].ravel())
    allpos = np.concatenate([d['frame_pos']] + chain)
    allq = np.concatenate([d['frame_charges'], np.tile(d['guest_charges'], len(chain))])
    c, s = ew.sfac(allpos, allq)
    np.testing.assert_array_equal(c[:-1], d['cosfacs'].ravel())
    np.testing.assert_array_equal(s[:-1], d['sinfacs'].ravel())
    dc, ds = ew.sfac(d['chain'][0], d['guest_charges'])
    assert ew.deltae(dc, c, ds, s) == pytest.approx(float(d['deltae']), rel=1e-13)


def test_mc_fixtures_cover_every_trial_kind_and_close_contact():
    kinds = set()
    close = False
    for name in NAMES:
        _, d = golden_cases.load_mc(name)
        kinds |= set(int(k) for k in d['kind'])
        close |= bool((np.abs(d['energy']) >= 1e9).any())
    assert kinds == {0, 1, 2} and close
