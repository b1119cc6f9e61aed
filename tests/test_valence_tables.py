"""CPU: the host valence tables (relative vectors, internal coordinates, terms)
that are uploaded to the device equal the oracle's, which reproduce the
reference's own tables (the valence40 fixture covers every internal-coordinate
kind 0-17 and every term kind 0-15), and the class tables are complete."""
import numpy as np

import golden_cases as gc
from oracle import OracleForceField
from yaff_gb300 import valence


def test_every_kind_has_a_class():
    assert sorted(valence.IC_CLASSES) == list(range(18))
    assert sorted(valence.TERM_CLASSES) == list(range(16))


def test_fixture_covers_every_kind():
    spec, _ = gc.load('valence40')
    rows = spec['valence']
    assert set(rows[:, 0].astype(int)) == set(range(16))
    ics = set(rows[:, 7].astype(int)) | set(rows[rows[:, 12] >= 0, 12].astype(int))
    assert ics == set(range(18))


def test_host_tables_match_oracle():
    spec, _ = gc.load('valence40')

    class _Atoms(object):
        natom = len(spec['pos'])

    vl = valence.ValenceList(valence.InternalCoordinateList(valence.DeltaList(_Atoms())))
    for term in valence.terms_from_rows(spec['valence']):
        vl.add_term(term)
    dij, ics, kinds, pars, vic = vl.arrays()
    orc = OracleForceField(spec)
    assert np.array_equal(dij[:, 0], orc.dl['i']) and np.array_equal(dij[:, 1], orc.dl['j'])
    keys = ['kind', 'i0', 'sign0', 'i1', 'sign1', 'i2', 'sign2', 'i3', 'sign3']
    assert np.array_equal(ics, np.stack([orc.ic[k] for k in keys], 1))
    assert np.array_equal(kinds, orc.vt['kind'])
    assert np.array_equal(pars, np.stack([orc.vt['par%d' % i] for i in range(6)], 1))
    assert np.array_equal(vic, np.stack([orc.vt['ic0'], orc.vt['ic1']], 1))


def test_term_validation():
    import pytest
    with pytest.raises(ValueError):
        valence.PolyFour([1, 2, 3, 4, 5], valence.Bond(0, 1))
    with pytest.raises(ValueError):
        valence.ValenceTerm([0] * 7, [valence.Bond(0, 1)])
