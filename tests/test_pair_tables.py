"""CPU: the host pair-potential classes fill their type-pair tables with the
same mixing rules as the oracle (whose energies match the reference's own
fixtures bit for bit), and reject malformed tables."""
import numpy as np
import pytest

import golden_cases as gc
from oracle import type_pair_tables
from yaff_gb300 import pair
from yaff_gb300.builder import PAIR_CLASSES, make_pair_pot

TABLE_KINDS = ('exprep', 'qmdffrep', 'ljcross', 'dampdisp', 'disp68bjdamp')


@pytest.mark.parametrize('name', [n for n in gc.case_names() if n.startswith('pairpot')])
def test_mixed_tables_match_oracle(name):
    spec, _ = gc.load(name)
    seen = 0
    for p in spec['pair']:
        if p['kind'] not in TABLE_KINDS:
            continue
        pp = make_pair_pot(p, spec, PAIR_CLASSES, None, 0.0)
        want = type_pair_tables(p)
        got = pp._device_table(len(spec['pos']))
        for k, w in enumerate(want):
            assert np.array_equal(got['cross%d' % k], w), (name, p['kind'], k)
        seen += 1
    assert seen >= 1


def test_fixtures_cover_every_extra_kind():
    kinds = set()
    for n in gc.case_names():
        if n.startswith('pairpot'):
            kinds |= {p['kind'] for p in gc.load(n)[0]['pair']}
    assert kinds == {'mm3cap', 'grimme'} | set(TABLE_KINDS)


def test_table_validation():
    ids = np.array([0, 1, 2])
    with pytest.raises(TypeError):
        pair.PairPotLJCross(ids, np.ones((3, 2)), np.ones((3, 2)), 5.0)
    with pytest.raises(ValueError):
        pair.PairPotLJCross(np.array([0, 3]), np.ones((3, 3)), np.ones((3, 3)), 5.0)
    with pytest.raises(ValueError):
        pair.PairPotExpRep(ids, np.array([[1.0, 2.0, 0], [0, 1, 0], [0, 0, 1]]), np.ones((3, 3)), 5.0)
