"""CPU: tail corrections (C0, C1 of every non-electrostatic pair part) from
the host pair classes against the reference's own values in the tailcorr*
fixtures (untruncated and Switch3; nlow / nhigh ranges; every pair kind
with a tail model).  The reference evaluates Maple closed forms whose
constants carry ten significant digits (e.g. 0.3666666667 for 1.1/3,
yaff/pes/tailcorr.c:254), so the bar is 1e-8 relative; the host integrals
are exact to FP64 rounding (closed forms beyond the cutoff, 48-point
Gauss-Legendre over the switching interval)."""
import numpy as np
import pytest

import golden_cases as gc
from yaff_gb300.builder import PAIR_CLASSES, make_pair_pot
from yaff_gb300.pair import Switch3

CASES = [n for n in gc.case_names() if n.startswith('tailcorr')]


@pytest.mark.parametrize('name', CASES)
def test_tail_corrections_match_reference(name):
    spec, data = gc.load(name)
    natom = len(spec['pos'])
    tr = spec.get('tr')
    trobj = Switch3(tr[1]) if tr is not None else None
    checked = 0
    for p in spec['pair']:
        if p['kind'] == 'ei':
            continue
        key = 'tailcorr_pair_%s' % p['kind']
        pp = make_pair_pot(p, spec, PAIR_CLASSES, trobj, 0.0)
        e, w = pp.prepare_tailcorrections(natom, spec['nlow'], spec['nhigh'])
        re, rw = float(data[key + '_ecorr']), float(data[key + '_wcorr'])
        assert abs(e - re) <= 1e-8 * abs(re), (key, e, re)
        assert abs(w - rw) <= 1e-8 * abs(rw), (key, w, rw)
        checked += 1
    assert checked >= 1


def test_cases_cover_kinds_and_truncations():
    kinds, trs = set(), set()
    for n in CASES:
        spec, _ = gc.load(n)
        kinds |= {p['kind'] for p in spec['pair'] if p['kind'] != 'ei'}
        trs.add(None if spec.get('tr') is None else spec['tr'][0])
    assert kinds == {'lj', 'mm3', 'mm3cap', 'grimme', 'exprep', 'qmdffrep', 'ljcross', 'dampdisp', 'disp68bjdamp'}
    assert trs == {None, 'switch3'}


def test_hammer_is_rejected():
    from yaff_gb300.pair import Hammer, PairPotLJ
    pp = PairPotLJ(np.ones(4), np.ones(4), 5.0, Hammer(1.0))
    with pytest.raises(NotImplementedError):
        pp.prepare_tailcorrections(4)
