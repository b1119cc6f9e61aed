"""Builds the reference's own ForceField from a configs.py spec.

TEST INFRASTRUCTURE ONLY: used (in the container that holds the reference
checkout) to generate golden fixtures and to pin the oracle port against the
reference itself.  Requires oracle/build_ref.sh to have been run.
"""
import numpy as np

import ref_shim


def build_reference_ff(spec):
    """Reference ForceField with the parts a spec describes, built the way the
    reference generator does (yaff/pes/generator.py:178-240)."""
    ref_shim.import_reference()
    from yaff.system import System
    from yaff.pes.ff import (ForceField, ForcePartPair, ForcePartEwaldReciprocal,
                             ForcePartEwaldCorrection, ForcePartEwaldNeutralizing,
                             ForcePartValence)
    from yaff.pes.nlist import NeighborList
    from yaff.pes.scaling import Scalings
    from yaff.pes.ext import Switch3, Hammer
    from yaff.pes.iclist import Bond, BendAngle
    from yaff.pes.vlist import Harmonic

    natom = len(spec['pos'])
    bonds = spec.get('bonds')
    system = System(numbers=np.full(natom, 6), pos=spec['pos'].copy(),
                    rvecs=spec['rvecs'].copy() if len(spec['rvecs']) else None,
                    charges=None if spec['charges'] is None else spec['charges'].copy(),
                    bonds=np.zeros((0, 2), int) if bonds is None else np.asarray(bonds, dtype=int),
                    masses=spec['masses'].copy())
    nlist = NeighborList(system, skin=spec['skin'], nlow=spec.get('nlow', 0),
                         nhigh=spec.get('nhigh', -1))
    scalings = Scalings(system, *spec['scalings'])
    tr = spec.get('tr')
    trobj = None
    if tr is not None:
        trobj = Switch3(tr[1]) if tr[0] == 'switch3' else Hammer(tr[1])
    parts = []
    ew = spec.get('ewald')
    alpha = ew['alpha'] if (ew is not None and system.cell.nvec == 3) else 0.0
    import yaff.pes.ext as rext
    from yaff_gb300.builder import make_pair_pot
    classes = {'lj': rext.PairPotLJ, 'mm3': rext.PairPotMM3, 'ei': rext.PairPotEI, 'mm3cap': rext.PairPotMM3CAP,
               'grimme': rext.PairPotGrimme, 'exprep': rext.PairPotExpRep, 'qmdffrep': rext.PairPotQMDFFRep,
               'ljcross': rext.PairPotLJCross, 'dampdisp': rext.PairPotDampDisp,
               'disp68bjdamp': rext.PairPotDisp68BJDamp}
    keep = []   # the reference's pair potentials borrow their argument arrays
    for p in spec['pair']:
        pp = make_pair_pot(p, spec, classes, trobj, alpha, keep)
        parts.append(ForcePartPair(system, nlist, scalings, pp))
    if ew is not None and system.cell.nvec == 3:
        diel = spec.get('dielectric', 1.0)
        nlow, nhigh = spec.get('nlow', 0), spec.get('nhigh', -1)
        parts.append(ForcePartEwaldReciprocal(system, ew['alpha'], ew['gcut'], diel, nlow, nhigh))
        parts.append(ForcePartEwaldCorrection(system, ew['alpha'], scalings, diel, nlow, nhigh))
        parts.append(ForcePartEwaldNeutralizing(system, ew['alpha'], diel, nlow, nhigh))
    bt = spec.get('bond_terms')
    at = spec.get('bend_terms')
    vr = spec.get('valence')
    if any(x is not None and len(x) for x in (bt, at, vr)):
        pv = ForcePartValence(system)
        for i, j, K, r0 in (bt if bt is not None else []):
            pv.add_term(Harmonic(K, r0, Bond(int(i), int(j))))
        for i, j, k, K, t0 in (at if at is not None else []):
            pv.add_term(Harmonic(K, t0, BendAngle(int(i), int(j), int(k))))
        if vr is not None and len(vr):
            from yaff_gb300.valence import terms_from_rows
            import yaff.pes.iclist as ric
            import yaff.pes.vlist as rvl
            icc = {c.kind: c for c in vars(ric).values()
                   if isinstance(c, type) and issubclass(c, ric.InternalCoordinate) and c.kind is not None}
            tcc = {c.kind: c for c in vars(rvl).values()
                   if isinstance(c, type) and issubclass(c, rvl.ValenceTerm) and c.kind is not None}
            for term in terms_from_rows(vr, icc, tcc):
                pv.add_term(term)
        parts.append(pv)
    if spec.get('tailcorr', False):
        from yaff.pes.ff import ForcePartTailCorrection
        for part in [q for q in parts if isinstance(q, ForcePartPair) and q.name != 'pair_ei']:
            parts.append(ForcePartTailCorrection(system, part, spec.get('nlow', 0), spec.get('nhigh', -1)))
    ff = ForceField(system, parts, nlist)
    ff._borrowed_arrays = keep
    return ff
