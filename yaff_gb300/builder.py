"""Builds a device ForceField from a configs.py spec (the parts the
reference generator would create: yaff/pes/generator.py:178-240)."""
import numpy as np

from .device import device_of
from .ff import (ForceField, ForcePartPair, ForcePartEwaldReciprocal, ForcePartEwaldCorrection,
                 ForcePartEwaldNeutralizing, ForcePartTailCorrection, ForcePartValence)
from .nlist import NeighborList
from . import pair as _pair
from .pair import Switch3, Hammer
from .scaling import Scalings
from .system import System
from .valence import Bond, BendAngle, Harmonic, terms_from_rows

__all__ = ['build_system', 'build_forcefield', 'make_pair_pot', 'PAIR_CLASSES']

PAIR_CLASSES = {'lj': _pair.PairPotLJ, 'mm3': _pair.PairPotMM3, 'ei': _pair.PairPotEI,
                'mm3cap': _pair.PairPotMM3CAP, 'grimme': _pair.PairPotGrimme, 'exprep': _pair.PairPotExpRep,
                'qmdffrep': _pair.PairPotQMDFFRep, 'ljcross': _pair.PairPotLJCross,
                'dampdisp': _pair.PairPotDampDisp, 'disp68bjdamp': _pair.PairPotDisp68BJDamp}


def _opt(p, key, conv):
    v = p.get(key)
    return None if v is None else conv(v)


def make_pair_pot(p, spec, classes, trobj, alpha, keep=None):
    """The pair potential a workload entry describes, from `classes` (kind
    name -> class with the reference's constructor arguments).  Tables are
    passed as fresh C-contiguous arrays, since mixing rules fill them in
    place; every array passed is also appended to `keep` when given (for
    classes that hold borrowed pointers to their arguments)."""
    k, rcut = p['kind'], spec['rcut']
    keep = [] if keep is None else keep

    def arr(key, dt=np.float64):
        if p.get(key) is None:
            return None
        a = np.array(p[key], dtype=dt, order='C')
        keep.append(a)
        return a

    cls = classes[k]
    if k == 'lj':
        return cls(arr('sigmas'), arr('epsilons'), rcut, trobj)
    if k in ('mm3', 'mm3cap'):
        return cls(arr('sigmas'), arr('epsilons'), arr('onlypaulis', np.intc), rcut, trobj)
    if k == 'ei':
        q = np.array(spec['charges'], dtype=np.float64)
        keep.append(q)
        return cls(q, alpha, rcut,
                   trobj if p.get('smooth', False) else None, spec.get('dielectric', 1.0), arr('radii'))
    if k == 'grimme':
        return cls(arr('r0'), arr('c6'), rcut, trobj)
    ids = arr('ffatype_ids', np.int64)
    if k in ('exprep', 'qmdffrep'):
        kw = {}
        if p.get('amps') is not None:
            kw.update(amps=arr('amps'), amp_mix=int(p['amp_mix']), amp_mix_coeff=float(p['amp_mix_coeff']))
        if p.get('bs') is not None:
            kw.update(bs=arr('bs'), b_mix=int(p['b_mix']), b_mix_coeff=float(p['b_mix_coeff']))
        return cls(ids, arr('amp_cross'), arr('b_cross'), rcut, trobj, **kw)
    if k == 'ljcross':
        return cls(ids, arr('eps_cross'), arr('sig_cross'), rcut, trobj)
    if k == 'dampdisp':
        return cls(ids, arr('cn_cross'), arr('b_cross'), rcut, trobj, cns=arr('cns'), bs=arr('bs'), vols=arr('vols'),
                   power=int(p.get('power', 6)))
    if k == 'disp68bjdamp':
        return cls(ids, arr('c6_cross'), arr('c8_cross'), arr('R_cross'), rcut, trobj,
                   c6_scale=float(p.get('c6_scale', 1.0)), c8_scale=float(p.get('c8_scale', 1.0)),
                   bj_a=float(p.get('bj_a', 0.0)), bj_b=float(p.get('bj_b', 0.0)))
    raise ValueError(k)


def build_system(spec):
    n = len(spec['pos'])
    return System(numbers=np.full(n, 6), pos=spec['pos'], rvecs=spec['rvecs'],
                  charges=spec.get('charges'), masses=spec.get('masses'),
                  bonds=np.zeros((0, 2), np.int64) if spec.get('bonds') is None else spec['bonds'])


def build_forcefield(spec, precision=None, system=None, stream=None):
    """ForceField for `spec` whose parts all run on the GPU; `precision` is
    'fp64' (plain), 'mixed' or 'mixed_kahan'; `stream` a cudaStream_t handle."""
    if system is None:
        system = build_system(spec)
    if precision is not None or stream is not None:
        device_of(system, precision, stream=stream)
    nlist = NeighborList(system, skin=spec['skin'], nlow=spec.get('nlow', 0), nhigh=spec.get('nhigh', -1))
    scalings = Scalings(system, *spec['scalings'])
    tr = spec.get('tr')
    trobj = None
    if tr is not None:
        trobj = Switch3(tr[1]) if tr[0] == 'switch3' else Hammer(tr[1])
    ew = spec.get('ewald')
    alpha = ew['alpha'] if (ew is not None and system.cell.nvec == 3) else 0.0
    parts = []
    for p in spec['pair']:
        pp = make_pair_pot(p, spec, PAIR_CLASSES, trobj, alpha)
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
        for term in terms_from_rows(vr if vr is not None else np.zeros((0, 17))):
            pv.add_term(term)
        parts.append(pv)
    if spec.get('tailcorr', False):
        # after every other part, as the reference generator appends them
        # (yaff/pes/generator.py:2209-2223)
        for part in [q for q in parts if isinstance(q, ForcePartPair) and q.name != 'pair_ei']:
            parts.append(ForcePartTailCorrection(system, part, spec.get('nlow', 0), spec.get('nhigh', -1)))
    return ForceField(system, parts, nlist)
