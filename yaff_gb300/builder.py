"""Builds a device ForceField from a configs.py spec (the parts the
reference generator would create: yaff/pes/generator.py:178-240)."""
import numpy as np

from .device import device_of
from .ff import (ForceField, ForcePartPair, ForcePartEwaldReciprocal, ForcePartEwaldCorrection,
                 ForcePartEwaldNeutralizing, ForcePartValence)
from .nlist import NeighborList
from .pair import PairPotLJ, PairPotMM3, PairPotEI, Switch3, Hammer
from .scaling import Scalings
from .system import System
from .valence import Bond, BendAngle, Harmonic, terms_from_rows

__all__ = ['build_system', 'build_forcefield']


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
        if p['kind'] == 'lj':
            pp = PairPotLJ(p['sigmas'], p['epsilons'], spec['rcut'], trobj)
        elif p['kind'] == 'mm3':
            pp = PairPotMM3(p['sigmas'], p['epsilons'], p['onlypaulis'], spec['rcut'], trobj)
        elif p['kind'] == 'ei':
            pp = PairPotEI(spec['charges'], alpha, spec['rcut'], trobj if p.get('smooth', False) else None,
                           spec.get('dielectric', 1.0), p.get('radii'))
        else:
            raise ValueError(p['kind'])
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
    return ForceField(system, parts, nlist)
