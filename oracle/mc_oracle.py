"""CPU restatement of the reference's MC trial energy (test infrastructure).

TEST INFRASTRUCTURE ONLY: the checker of the GPU trial kernels.  Follows
Trial.insertion_energy (yaff/sampling/mctrials.py:69-126) with the reference
MC's reci_ei = 'ewald_interaction' (mc.py:596-597): the guest-guest and the
host-guest energies are full evaluations of force fields built with
nlow = nhigh (pair terms, Ewald correction and neutralizing background,
no reciprocal part; oracle.OracleForceField), each replaced by 1e10 when the
guest is closer than the close-contact distance to an atom of that
subsystem (MIC distances), plus the reciprocal interaction through the
structure factors (ForcePartEwaldReciprocalInteraction.insertion_energy,
yaff/pes/ff.py:1211-1253, on orc_ewald_prefactors / structurefactors /
deltae, ewald.c:441-522).  A translation is the deletion at the old position
followed by the insertion at the new one with the structure factors reduced
by the deleted guest (TrialCartesian.compute, mctrials.py:148-168).
"""
import numpy as np

from oracle import OracleForceField, OracleCell, lib, _p


def _spec(pos, charges, sig, eps, rvecs, rcut, alpha, gcut, nlow):
    n = len(pos)
    return {'name': 'mc', 'pos': np.ascontiguousarray(pos, dtype=float),
            'rvecs': np.ascontiguousarray(rvecs, dtype=float), 'charges': np.ascontiguousarray(charges, dtype=float),
            'masses': np.ones(n), 'bonds': None,
            'pair': [{'kind': 'lj', 'sigmas': np.ascontiguousarray(sig, dtype=float),
                      'epsilons': np.ascontiguousarray(eps, dtype=float)}, {'kind': 'ei'}],
            'rcut': rcut, 'skin': 0.0, 'tr': None, 'ewald': {'alpha': alpha, 'gcut': gcut}, 'dielectric': 1.0,
            'scalings': (0.0, 0.0, 1.0, 1.0), 'nlow': nlow, 'nhigh': nlow,
            'bond_terms': np.zeros((0, 4)), 'bend_terms': np.zeros((0, 5))}


def _ff_energy(spec):
    ff = OracleForceField(spec)
    ff.compute()
    return sum(e for name, e in ff.part_energies.items() if name != 'ewald_reci')


def _dmin(cell, pos0, pos1):
    if len(pos1) == 0:
        return np.inf
    d = pos0[:, None, :] - pos1[None, :, :]
    out = np.inf
    for v in d.reshape(-1, 3):
        w = cell.mic(v)
        out = min(out, np.sqrt((w * w).sum()))
    return out


class EwaldInteraction(object):
    """Prefactors and structure factors on the reference's dense layout (one
    extra element absorbs the reference's store one past the array)."""

    def __init__(self, rvecs, alpha, gcut):
        self.cell = OracleCell(rvecs)
        self.gmax = np.ascontiguousarray(np.ceil(gcut / self.cell.gspacings - 0.5).astype(np.int64))
        self.alpha, self.gcut = alpha, gcut
        self.n = int((2 * self.gmax[0] + 1) * (2 * self.gmax[1] + 1) * (self.gmax[2] + 1))
        self.pref = np.zeros(self.n + 1)
        lib().orc_ewald_prefactors(_p(self.cell.gvecs), self.cell.volume, alpha, _p(self.gmax), gcut,
                                   _p(self.pref))

    def sfac(self, pos, q):
        c, s = np.zeros(self.n + 1), np.zeros(self.n + 1)
        p = np.ascontiguousarray(pos, dtype=float).reshape(-1, 3)
        qq = np.ascontiguousarray(q, dtype=float)
        lib().orc_ewald_structurefactors(_p(p), len(p), _p(qq), _p(self.cell.gvecs), _p(self.gmax), self.gcut,
                                         _p(c), _p(s))
        return c, s

    def deltae(self, dc, c, ds, s):
        return lib().orc_ewald_deltae(_p(dc), _p(c), _p(ds), _p(s), _p(self.pref), self.n)


def trial_energy(case, guests, kind, g, newpos):
    """U(after) - U(before) of one trial (kind 0 insert at newpos, 1 delete
    guest g, 2 translate guest g to newpos) against framework + guests."""
    fw, gt = case['framework'], case['guest']
    M = len(gt['charges'])
    rv, rcut, alpha, gcut, cc = fw['rvecs'], case['rcut'], case['alpha'], case['gcut'], case['close_contact']
    cell = OracleCell(rv)
    n = len(guests)
    ew = EwaldInteraction(rv, alpha, gcut)
    allpos = np.concatenate([fw['pos']] + list(guests)) if n else fw['pos']
    S = ew.sfac(allpos, np.concatenate([fw['charges'], np.tile(gt['charges'], n)]))

    def part(moving, others, sign, S):
        ng = len(others) + 1
        gpos = np.concatenate(list(others) + [moving]) if others else moving
        dg = _dmin(cell, moving, np.concatenate(others) if others else np.zeros((0, 3)))
        e = 1e10 if dg < cc else _ff_energy(_spec(gpos, np.tile(gt['charges'], ng), np.tile(gt['sigmas'], ng),
                                                  np.tile(gt['epsilons'], ng), rv, rcut, alpha, gcut,
                                                  M * len(others)))
        dh = _dmin(cell, moving, fw['pos'])
        nf = len(fw['pos'])
        e += 1e10 if dh < cc else _ff_energy(_spec(np.concatenate([fw['pos'], moving]),
                                                   np.concatenate([fw['charges'], gt['charges']]),
                                                   np.concatenate([fw['sigmas'], gt['sigmas']]),
                                                   np.concatenate([fw['epsilons'], gt['epsilons']]), rv, rcut,
                                                   alpha, gcut, nf))
        dc, ds = ew.sfac(moving, gt['charges'])
        if sign == -1:
            S = (S[0] - dc, S[1] - ds)
        e += ew.deltae(dc, S[0], ds, S[1])
        return sign * e, S

    if kind == 0:
        return part(newpos, list(guests), 1, S)[0]
    others = [guests[i] for i in range(n) if i != g]
    e, S = part(guests[g], others, -1, S)
    if kind == 1:
        return e
    return e + part(newpos, others, 1, S)[0]
