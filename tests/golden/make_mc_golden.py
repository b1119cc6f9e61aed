"""Generate tests/golden/mc_trials_*.npz by running the reference's own MC
trial code (yaff/sampling/mctrials.py:69-126 on the reference ForceField and
ForcePartEwaldReciprocalInteraction).

Run in a container that holds the reference checkout after
``sh oracle/build_ref.sh``:

    python tests/golden/make_mc_golden.py

Each case stores a framework, a guest template, one chain of guests, a list
of trials (kind 0 insertion, 1 deletion, 2 translation; guest index; new
guest positions) and the reference energy difference of each trial, plus the
reference's prefactor and structure-factor arrays of the chain and a
compute_ewald_deltae value.  The trial energies come from the reference's
Trial.insertion_energy called the way TrialInsertion / TrialDeletion /
TrialCartesian.compute call it, on reference force fields built with
nlow = nhigh (guest-guest and host-guest) and the reference MC's
reci_ei = 'ewald_interaction' (no reciprocal part in the force fields).
"""
import os
import sys
import types
import warnings

import numpy as np

warnings.filterwarnings('ignore')
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, 'oracle'))

from yaff_gb300 import configs  # noqa: E402
from yaff_gb300.units import angstrom  # noqa: E402
import ref_shim  # noqa: E402
from ref_ff import build_reference_ff  # noqa: E402


def ff_spec(pos, charges, sig, eps, rvecs, rcut, alpha, gcut, nlow):
    spec = configs._base_spec('mc', np.ascontiguousarray(pos), np.ascontiguousarray(rvecs))
    spec['charges'] = np.ascontiguousarray(charges, dtype=float)
    spec['pair'] = [{'kind': 'lj', 'sigmas': np.ascontiguousarray(sig, dtype=float),
                     'epsilons': np.ascontiguousarray(eps, dtype=float)}, {'kind': 'ei'}]
    spec['rcut'] = rcut
    spec['ewald'] = {'alpha': alpha, 'gcut': gcut}
    spec['nlow'] = nlow
    spec['nhigh'] = nlow
    return spec


def reference_ff(spec):
    ff = build_reference_ff(spec)
    ff.parts = [p for p in ff.parts if p.name != 'ewald_reci']  # reci_ei = 'ewald_interaction'
    return ff


def reference_trial(case, guests, kind, g, newpos):
    """U(after) - U(before) of one trial through the reference's code."""
    ref_shim.import_reference()
    from yaff.sampling.mctrials import Trial
    from yaff.pes.ff import ForcePartEwaldReciprocalInteraction
    from yaff.system import System
    fw, gt = case['framework'], case['guest']
    M = len(gt['charges'])
    rv, rcut, alpha, gcut = fw['rvecs'], case['rcut'], case['alpha'], case['gcut']
    n = len(guests)
    others = [guests[i] for i in range(n) if kind == 0 or i != g]
    moving = newpos if kind == 0 else guests[g]
    # guest-guest force field: the other guests, then the moving guest
    gpos = np.concatenate(others + [moving]) if others else moving.copy()
    ng = len(others) + 1
    ff = reference_ff(ff_spec(gpos, np.tile(gt['charges'], ng), np.tile(gt['sigmas'], ng),
                              np.tile(gt['epsilons'], ng), rv, rcut, alpha, gcut, M * len(others)))
    # host-guest force field: the framework, then the moving guest
    nf = len(fw['pos'])
    hpos = np.concatenate([fw['pos'], moving])
    ext = reference_ff(ff_spec(hpos, np.concatenate([fw['charges'], gt['charges']]),
                               np.concatenate([fw['sigmas'], gt['sigmas']]),
                               np.concatenate([fw['epsilons'], gt['epsilons']]), rv, rcut, alpha, gcut, nf))
    # current state: framework + all guests
    allpos = np.concatenate([fw['pos']] + list(guests)) if n else fw['pos'].copy()
    allq = np.concatenate([fw['charges'], np.tile(gt['charges'], n)])
    ewi = ForcePartEwaldReciprocalInteraction(ext.system.cell, alpha, gcut, pos=allpos, charges=allq)
    shape = ewi.cosfacs.shape
    guest_sys = System(numbers=np.array([8, 1, 1][:M]), pos=gt['pos'].copy(), rvecs=rv.copy())
    mc = types.SimpleNamespace(guest=guest_sys, close_contact=case['close_contact'], eguest=0.0,
                               external_potential=ext, ewald_reci=ewi,
                               cosfacs_ins=np.zeros(shape), sinfacs_ins=np.zeros(shape),
                               cosfacs_del=np.zeros(shape), sinfacs_del=np.zeros(shape))
    trial = Trial(mc)
    if kind == 0:
        return trial.insertion_energy(ff)
    if kind == 1:
        return trial.insertion_energy(ff, sign=-1)
    e = trial.insertion_energy(ff, sign=-1)
    ff.system.pos[-M:] = newpos
    e += trial.insertion_energy(ff, sign=1)
    return e


def make_case(name, nframe, box, nguest, rcut, seed, ntrial=8):
    rng = np.random.default_rng(seed)
    fw = configs.mc_framework(natom=nframe, box=box, seed=seed)
    gt = configs.mc_guest()
    ew = configs.ewald_params(rcut * angstrom)
    case = {'framework': fw, 'guest': gt, 'rcut': rcut * angstrom, 'alpha': ew['alpha'], 'gcut': ew['gcut'],
            'close_contact': 0.4 * angstrom}
    guests = configs.mc_place_guests(rng, nguest, fw['rvecs'])
    kinds, gidx, newpos, energy = [], [], [], []
    for kind in (0, 1, 2):
        for t in range(ntrial):
            g = int(rng.integers(0, nguest))
            if kind == 0:
                npos = configs.mc_place_guests(rng, 1, fw['rvecs'])[0]
            elif kind == 1:
                npos = np.zeros((3, 3))
            else:
                npos = guests[g] + rng.uniform(-1.0, 1.0, 3) * angstrom
            e = reference_trial(case, guests, kind, g, npos)
            kinds.append(kind)
            gidx.append(-1 if kind == 0 else g)
            newpos.append(npos)
            energy.append(e)
    # the reference's structure-factor functions on the chain
    ref_shim.import_reference()
    from yaff.pes.ext import compute_ewald_prefactors, compute_ewald_structurefactors, compute_ewald_deltae, Cell
    cell = Cell(fw['rvecs'].copy())
    gmax = np.ceil(case['gcut'] / cell.gspacings - 0.5).astype(int)
    shape = (2 * gmax[0] + 1, 2 * gmax[1] + 1, gmax[2] + 1)
    pref = np.zeros(shape)
    compute_ewald_prefactors(cell, case['alpha'], gmax, case['gcut'], pref)
    allpos = np.ascontiguousarray(np.concatenate([fw['pos']] + list(guests)))
    allq = np.ascontiguousarray(np.concatenate([fw['charges'], np.tile(gt['charges'], nguest)]))
    cos, sin = np.zeros(shape), np.zeros(shape)
    compute_ewald_structurefactors(allpos, allq, cell, case['alpha'], gmax, case['gcut'], cos, sin)
    dcos, dsin = np.zeros(shape), np.zeros(shape)
    compute_ewald_structurefactors(np.ascontiguousarray(guests[0]), np.ascontiguousarray(gt['charges']), cell,
                                   case['alpha'], gmax, case['gcut'], dcos, dsin)
    de = compute_ewald_deltae(pref, dcos, cos, dsin, sin)
    np.savez_compressed(os.path.join(HERE, name + '.npz'),
                        frame_pos=fw['pos'], frame_charges=fw['charges'], frame_sigmas=fw['sigmas'],
                        frame_epsilons=fw['epsilons'], rvecs=fw['rvecs'], guest_pos=gt['pos'],
                        guest_charges=gt['charges'], guest_sigmas=gt['sigmas'], guest_epsilons=gt['epsilons'],
                        rcut=case['rcut'], alpha=case['alpha'], gcut=case['gcut'],
                        close_contact=case['close_contact'], chain=guests, kind=np.array(kinds),
                        guest=np.array(gidx), newpos=np.array(newpos), energy=np.array(energy), gmax=gmax,
                        prefactors=pref, cosfacs=cos, sinfacs=sin, dcos=dcos, dsin=dsin, deltae=de)
    print(name, 'nk-dense', pref.size, 'trials', len(energy), 'E range', min(energy), max(energy))


def main():
    if not ref_shim.reference_available():
        raise SystemExit('reference not available: run oracle/build_ref.sh in a container with the checkout')
    make_case('mc_trials_a', 300, 26.0, 25, 12.0, seed=11)
    make_case('mc_trials_b', 60, 13.0, 6, 9.0, seed=12)


if __name__ == '__main__':
    main()
