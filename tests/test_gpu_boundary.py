"""GPU: the device parts driven the way the reference drives its parts.

The reference's ForceField (yaff/pes/ff.py:178-273) and VerletIntegrator
(yaff/sampling/verlet.py:320-367) are restated below in their call sequence:
update_pos writes system.pos in place and flags the neighbour list;
compute updates the list once and sums part.compute(gpos, vtens); parts are
never told about position changes; the integrator keeps its own positions
and calls ff.update_pos / ff.compute every step.  The system handed to the
parts is a stand-in with the reference System's attributes (numbers, pos,
natom, cell.rvecs / cell.nvec / cell.update_rvecs, charges, masses, bonds
and the neighs1..4 sets), not a yaff_gb300.System.  Checks: energies,
gradients and virials equal this package's own fused ForceField and the
reference's golden values (water64: LJ + EI + Ewald + valence with 1-2/1-3
exclusions, skin path and rebuild steps), a short MD run equals this
package's VerletIntegrator, and a cell change made on the stand-in's cell
reaches the device.
"""
import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu


class RefCell(object):
    """Stand-in for the reference Cell: rvecs, nvec, update_rvecs."""

    def __init__(self, rvecs):
        self.update_rvecs(rvecs)

    def update_rvecs(self, rvecs):
        self._rvecs = np.array(rvecs, dtype=float)

    @property
    def rvecs(self):
        return self._rvecs

    @property
    def nvec(self):
        return len(self._rvecs)


class RefSystem(object):
    """Stand-in for the reference System (yaff/system.py:50-235): the
    attributes the force field reads, with the 1-2 .. 1-4 sets derived the
    reference's way."""

    def __init__(self, numbers, pos, rvecs, charges, masses, bonds):
        self.numbers = np.asarray(numbers)
        self.pos = np.array(pos, dtype=float)
        self.natom = len(self.pos)
        self.cell = RefCell(rvecs)
        self.charges = np.array(charges, dtype=float)
        self.masses = np.array(masses, dtype=float)
        self.radii = None
        self.bonds = None if bonds is None else np.asarray(bonds)
        if self.bonds is not None:
            from yaff_gb300.system import System
            tmp = System(self.numbers, self.pos, rvecs=rvecs, bonds=self.bonds)
            self.neighs1, self.neighs2, self.neighs3, self.neighs4 = tmp.neighs1, tmp.neighs2, tmp.neighs3, tmp.neighs4


class RefForceField(object):
    """The reference ForceField's call sequence (ff.py:178-273, ForcePart
    compute semantics ff.py:117-168)."""

    def __init__(self, system, parts, nlist=None):
        self.system = system
        self.parts = list(parts)
        self.nlist = nlist
        self.needs_nlist_update = nlist is not None
        self.gpos = np.zeros((system.natom, 3))
        self.vtens = np.zeros((3, 3))

    def update_pos(self, pos):
        self.system.pos[:] = pos
        if self.nlist is not None:
            self.needs_nlist_update = True

    def update_rvecs(self, rvecs):
        self.system.cell.update_rvecs(rvecs)
        if self.nlist is not None:
            self.nlist.update_rmax()
            self.needs_nlist_update = True

    def compute(self, gpos=None, vtens=None):
        my_g = None if gpos is None else self.gpos
        my_v = None if vtens is None else self.vtens
        if my_g is not None:
            my_g[:] = 0.0
        if my_v is not None:
            my_v[:] = 0.0
        if self.needs_nlist_update:
            self.nlist.update()
            self.needs_nlist_update = False
        e = sum([part.compute(my_g, my_v) for part in self.parts])
        if gpos is not None:
            gpos += my_g
        if vtens is not None:
            vtens += my_v
        return e


def ref_verlet(ff, timestep, vel0, nstep):
    """The reference VerletIntegrator's initialize / propagate sequence
    (verlet.py:320-367); returns (epot per step, final pos, final vel)."""
    masses = ff.system.masses
    pos = ff.system.pos.copy()
    vel = vel0.copy()
    gpos = np.zeros(pos.shape)
    ff.update_pos(pos)
    epot = [ff.compute(gpos)]
    for _ in range(nstep):
        acc = -gpos / masses.reshape(-1, 1)
        vel += 0.5 * acc * timestep
        pos += timestep * vel
        ff.update_pos(pos)
        gpos[:] = 0.0
        vtens = np.zeros((3, 3))
        epot.append(ff.compute(gpos, vtens))
        acc = -gpos / masses.reshape(-1, 1)
        vel += 0.5 * acc * timestep
    return np.array(epot), pos, vel


def _parts_on(system, spec, precision):
    """The device parts of `spec` built on `system` (any object with the
    reference System's attributes), in the reference generator's order."""
    import yaff_gb300 as ygb
    from yaff_gb300.builder import make_pair_pot, PAIR_CLASSES
    ygb.set_default_precision(precision)
    try:
        nlist = ygb.NeighborList(system, skin=spec['skin'])
        scal = ygb.Scalings(system, *spec['scalings'])
        alpha = spec['ewald']['alpha']
        parts = [ygb.ForcePartPair(system, nlist, scal, make_pair_pot(p, spec, PAIR_CLASSES, None, alpha))
                 for p in spec['pair']]
        parts += [ygb.ForcePartEwaldReciprocal(system, alpha, spec['ewald']['gcut']),
                  ygb.ForcePartEwaldCorrection(system, alpha, scal), ygb.ForcePartEwaldNeutralizing(system, alpha)]
        pv = ygb.ForcePartValence(system)
        for i, j, K, r0 in spec['bond_terms']:
            pv.add_term(ygb.Harmonic(K, r0, ygb.Bond(int(i), int(j))))
        for i, j, k, K, t0 in spec['bend_terms']:
            pv.add_term(ygb.Harmonic(K, t0, ygb.BendAngle(int(i), int(j), int(k))))
        parts.append(pv)
    finally:
        ygb.set_default_precision('fp64')
    return parts, nlist


def _ref_system(spec):
    return RefSystem(np.full(len(spec['pos']), 8), spec['pos'], spec['rvecs'], spec['charges'], spec['masses'],
                     spec['bonds'])


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_reference_call_sequence_matches_golden(precision):
    spec, data = gc.load('water64')
    system = _ref_system(spec)
    parts, nlist = _parts_on(system, spec, precision)
    ff = RefForceField(system, parts, nlist)
    etol, gtol = (1e-10, 1e-9) if precision == 'fp64' else (1e-6, 1e-5)
    n = len(spec['pos'])
    for s in range(int(data['nsteps'])):
        ff.update_pos(data['step%d_pos' % s])
        g = np.zeros((n, 3))
        v = np.zeros((3, 3))
        e = ff.compute(g, v)
        scale = np.abs(data['step%d_part_energy' % s]).max()
        assert abs(e - float(data['step%d_energy' % s])) <= etol * scale
        assert gc.rel_rms(g, data['step%d_gpos' % s]) <= gtol
        assert gc.rel_rms(v, data['step%d_vtens' % s]) <= gtol
        assert nlist.nneigh == int(data['step%d_nneigh' % s])
    # the stand-in's positions are the array the device reads from
    assert ff.system.pos is parts[0].system.pos


def test_reference_call_sequence_md_matches_own_integrator():
    import yaff_gb300 as ygb
    from yaff_gb300.units import femtosecond
    from yaff_gb300.verlet import VerletIntegrator
    spec, data = gc.load('water64')
    rng = np.random.default_rng(5)
    vel0 = rng.normal(0, 1, spec['pos'].shape) * np.sqrt(300 * 3.166811563e-6 / spec['masses'])[:, None]
    system = _ref_system(spec)
    parts, nlist = _parts_on(system, spec, 'fp64')
    ep, pos, vel = ref_verlet(RefForceField(system, parts, nlist), 0.5 * femtosecond, vel0, 20)
    own = ygb.build_forcefield(spec, precision='fp64')
    e_own = []
    vi = VerletIntegrator(own, 0.5 * femtosecond, vel0=vel0.copy(), hooks=[lambda it: e_own.append(it.epot)])
    e_own.insert(0, vi.epot)
    vi.run(20)
    assert np.abs(ep - np.array(e_own)).max() <= 1e-10 * np.abs(ep).max()
    assert np.abs(pos - vi.pos).max() <= 1e-10 * np.abs(pos).max()
    assert nlist.nrebuild >= 1


def test_cell_change_on_the_standin_reaches_the_device():
    import yaff_gb300 as ygb
    spec, data = gc.load('water64')
    system = _ref_system(spec)
    parts, nlist = _parts_on(system, spec, 'fp64')
    ff = RefForceField(system, parts, nlist)
    n = len(spec['pos'])
    ff.update_pos(spec['pos'])
    ff.compute(np.zeros((n, 3)))
    rv = spec['rvecs'] * 1.01
    ff.update_rvecs(rv)
    ff.update_pos(spec['pos'] * 1.01)
    g = np.zeros((n, 3))
    e = ff.compute(g)
    spec2 = dict(spec)
    spec2['rvecs'] = rv
    spec2['pos'] = spec['pos'] * 1.01
    own = ygb.build_forcefield(spec2, precision='fp64')
    # the reference leaves the Ewald part's k-space extent (gmax) as it was
    # set up; so does the stand-in path, and the own force field built on the
    # new cell has the same extent here (a 1 % change)
    assert list(own.part_ewald_reci.gmax) == list(parts[len(spec['pair'])].gmax)
    g2 = np.zeros((n, 3))
    e2 = own.compute(g2)
    assert abs(e - e2) <= 1e-10 * abs(e2)
    assert gc.rel_rms(g, g2) <= 1e-9
