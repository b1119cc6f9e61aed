"""Velocity Verlet driving a force field through ForceField.compute, and
the thermostats of the reference.

Same integration step, initial-velocity recipe, Verlet-hook protocol (init /
pre / post, conserved-energy corrections) and conserved-quantity tracking as
the reference's VerletIntegrator (yaff/sampling/verlet.py:320-446) and
get_random_vel (yaff/sampling/utils.py:42-77): positions and velocities stay
FP64 NumPy arrays on the host; every step calls ``ff.update_pos`` and
``ff.compute(gpos, vtens)`` exactly as the reference does, so the device
force field is a drop-in for its force evaluation.  The Berendsen, Langevin,
CSVR and Nose-Hoover-chain thermostats (yaff/sampling/nvt.py:110-500) work
as host hooks of VerletIntegrator and, through ``DeviceVerlet(thermostat=)``,
inside the device-resident step; the Berendsen barostat (yaff/sampling/npt.py)
as a host hook.  The other barostats, HDF5 output and restarts are not part of
this module.
"""
import numpy as np

from .units import boltzmann, femtosecond

__all__ = ['get_random_vel', 'ConsErrTracker', 'VerletIntegrator', 'VerletHook', 'clean_momenta',
           'get_ndof_internal_md', 'get_ndof_baro', 'cell_symmetrize', 'BerendsenBarostat', 'BerendsenThermostat', 'LangevinThermostat', 'CSVRThermostat', 'NHChain',
           'NHCThermostat', 'DeviceVerlet']


def remove_com_moment(vel, masses):
    """Subtracts the centre-of-mass velocity (yaff/sampling/utils.py:80-96)."""
    com_vel = np.dot(masses, vel) / masses.sum()
    vel[:] -= com_vel


def remove_angular_moment(pos, vel, masses):
    """Subtracts the rigid rotation with the system's angular momentum about
    its centre of mass (yaff/sampling/utils.py:98-131)."""
    com = np.dot(masses, pos) / masses.sum()
    r = pos - com
    ang = (np.cross(r, vel) * masses[:, None]).sum(0)
    inert = (masses[:, None, None] * (np.eye(3)[None] * (r ** 2).sum(1)[:, None, None]
                                      - r[:, :, None] * r[:, None, :])).sum(0)
    omega = np.dot(np.linalg.pinv(inert), ang)
    vel[:] -= np.cross(omega, r)


def clean_momenta(pos, vel, masses, cell):
    """Removes the external momenta a thermostat must not touch: the COM
    velocity and, for isolated systems, the angular momentum
    (yaff/sampling/utils.py:133-158)."""
    remove_com_moment(vel, masses)
    if cell.nvec == 0:
        remove_angular_moment(pos, vel, masses)
    elif cell.nvec == 1:
        raise NotImplementedError


def get_ndof_baro(dim, anisotropic, vol_constraint):
    """Degrees of freedom of the cell (yaff/sampling/utils.py:406-428)."""
    n = dim * (dim + 1) // 2 if anisotropic else 1
    return n - 1 if vol_constraint else n


def cell_symmetrize(ff):
    """Rotates the cell (and the positions with it) so that the cell matrix
    is symmetric: rvecs @ V U^T from its singular value decomposition
    (yaff/sampling/utils.py:289-331)."""
    cell = ff.system.cell.rvecs.copy()
    U, s, Vt = np.linalg.svd(cell)
    rot_mat = np.dot(Vt.T, U.T)
    ff.update_rvecs(np.dot(cell, rot_mat))
    ff.update_pos(np.dot(ff.system.pos, rot_mat))
    return rot_mat


def get_ndof_internal_md(natom, nper):
    """Internal degrees of freedom (yaff/sampling/utils.py:259-287)."""
    if nper == 0:
        return {1: 0, 2: 1}.get(natom, 3 * natom - 6)
    if nper == 1:
        return 3 * natom - 4
    return 3 * natom - 3


def get_random_vel(temp0, scalevel0, masses, select=None, rng=None):
    """Maxwell-Boltzmann velocities at temp0, optionally rescaled so that the
    instantaneous temperature equals temp0 (the reference's recipe; a seeded
    ``rng`` replaces the global NumPy generator)."""
    if select is not None:
        masses = masses[select]
    shape = len(masses), 3
    normal = np.random.normal if rng is None else rng.normal
    result = normal(0, 1, shape) * np.sqrt(boltzmann * temp0 / masses).reshape(-1, 1)
    if scalevel0 and temp0 > 0:
        temp = (result ** 2 * masses.reshape(-1, 1)).mean() / boltzmann
        result *= np.sqrt(temp0 / temp)
    return result


class ConsErrTracker(object):
    """Running variances of the kinetic and conserved energy (Knuth's update);
    ``get()`` is sqrt(var(Econs) / var(Ekin))."""

    def __init__(self):
        self.counter = 0
        self.ekin_m = self.ekin_s = self.econs_m = self.econs_s = 0.0

    def update(self, ekin, econs):
        if self.counter == 0:
            self.ekin_m = ekin
            self.econs_m = econs
        else:
            d = ekin - self.ekin_m
            self.ekin_m += d / (self.counter + 1)
            self.ekin_s += d * (ekin - self.ekin_m)
            d = econs - self.econs_m
            self.econs_m += d / (self.counter + 1)
            self.econs_s += d * (econs - self.econs_m)
        self.counter += 1

    def get(self):
        if self.counter > 1 and self.ekin_s > 0:
            return np.sqrt(self.econs_s / self.ekin_s)
        return 0.0


class VerletHook(object):
    """A hook that acts inside the Verlet step (thermostats, barostats):
    ``init`` at initialization, ``pre`` before the first half kick, ``post``
    after the second, on the steps ``expects_call`` selects;
    ``econs_correction`` is added to the conserved energy
    (yaff/sampling/verlet.py:418-446).  ``method`` is 'thermostat' or
    'barostat' (a VerletIntegrator given one of each combines them as
    TBCombination does)."""
    device_kind = None
    method = None

    def __init__(self, start=0, step=1):
        self.start = start
        self.step = step
        self.econs_correction = 0.0

    def expects_call(self, counter):
        return counter >= self.start and (counter - self.start) % self.step == 0

    def __call__(self, iterative):
        pass

    def init(self, iterative):
        raise NotImplementedError

    def pre(self, iterative, G1_add=None):
        raise NotImplementedError

    def post(self, iterative, G1_add=None):
        raise NotImplementedError


def _normal(rng, *shape):
    """Standard normal numbers from `rng` (None: NumPy's global generator,
    as the reference draws them)."""
    return (np.random if rng is None else rng).normal(0, 1, shape if shape else None)


class BerendsenThermostat(VerletHook):
    """Weak-coupling velocity rescaling (yaff/sampling/nvt.py:110-159)."""
    method = 'thermostat'
    device_kind = 1

    def __init__(self, temp, start=0, timecon=100 * femtosecond, restart=False):
        self.temp = temp
        self.timecon = timecon
        self.restart = restart
        VerletHook.__init__(self, start, 1)

    def init(self, iterative):
        if not self.restart:
            clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.ff.system.cell)
        if iterative.ndof is None:
            iterative.ndof = get_ndof_internal_md(iterative.pos.shape[0], iterative.ff.system.cell.nvec)

    def pre(self, iterative, G1_add=None):
        ekin = iterative.ekin
        temp_inst = 2.0 * iterative.ekin / (boltzmann * iterative.ndof)
        c = np.sqrt(1 + iterative.timestep / self.timecon * (self.temp / temp_inst - 1))
        iterative.vel[:] = c * iterative.vel
        iterative.ekin = iterative._compute_ekin()
        self.econs_correction += (1 - c ** 2) * ekin

    def post(self, iterative, G1_add=None):
        pass


class LangevinThermostat(VerletHook):
    """Ornstein-Uhlenbeck velocity update for half a step before and after
    each Verlet step (Bussi and Parrinello, Phys. Rev. E 75, 056707 (2007);
    yaff/sampling/nvt.py:162-213)."""
    method = 'thermostat'
    device_kind = 2

    def __init__(self, temp, start=0, timecon=100 * femtosecond, rng=None):
        self.temp = temp
        self.timecon = timecon
        self.rng = rng
        VerletHook.__init__(self, start, 1)

    def init(self, iterative):
        clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.ff.system.cell)

    def pre(self, iterative, G1_add=None):
        ekin0 = iterative.ekin
        self.thermo(iterative)
        self.econs_correction += ekin0 - iterative.ekin

    def post(self, iterative, G1_add=None):
        ekin0 = iterative.ekin
        self.thermo(iterative)
        self.econs_correction += ekin0 - iterative.ekin

    def thermo(self, iterative):
        c1 = np.exp(-iterative.timestep / self.timecon / 2)
        c2 = np.sqrt((1.0 - c1 ** 2) * self.temp * boltzmann / iterative.masses).reshape(-1, 1)
        iterative.vel[:] = c1 * iterative.vel + c2 * _normal(self.rng, *iterative.vel.shape)
        iterative.ekin = iterative._compute_ekin()


class CSVRThermostat(VerletHook):
    """Canonical sampling through velocity rescaling (Bussi, Donadio and
    Parrinello, J. Chem. Phys. 126, 014101 (2007); yaff/sampling/nvt.py:
    215-268)."""
    method = 'thermostat'
    device_kind = 3

    def __init__(self, temp, start=0, timecon=100 * femtosecond, rng=None):
        self.temp = temp
        self.timecon = timecon
        self.rng = rng
        VerletHook.__init__(self, start, 1)

    def init(self, iterative):
        clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.ff.system.cell)
        if iterative.ndof is None:
            iterative.ndof = get_ndof_internal_md(iterative.pos.shape[0], iterative.ff.system.cell.nvec)
        self.kin = 0.5 * iterative.ndof * boltzmann * self.temp

    def pre(self, iterative, G1_add=None):
        c = np.exp(-iterative.timestep / self.timecon)
        R = _normal(self.rng)
        S = (_normal(self.rng, iterative.ndof - 1) ** 2).sum()
        iterative.ekin = iterative._compute_ekin()
        fact = (1 - c) * self.kin / iterative.ndof / iterative.ekin
        alpha = np.sign(R + np.sqrt(c / fact)) * np.sqrt(c + (S + R ** 2) * fact + 2 * R * np.sqrt(c * fact))
        iterative.vel[:] = alpha * iterative.vel
        ekin_new = alpha ** 2 * iterative.ekin
        self.econs_correction += (1 - alpha ** 2) * iterative.ekin
        iterative.ekin = ekin_new

    def post(self, iterative, G1_add=None):
        pass


class NHChain(object):
    """Nose-Hoover chain of `length` beads with masses from the time
    constant; one call propagates it over half a step and rescales the
    atomic velocities (Martyna, Tuckerman, Tobias and Klein, Mol. Phys. 87,
    1117 (1996); yaff/sampling/nvt.py:346-427)."""

    def __init__(self, length, timestep, temp, ndof, pos0, vel0, timecon=100 * femtosecond, rng=None):
        self.length = length
        self.timestep = timestep
        self.temp = temp
        self.timecon = timecon
        self.rng = rng
        self.restart_pos = pos0 is not None
        self.restart_vel = vel0 is not None
        self.pos = np.array(pos0, float) if self.restart_pos else np.zeros(length)
        self.vel = np.array(vel0, float) if self.restart_vel else np.zeros(length)
        if ndof > 0:
            self.set_ndof(ndof)

    def set_ndof(self, ndof):
        self.ndof = ndof
        angfreq = 2 * np.pi / self.timecon
        self.masses = np.ones(self.length) * (boltzmann * self.temp / angfreq ** 2)
        self.masses[0] *= ndof
        if not self.restart_vel:
            self.vel = self.get_random_vel_therm()

    def get_random_vel_therm(self):
        return _normal(self.rng, self.length) * np.sqrt(self.masses * boltzmann * self.temp) / self.masses

    def __call__(self, ekin, vel, G1_add):
        def do_bead(k, ekin):
            if k == 0:
                g = 2 * ekin - self.ndof * self.temp * boltzmann
                if G1_add is not None:
                    g += G1_add
            else:
                g = self.masses[k - 1] * self.vel[k - 1] ** 2 - self.temp * boltzmann
            g /= self.masses[k]
            if k == self.length - 1:
                self.vel[k] += g * self.timestep / 4
            else:
                self.vel[k] *= np.exp(-self.vel[k + 1] * self.timestep / 8)
                self.vel[k] += g * self.timestep / 4
                self.vel[k] *= np.exp(-self.vel[k + 1] * self.timestep / 8)

        for k in range(self.length - 1, -1, -1):
            do_bead(k, ekin)
        self.pos += self.vel * self.timestep / 2
        factor = np.exp(-self.vel[0] * self.timestep / 2)
        vel *= factor
        ekin *= factor ** 2
        for k in range(0, self.length):
            do_bead(k, ekin)
        return vel, ekin

    def get_econs_correction(self):
        kt = boltzmann * self.temp
        return 0.5 * (self.vel ** 2 * self.masses).sum() + kt * (self.ndof * self.pos[0] + self.pos[1:].sum())


class NHCThermostat(VerletHook):
    """Nose-Hoover chain thermostat (Martyna, Klein and Tuckerman, J. Chem.
    Phys. 97, 2635 (1992); yaff/sampling/nvt.py:430-498)."""
    method = 'thermostat'
    device_kind = 4

    def __init__(self, temp, start=0, timecon=100 * femtosecond, chainlength=3, chain_pos0=None, chain_vel0=None,
                 restart=False, rng=None):
        self.temp = temp
        self.restart = restart
        self.chain = NHChain(chainlength, 0.0, temp, 0, chain_pos0, chain_vel0, timecon, rng)
        VerletHook.__init__(self, start, 1)

    def init(self, iterative):
        if not self.restart:
            clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.ff.system.cell)
        if iterative.ndof is None:
            iterative.ndof = get_ndof_internal_md(iterative.pos.shape[0], iterative.ff.system.cell.nvec)
        self.chain.timestep = iterative.timestep
        self.chain.set_ndof(iterative.ndof)

    def pre(self, iterative, G1_add=None):
        vel_new, iterative.ekin = self.chain(iterative.ekin, iterative.vel, G1_add)
        iterative.vel[:] = vel_new

    def post(self, iterative, G1_add=None):
        vel_new, iterative.ekin = self.chain(iterative.ekin, iterative.vel, G1_add)
        iterative.vel[:] = vel_new
        self.econs_correction = self.chain.get_econs_correction()


class BerendsenBarostat(VerletHook):
    """Weak-coupling cell rescaling towards the pressure `press`: after each
    step positions and cell are multiplied by mu = 1 - dt/W (P0 - P) (made
    symmetric; isotropic unless `anisotropic`), the forces are evaluated
    again, and the energy change goes into the conserved-energy correction
    (Berendsen et al., J. Chem. Phys. 81, 3684 (1984); yaff/sampling/npt.py:
    232-330).  A host hook: each step makes one extra force evaluation at the
    rescaled cell, through ForceField.update_rvecs."""
    method = 'barostat'

    def __init__(self, ff, temp, press, start=0, step=1, timecon=1000 * femtosecond, beta=None,
                 anisotropic=True, vol_constraint=False, restart=False):
        from .units import bar
        self.temp = temp
        self.press = press
        self.timecon_press = timecon
        self.beta = 4.57e-5 / bar if beta is None else beta
        self.mass_press = 3.0 * timecon / self.beta
        self.anisotropic = anisotropic
        self.vol_constraint = vol_constraint
        self.dim = ff.system.cell.nvec
        self.baro_ndof = get_ndof_baro(self.dim, self.anisotropic, self.vol_constraint)
        if self.anisotropic:
            cell_symmetrize(ff)
        self.cell = ff.system.cell.rvecs.copy()
        self.restart = restart
        VerletHook.__init__(self, start, step)

    def init(self, iterative):
        self.timestep_press = iterative.timestep
        if not self.restart:
            clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.ff.system.cell)
        iterative.gpos[:] = 0.0
        iterative.vtens[:] = 0.0
        iterative.epot = iterative.ff.compute(iterative.gpos, iterative.vtens)
        if iterative.ndof is None:
            iterative.ndof = get_ndof_internal_md(iterative.pos.shape[0], iterative.ff.system.cell.nvec)
        self.mass_press *= np.sqrt(iterative.ndof)

    def pre(self, iterative, G1_add=None):
        pass

    def post(self, iterative, G1_add=None):
        epot0 = iterative.epot
        ptens = (np.dot(iterative.vel.T * iterative.masses, iterative.vel) - iterative.vtens) / \
            iterative.ff.system.cell.volume
        dmu = self.timestep_press / self.mass_press * (self.press * np.eye(3) - ptens)
        if self.vol_constraint:
            dmu -= np.trace(dmu) / self.dim * np.eye(self.dim)
        mu = np.eye(3) - dmu
        mu = 0.5 * (mu + mu.T)
        if not self.anisotropic:
            mu = ((np.trace(mu) / 3.0) ** (1.0 / 3.0)) * np.eye(3)
        pos_new = np.dot(iterative.pos, mu)
        rvecs_new = np.dot(iterative.rvecs, mu)
        iterative.ff.update_pos(pos_new)
        iterative.pos[:] = pos_new
        iterative.ff.update_rvecs(rvecs_new)
        iterative.rvecs[:] = rvecs_new
        iterative.gpos[:] = 0.0
        iterative.vtens[:] = 0.0
        iterative.epot = iterative.ff.compute(iterative.gpos, iterative.vtens)
        self.econs_correction += epot0 - iterative.epot


def get_random_vel_press(mass, temp, rng=None):
    """Symmetric 3x3 barostat velocity drawn from the Maxwell-Boltzmann
    distribution of a cell mass `mass` at `temp` (off-diagonal entries
    divided by sqrt(2): p_ab = p_ba is one degree of freedom)
    (yaff/sampling/utils.py:378-403)."""
    rand = (np.random if rng is None else rng).normal(0, np.sqrt(mass * boltzmann * temp), (3, 3)) / mass
    vel_press = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            vel_press[i, j] = rand[i, j] if i >= j else rand[j, i]
            if i != j:
                vel_press[i, j] /= np.sqrt(2)
    return vel_press


def _cell_propagate(iterative, vel_press, timestep, anisotropic, vol_constraint):
    """The barostat's position, cell and velocity propagation around the
    forces at the new cell: iL v_g h/2 on positions and cell vectors, a new
    force evaluation, then -iL (v_g + Tr(v_g)/ndof) h/2 on the velocities
    (yaff/sampling/npt.py:435-478, :642-688; Martyna, Tuckerman, Tobias and
    Klein, Mol. Phys. 87, 1117 (1996))."""
    if anisotropic:
        dr, qg = np.linalg.eigh(vel_press)
        rot = np.dot(np.dot(qg, np.diagflat(np.exp(dr * timestep / 2))), qg.T)
        pos_new = np.dot(iterative.pos, rot)
        rvecs_new = np.dot(iterative.rvecs, rot)
    else:
        c = np.exp(vel_press * timestep / 2)
        pos_new = c * iterative.pos
        rvecs_new = c * iterative.rvecs
    iterative.ff.update_pos(pos_new)
    iterative.pos[:] = pos_new
    iterative.ff.update_rvecs(rvecs_new)
    iterative.rvecs[:] = rvecs_new
    iterative.gpos[:] = 0.0
    iterative.vtens[:] = 0.0
    iterative.epot = iterative.ff.compute(iterative.gpos, iterative.vtens)
    if anisotropic:
        if vol_constraint:
            dg, eg = np.linalg.eigh(vel_press)
        else:
            dg, eg = np.linalg.eigh(vel_press + (np.trace(vel_press) / iterative.ndof) * np.eye(3))
        rot = np.dot(np.dot(eg, np.diagflat(np.exp(-dg * timestep / 2))), eg.T)
        vel_new = np.dot(iterative.vel, rot)
    else:
        vel_new = np.exp(-((1.0 + 3.0 / iterative.ndof) * vel_press) * timestep / 2) * iterative.vel
    iterative.vel[:] = vel_new
    iterative.ekin = iterative._compute_ekin()


def _press_force(iterative, press, mass_press):
    """G = (P_int V + (2 Ekin/ndof - P V) 1) / W, with P_int V the symmetrized
    kinetic minus virial tensor."""
    ptens_vol = np.dot(iterative.vel.T * iterative.masses, iterative.vel) - iterative.vtens
    ptens_vol = 0.5 * (ptens_vol.T + ptens_vol)
    vol = iterative.ff.system.cell.volume
    return (ptens_vol + (2.0 * iterative.ekin / iterative.ndof - press * vol) * np.eye(3)) / mass_press


class LangevinBarostat(VerletHook):
    """Langevin piston barostat (Feller, Zhang, Pastor and Brooks, J. Chem.
    Phys. 103, 4613 (1995); yaff/sampling/npt.py:333-512): the cell velocity
    tensor feels the pressure difference, a friction 1/timecon and random
    forces; positions, cell and velocities follow it as in the MTK
    propagator.  Host hook; random numbers from `rng` (None: NumPy's global
    generator, in the reference's call order)."""
    method = 'barostat'

    def __init__(self, ff, temp, press, start=0, step=1, timecon=1000 * femtosecond, anisotropic=True,
                 vol_constraint=False, rng=None):
        self.temp = temp
        self.press = press
        self.timecon = timecon
        self.anisotropic = anisotropic
        self.vol_constraint = vol_constraint
        self.rng = rng
        self.dim = ff.system.cell.nvec
        self.baro_ndof = get_ndof_baro(self.dim, self.anisotropic, self.vol_constraint)
        if self.anisotropic:
            cell_symmetrize(ff)
        self.cell = ff.system.cell.rvecs.copy()
        VerletHook.__init__(self, start, step)

    def init(self, iterative):
        self.timestep_press = iterative.timestep
        clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.ff.system.cell)
        if iterative.ndof is None:
            iterative.ndof = iterative.pos.size
        self.mass_press = (iterative.ndof + 3) / 3 * boltzmann * self.temp * (self.timecon / (2 * np.pi)) ** 2
        self.vel_press = get_random_vel_press(self.mass_press, self.temp, self.rng)
        if self.vol_constraint:
            self.vel_press -= np.trace(self.vel_press) / 3 * np.eye(3)
        if not self.anisotropic:
            self.vel_press = self.vel_press[0][0]
        iterative.gpos[:] = 0.0
        iterative.vtens[:] = 0.0
        iterative.epot = iterative.ff.compute(iterative.gpos, iterative.vtens)

    def pre(self, iterative, chainvel0=None):
        epot0, ekin0 = iterative.epot, iterative.ekin
        self.baro(iterative, chainvel0)
        self.econs_correction += epot0 - iterative.epot + ekin0 - iterative.ekin

    def post(self, iterative, chainvel0=None):
        epot0, ekin0 = iterative.epot, iterative.ekin
        self.baro(iterative, chainvel0)
        self.econs_correction += epot0 - iterative.epot + ekin0 - iterative.ekin

    def baro(self, iterative, chainvel0):
        def update_baro_vel():
            self.vel_press *= np.exp(-self.timestep_press / (8 * self.timecon))
            if chainvel0 is not None:
                self.vel_press *= np.exp(-self.timestep_press * chainvel0 / 8)
            g = _press_force(iterative, self.press, self.mass_press)
            r = self.getR()
            if self.vol_constraint:
                g -= np.trace(g) / self.dim * np.eye(self.dim)
                r -= np.trace(r) / self.dim * np.eye(self.dim)
            if not self.anisotropic:
                g = np.trace(g)
                r = r[0][0]
            self.vel_press += (g - r / self.mass_press) * self.timestep_press / 4
            self.vel_press *= np.exp(-self.timestep_press / (8 * self.timecon))
            if chainvel0 is not None:
                self.vel_press *= np.exp(-self.timestep_press * chainvel0 / 8)

        update_baro_vel()
        _cell_propagate(iterative, self.vel_press, self.timestep_press, self.anisotropic, self.vol_constraint)
        update_baro_vel()

    def getR(self):
        """Symmetric random force tensor of the piston."""
        rand = (np.random if self.rng is None else self.rng).normal(0, 1, (3, 3)) * \
            np.sqrt(2 * self.mass_press * boltzmann * self.temp / (self.timestep_press * self.timecon))
        r = np.zeros((3, 3))
        for i in range(3):
            for j in range(3):
                r[i, j] = rand[i, j] if i >= j else rand[j, i]
        return r


class MTKBarostat(VerletHook):
    """Martyna-Tobias-Klein barostat (J. Chem. Phys. 101, 4177 (1994)) with
    the symplectic propagator of Martyna, Tuckerman, Tobias and Klein (Mol.
    Phys. 87, 1117 (1996)); yaff/sampling/npt.py:514-729.  Deterministic;
    `baro_thermo` (an NHCThermostat) thermostats the cell velocity itself.
    Host hook."""
    method = 'barostat'

    def __init__(self, ff, temp, press, start=0, step=1, timecon=1000 * femtosecond, anisotropic=True,
                 vol_constraint=False, baro_thermo=None, vel_press0=None, restart=False, rng=None):
        self.temp = temp
        self.press = press
        self.timecon_press = timecon
        self.anisotropic = anisotropic
        self.vol_constraint = vol_constraint
        self.baro_thermo = baro_thermo
        self.rng = rng
        self.dim = ff.system.cell.nvec
        self.restart = restart
        self.baro_ndof = get_ndof_baro(self.dim, self.anisotropic, self.vol_constraint)
        if self.anisotropic and not self.restart:
            cell_symmetrize(ff)
        self.cell = ff.system.cell.rvecs.copy()
        self.vel_press = vel_press0
        VerletHook.__init__(self, start, step)

    def init(self, iterative):
        self.timestep_press = iterative.timestep
        if not self.restart:
            clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.ff.system.cell)
        if iterative.ndof is None:
            iterative.ndof = get_ndof_internal_md(len(iterative.pos), iterative.ff.system.cell.nvec)
        angfreq = 2 * np.pi / self.timecon_press
        self.mass_press = (iterative.ndof + self.dim ** 2) * boltzmann * self.temp / angfreq ** 2
        if self.vel_press is None:
            self.vel_press = get_random_vel_press(self.mass_press, self.temp, self.rng)
            if not self.anisotropic:
                self.vel_press = self.vel_press[0][0]
        if self.baro_thermo is not None:
            self.baro_thermo.chain.timestep = iterative.timestep
            self.baro_thermo.chain.set_ndof(self.baro_ndof)
        if self.vol_constraint:
            self.vel_press -= np.trace(self.vel_press) / 3 * np.eye(3)
        iterative.gpos[:] = 0.0
        iterative.vtens[:] = 0.0
        iterative.epot = iterative.ff.compute(iterative.gpos, iterative.vtens)

    def _thermostat_cell(self):
        # the cell thermostat sees the cell kinetic energy; v_g itself is
        # updated in baro()
        vel_copy = np.zeros(np.shape(self.vel_press))
        vel_copy[...] = self.vel_press
        self.baro_thermo.chain(self._compute_ekin_baro(), vel_copy, 0)

    def pre(self, iterative, chainvel0=None):
        if self.baro_thermo is not None:
            chainvel0 = self.baro_thermo.chain.vel[0]
        self.baro(iterative, chainvel0)
        if self.baro_thermo is not None:
            self._thermostat_cell()

    def post(self, iterative, chainvel0=None):
        if self.baro_thermo is not None:
            self._thermostat_cell()
            chainvel0 = self.baro_thermo.chain.vel[0]
        self.baro(iterative, chainvel0)
        self.econs_correction = self._compute_ekin_baro()
        if not self.vol_constraint:
            self.econs_correction += self.press * iterative.ff.system.cell.volume
        if self.baro_thermo is not None:
            self.econs_correction += self.baro_thermo.chain.get_econs_correction()

    def baro(self, iterative, chainvel0):
        def update_baro_vel():
            if chainvel0 is not None:
                self.vel_press *= np.exp(-self.timestep_press * chainvel0 / 8)
            g = _press_force(iterative, self.press, self.mass_press)
            if not self.anisotropic:
                g = np.trace(g)
            if self.vol_constraint:
                g -= np.trace(g) / self.dim * np.eye(self.dim)
            self.vel_press += g * self.timestep_press / 4
            if chainvel0 is not None:
                self.vel_press *= np.exp(-self.timestep_press * chainvel0 / 8)

        update_baro_vel()
        _cell_propagate(iterative, self.vel_press, self.timestep_press, self.anisotropic, self.vol_constraint)
        update_baro_vel()

    def add_press_cont(self):
        """The cell's contribution to the first chain bead's force of a
        particle Nose-Hoover chain (zero when the cell has its own chain)."""
        if self.baro_thermo is None:
            return 2 * self._compute_ekin_baro() - self.baro_ndof * self.temp * boltzmann
        return 0

    def _compute_ekin_baro(self):
        if self.anisotropic:
            return 0.5 * self.mass_press * np.trace(np.dot(self.vel_press.T, self.vel_press))
        return 0.5 * self.mass_press * self.vel_press ** 2


class TBCombination(VerletHook):
    """A thermostat and a barostat called in the reference's succession with
    their coupling (yaff/sampling/npt.py:45-157): the barostat first in
    ``pre`` and last in ``post``; with a Nose-Hoover chain the first bead's
    velocity scales the cell velocity; with an MTK barostat the cell's
    kinetic energy enters the chain's first bead."""

    def __init__(self, thermostat, barostat, start=0):
        if thermostat.method != 'thermostat':
            thermostat, barostat = barostat, thermostat
        if thermostat.method != 'thermostat' or barostat.method != 'barostat':
            raise TypeError('TBCombination needs one thermostat and one barostat')
        self.thermostat = thermostat
        self.barostat = barostat
        self.step_thermo = thermostat.step
        self.step_baro = barostat.step
        VerletHook.__init__(self, start, min(self.step_thermo, self.step_baro))

    def init(self, iterative):
        set_ndof = iterative.ndof is not None
        self.thermostat.init(iterative)
        self.barostat.init(iterative)
        p_cm_fluct = isinstance(self.thermostat, LangevinThermostat) or isinstance(self.barostat, LangevinBarostat)
        if (not set_ndof) and p_cm_fluct:
            iterative.ndof = iterative.pos.size
        self.chainvel0 = None
        self.G1_add = None

    def pre(self, iterative, G1_add=None):
        if self._expects(iterative, self.step_baro):
            if isinstance(self.thermostat, NHCThermostat):
                self.chainvel0 = self.thermostat.chain.vel[0]
            self.barostat.pre(iterative, self.chainvel0)
        if self._expects(iterative, self.step_thermo):
            if isinstance(self.barostat, MTKBarostat):
                self.G1_add = self.barostat.add_press_cont()
            self.thermostat.pre(iterative, self.G1_add)

    def post(self, iterative, G1_add=None):
        if self._expects(iterative, self.step_thermo):
            if isinstance(self.barostat, MTKBarostat):
                self.G1_add = self.barostat.add_press_cont()
            self.thermostat.post(iterative, self.G1_add)
        if self._expects(iterative, self.step_baro):
            if isinstance(self.thermostat, NHCThermostat):
                self.chainvel0 = self.thermostat.chain.vel[0]
            self.barostat.post(iterative, self.chainvel0)
        self.econs_correction = self.thermostat.econs_correction + self.barostat.econs_correction
        if isinstance(self.thermostat, NHCThermostat) and not (
                isinstance(self.barostat, MTKBarostat) and self.barostat.baro_thermo is not None):
            # the particle chain also thermostats the cell
            self.econs_correction += self.barostat.baro_ndof * boltzmann * self.thermostat.temp * \
                self.thermostat.chain.pos[0]

    def _expects(self, iterative, step):
        return iterative.counter >= self.start and (iterative.counter - self.start) % step == 0


def _combine_hooks(hooks):
    """A thermostat and a barostat given as separate hooks are replaced by
    their TBCombination (appended last), as the reference's integrator does
    (yaff/sampling/verlet.py:205-233)."""
    thermo = [h for h in hooks if getattr(h, 'method', None) == 'thermostat']
    baro = [h for h in hooks if getattr(h, 'method', None) == 'barostat']
    if thermo and baro:
        hooks = [h for h in hooks if h is not thermo[0] and h is not baro[0]]
        hooks.append(TBCombination(thermo[0], baro[0]))
    return hooks


class VerletIntegrator(object):
    """Velocity Verlet with the reference's hook protocol.

    ff: object with ``system`` (pos, masses, cell), ``update_pos`` and
    ``compute(gpos, vtens)``.  vel0: initial velocities (default: seeded
    Maxwell-Boltzmann at temp0).  hooks: VerletHook objects (thermostats,
    called before and after the Verlet step) and plain callables
    f(integrator), called after every step.  ndof: degrees of freedom (None:
    set by a thermostat's init, else 3 N).
    """

    def __init__(self, ff, timestep=None, vel0=None, temp0=300.0, scalevel0=True, hooks=None, rng=None, ndof=None,
                 restart=None):
        self.ff = ff
        state = None
        if restart is not None:
            # continue from a RestartWriter state (the reference's restart_h5,
            # yaff/sampling/verlet.py:113-142): positions and cell always,
            # velocities and time step unless given
            from .io import read_restart
            state = read_restart(restart) if isinstance(restart, str) else restart
            cell = getattr(ff.system, 'cell', None)
            rv = np.asarray(state['rvecs'])
            if cell is not None and rv.size and not np.array_equal(rv, cell.rvecs):
                ff.update_rvecs(rv)
            ff.system.pos[:] = state['pos']
            if vel0 is None:
                vel0 = state['vel']
            if timestep is None:
                timestep = float(state['timestep'])
        if timestep is None:
            raise AssertionError('No Verlet timestep is found')
        self.timestep = timestep
        system = ff.system
        self.pos = system.pos.copy()
        self.masses = np.asarray(system.masses, dtype=np.float64)
        cell = getattr(system, 'cell', None)
        self.rvecs = cell.rvecs.copy() if cell is not None and cell.nvec > 0 else None
        if vel0 is None:
            vel0 = get_random_vel(temp0, scalevel0, self.masses, rng=rng)
        self.vel = np.array(vel0, dtype=np.float64)
        self.gpos = np.zeros(self.pos.shape)
        self.vtens = np.zeros((3, 3))
        if hooks is not None and not isinstance(hooks, (list, tuple)):
            hooks = [hooks]
        self.hooks = _combine_hooks(list(hooks or []))
        self.ndof = ndof
        self.time = 0.0
        self.counter = 0
        self.cons_err = ConsErrTracker()
        if state is not None:
            for hook in self.hooks:
                if isinstance(hook, VerletHook) and hasattr(hook, 'restart'):
                    hook.restart = True   # no momentum cleaning on a restart
        self.initialize()
        if state is not None:
            self._restore(state)

    def _restore(self, state):
        """Counter, time, thermostat states and the conserved-energy tracker
        of a restart record (after initialize, which recomputed the forces
        at the restored positions)."""
        self.counter = int(state['counter'])
        self.time = float(state['time'])
        vhooks = [h for h in self.hooks if isinstance(h, VerletHook)]
        corr = np.asarray(state.get('hook_econs_correction', np.zeros(0)))
        for k, hook in enumerate(vhooks):
            if k < len(corr):
                hook.econs_correction = float(corr[k])
            chain = getattr(hook, 'chain', None)
            if chain is not None and ('hook%d_chain_pos' % k) in state:
                chain.pos[:] = state['hook%d_chain_pos' % k]
                chain.vel[:] = state['hook%d_chain_vel' % k]
                hook.econs_correction = chain.get_econs_correction()
        if 'cons_err' in state:
            c = state['cons_err']
            self.cons_err.counter = int(c[0])
            self.cons_err.ekin_m, self.cons_err.ekin_s, self.cons_err.econs_m, self.cons_err.econs_s = (
                float(c[1]), float(c[2]), float(c[3]), float(c[4]))
        self.ekin = self._compute_ekin()
        self.temp = self.ekin / self.ndof * 2.0 / boltzmann
        self.etot = self.ekin + self.epot
        self.econs = self.etot + self.econs_correction

    def _verlet_hooks(self, kind):
        for hook in self.hooks:
            if isinstance(hook, VerletHook) and (kind == 'init' or hook.expects_call(self.counter)):
                getattr(hook, kind)(self)

    def _compute_ekin(self):
        return 0.5 * (self.vel ** 2 * self.masses.reshape(-1, 1)).sum()

    @property
    def econs_correction(self):
        return sum(h.econs_correction for h in self.hooks if isinstance(h, VerletHook))

    def compute_properties(self):
        self.ekin = self._compute_ekin()
        self.temp = self.ekin / self.ndof * 2.0 / boltzmann
        self.etot = self.ekin + self.epot
        self.econs = self.etot + self.econs_correction
        self.cons_err.update(self.ekin, self.econs)

    def initialize(self):
        self.gpos[:] = 0.0
        self.ff.update_pos(self.pos)
        self.epot = self.ff.compute(self.gpos)
        self.acc = -self.gpos / self.masses.reshape(-1, 1)
        self._verlet_hooks('init')
        if self.ndof is None:
            self.ndof = self.pos.size
        self.compute_properties()

    def propagate(self):
        self._verlet_hooks('pre')
        self.acc = -self.gpos / self.masses.reshape(-1, 1)
        self.vel += 0.5 * self.acc * self.timestep
        self.pos += self.timestep * self.vel
        self.ff.update_pos(self.pos)
        self.gpos[:] = 0.0
        self.vtens[:] = 0.0
        self.epot = self.ff.compute(self.gpos, self.vtens)
        self.acc = -self.gpos / self.masses.reshape(-1, 1)
        self.vel += 0.5 * self.acc * self.timestep
        self.ekin = self._compute_ekin()
        self._verlet_hooks('post')
        self.time += self.timestep
        self.counter += 1
        self.compute_properties()
        for hook in self.hooks:
            if not isinstance(hook, VerletHook):
                hook(self)

    def run(self, nstep):
        for _ in range(nstep):
            self.propagate()


def drift_per_ps(times, econs, natom):
    """Slope of a linear fit of the conserved energy, per atom and per ps
    (hartree / atom / ps; times in atomic units)."""
    from .units import picosecond
    t = np.asarray(times) / picosecond
    a = np.polyfit(t, np.asarray(econs), 1)[0]
    return a / natom


class DeviceVerlet(object):
    """Velocity Verlet with positions, velocities, masses and the neighbour
    list resident in HBM (yg_md_* of libyaffgb.so); NVE, or NVT with
    ``thermostat`` a BerendsenThermostat, LangevinThermostat, CSVRThermostat
    or NHCThermostat (its init runs on the host, its pre / post updates in
    the device step; the stochastic ones draw from a counter-based generator
    keyed by ``seed``, not from NumPy).

    The same step as VerletIntegrator (yaff/sampling/verlet.py:339-367) and
    the same skin rule for rebuilding the list (yaff/pes/nlist.py:207-218),
    but the host only reads one scalar per step (the largest displacement
    since the last rebuild); the force evaluation and the second half kick
    are replayed from a CUDA graph when ``use_graph`` is set.  ``ff`` must run
    entirely on the fused device path (ForceField.device_md_terms).  The
    energy log holds (epot, ekin) of step 0 and of every step run since.
    """

    def __init__(self, ff, timestep=None, vel0=None, temp0=300.0, scalevel0=True, rng=None, max_steps=1000,
                 use_graph=True, thermostat=None, seed=0, ndof=None, restart=None):
        from . import _lib
        from ._lib import check, ptr
        self._lib, self._check, self._ptr = _lib, check, ptr
        self.ff = ff
        system = ff.system
        # continue from a restart record (RestartWriter / save_restart):
        # positions, cell, velocities, counter, time step, thermostat state
        self.counter0 = 0
        self.econs_offset = 0.0
        if restart is not None:
            from .io import read_restart
            state = read_restart(restart) if isinstance(restart, str) else restart
            rv = np.asarray(state['rvecs'])
            if rv.size and not np.array_equal(rv, system.cell.rvecs):
                ff.update_rvecs(rv)
            system.pos[:] = state['pos']
            if vel0 is None:
                vel0 = state['vel']
            if timestep is None:
                timestep = float(state['timestep'])
            self.counter0 = int(state['counter'])
            if thermostat is not None:
                thermostat.restart = True
                corr = np.asarray(state.get('hook_econs_correction', np.zeros(0)))
                if getattr(thermostat, 'device_kind', None) == 4 and 'hook0_chain_pos' in state:
                    thermostat.chain.pos[:] = state['hook0_chain_pos']
                    thermostat.chain.vel[:] = state['hook0_chain_vel']
                    thermostat.chain.restart_pos = thermostat.chain.restart_vel = True
                elif len(corr):
                    # the accumulated correction of the weak-coupling and
                    # stochastic thermostats continues from the saved value
                    self.econs_offset = float(corr[0])
                # a fresh noise stream for the continued run
                seed = (int(seed) * 0x9E3779B1 + self.counter0) & 0xFFFFFFFFFFFF
        if timestep is None:
            raise AssertionError('No Verlet timestep is found')
        self.timestep = float(timestep)
        self.use_graph = bool(use_graph)
        self.natom = system.natom
        self.masses = np.ascontiguousarray(system.masses, dtype=np.float64)
        if vel0 is None:
            vel0 = get_random_vel(temp0, scalevel0, self.masses, rng=rng)
        vel0 = np.array(vel0, dtype=np.float64, order='C')
        # one evaluation through the fused path builds the list and uploads
        # every parameter the device step needs
        ff.update_pos(system.pos)
        ff.compute(np.zeros((self.natom, 3)))
        self.thermostat = thermostat
        self.ndof = ndof
        if thermostat is not None:
            # the thermostat's own init on the host (momenta, degrees of
            # freedom, chain), as the reference's VerletIntegrator calls it
            self.pos, self.vel, self.ekin = system.pos.copy(), vel0, None
            self.ekin = self._compute_ekin()
            thermostat.init(self)
            if self.ndof is None:
                self.ndof = get_ndof_internal_md(self.natom, system.cell.nvec)
            vel0 = np.ascontiguousarray(self.vel)
        self.dev, self.mask, self.const_energy = ff.device_md_terms()
        self.skin = float(ff.nlist.skin) if ff.nlist is not None else 0.0
        self.max_steps = int(max_steps)
        check(self.dev.lib.yg_md_setup(self.dev.ctx, ptr(self.masses), ptr(vel0), self.timestep, self.mask,
                                       self.const_energy, self.max_steps), 'yg_md_setup')
        if thermostat is not None:
            kind = thermostat.device_kind
            if kind is None:
                raise NotImplementedError('%s has no device form' % type(thermostat).__name__)
            timecon = thermostat.chain.timecon if kind == 4 else thermostat.timecon
            nc = thermostat.chain.length if kind == 4 else 0
            cp = np.ascontiguousarray(thermostat.chain.pos, float) if kind == 4 else None
            cv = np.ascontiguousarray(thermostat.chain.vel, float) if kind == 4 else None
            cm = np.ascontiguousarray(thermostat.chain.masses, float) if kind == 4 else None
            check(self.dev.lib.yg_md_thermostat(self.dev.ctx, kind, boltzmann * thermostat.temp, float(timecon),
                                                int(self.ndof), nc, ptr(cp), ptr(cv), ptr(cm), int(seed)),
                  'yg_md_thermostat')
        self.counter = 0
        self.nrebuild = 0

    def _compute_ekin(self):
        return 0.5 * (self.vel ** 2 * self.masses.reshape(-1, 1)).sum()

    def thermo_state(self):
        """(conserved-energy correction, chain positions, chain velocities)
        of the device thermostat."""
        import ctypes
        e = ctypes.c_double()
        n = self.thermostat.chain.length if getattr(self.thermostat, 'device_kind', None) == 4 else 0
        cp, cv = np.zeros(n), np.zeros(n)
        self._check(self.dev.lib.yg_md_thermo_get(self.dev.ctx, ctypes.byref(e), self._ptr(cp), self._ptr(cv)),
                    'yg_md_thermo_get')
        return e.value, cp, cv

    def run(self, nstep):
        import ctypes
        nreb = ctypes.c_int64()
        self._check(self.dev.lib.yg_md_run(self.dev.ctx, int(nstep), int(self.use_graph), self.skin,
                                           ctypes.byref(nreb)), 'yg_md_run')
        self.counter += int(nstep)
        self.nrebuild += nreb.value

    def fetch(self, pos=True, vel=True):
        """(pos, vel, log) on the host; log is (counter + 1) x (epot, ekin)."""
        import ctypes
        p = np.zeros((self.natom, 3)) if pos else None
        v = np.zeros((self.natom, 3)) if vel else None
        log = np.zeros((self.counter + 1, 2))
        n = ctypes.c_int64()
        self._check(self.dev.lib.yg_md_get(self.dev.ctx, self._ptr(p), self._ptr(v), self._ptr(log),
                                           ctypes.byref(n)), 'yg_md_get')
        return p, v, log[:n.value]

    def save_restart(self, fn):
        """Writes the run's current state as a restart record (the layout of
        io.RestartWriter): counter (continuing a restarted run's count),
        time, positions, velocities, cell, conserved energy and the
        thermostat's state."""
        from .io import restart_state, _write_npz
        pos, vel, log = self.fetch()
        hooks = []
        corr = 0.0
        if self.thermostat is not None:
            corr, cp, cv = self.thermo_state()
            if getattr(self.thermostat, 'device_kind', None) == 4:
                self.thermostat.chain.pos[:] = cp
                self.thermostat.chain.vel[:] = cv
            corr += self.econs_offset
            self.thermostat.econs_correction = corr
            hooks = [self.thermostat]
        counter = self.counter0 + self.counter
        econs = float(log[-1, 0] + log[-1, 1] + corr)
        cell = self.ff.system.cell
        _write_npz(fn, restart_state(counter, counter * self.timestep, self.timestep, pos, vel, cell.rvecs, econs,
                                     None, hooks))

    def sync_host(self):
        """Copies the device positions back into the system; the next host
        compute() rebuilds the neighbour list."""
        p, _, _ = self.fetch(pos=True, vel=False)
        self.ff.system.pos[:] = p
        self.ff.update_pos(p)
        if self.ff.nlist is not None:
            self.ff.nlist.rebuild_next = True
        return p
