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
    """A hook that acts inside the Verlet step (thermostats): ``init`` at
    initialization, ``pre`` before the first half kick, ``post`` after the
    second; ``econs_correction`` is added to the conserved energy
    (yaff/sampling/verlet.py:418-446)."""
    device_kind = None

    def __init__(self, start=0, step=1):
        self.econs_correction = 0.0

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


class VerletIntegrator(object):
    """Velocity Verlet with the reference's hook protocol.

    ff: object with ``system`` (pos, masses, cell), ``update_pos`` and
    ``compute(gpos, vtens)``.  vel0: initial velocities (default: seeded
    Maxwell-Boltzmann at temp0).  hooks: VerletHook objects (thermostats,
    called before and after the Verlet step) and plain callables
    f(integrator), called after every step.  ndof: degrees of freedom (None:
    set by a thermostat's init, else 3 N).
    """

    def __init__(self, ff, timestep, vel0=None, temp0=300.0, scalevel0=True, hooks=None, rng=None, ndof=None):
        self.ff = ff
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
        self.hooks = list(hooks or [])
        self.ndof = ndof
        self.time = 0.0
        self.counter = 0
        self.cons_err = ConsErrTracker()
        self.initialize()

    def _verlet_hooks(self, kind):
        for hook in self.hooks:
            if isinstance(hook, VerletHook):
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

    def __init__(self, ff, timestep, vel0=None, temp0=300.0, scalevel0=True, rng=None, max_steps=1000,
                 use_graph=True, thermostat=None, seed=0, ndof=None):
        from . import _lib
        from ._lib import check, ptr
        self._lib, self._check, self._ptr = _lib, check, ptr
        self.ff = ff
        self.timestep = float(timestep)
        self.use_graph = bool(use_graph)
        system = ff.system
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

    def sync_host(self):
        """Copies the device positions back into the system; the next host
        compute() rebuilds the neighbour list."""
        p, _, _ = self.fetch(pos=True, vel=False)
        self.ff.system.pos[:] = p
        self.ff.update_pos(p)
        if self.ff.nlist is not None:
            self.ff.nlist.rebuild_next = True
        return p
