"""Velocity Verlet (NVE) driving a force field through ForceField.compute.

Same integration step, initial-velocity recipe and conserved-quantity
tracking as the reference's VerletIntegrator (yaff/sampling/verlet.py:320-390,
:476-516) and get_random_vel (yaff/sampling/utils.py:42-77): positions and
velocities stay FP64 NumPy arrays on the host; every step calls
``ff.update_pos`` and ``ff.compute(gpos, vtens)`` exactly as the reference
does, so the device force field is a drop-in for its force evaluation.
Thermostat/barostat hooks, HDF5 output and restarts are not part of this
module.
"""
import numpy as np

from .units import boltzmann

__all__ = ['get_random_vel', 'ConsErrTracker', 'VerletIntegrator']


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


class VerletIntegrator(object):
    """NVE velocity Verlet.

    ff: object with ``system`` (pos, masses), ``update_pos`` and
    ``compute(gpos, vtens)``.  vel0: initial velocities (default: seeded
    Maxwell-Boltzmann at temp0).  hooks: callables f(integrator) after every
    step.
    """

    def __init__(self, ff, timestep, vel0=None, temp0=300.0, scalevel0=True, hooks=None, rng=None, ndof=None):
        self.ff = ff
        self.timestep = timestep
        system = ff.system
        self.pos = system.pos.copy()
        self.masses = np.asarray(system.masses, dtype=np.float64)
        if vel0 is None:
            vel0 = get_random_vel(temp0, scalevel0, self.masses, rng=rng)
        self.vel = np.array(vel0, dtype=np.float64)
        self.gpos = np.zeros(self.pos.shape)
        self.vtens = np.zeros((3, 3))
        self.hooks = list(hooks or [])
        self.ndof = self.pos.size if ndof is None else ndof
        self.time = 0.0
        self.counter = 0
        self.econs_correction = 0.0
        self.cons_err = ConsErrTracker()
        self.initialize()

    def _compute_ekin(self):
        return 0.5 * ((self.vel ** 2).sum(axis=1) * self.masses).sum()

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
        self.compute_properties()

    def propagate(self):
        self.acc = -self.gpos / self.masses.reshape(-1, 1)
        self.vel += 0.5 * self.acc * self.timestep
        self.pos += self.timestep * self.vel
        self.ff.update_pos(self.pos)
        self.gpos[:] = 0.0
        self.vtens[:] = 0.0
        self.epot = self.ff.compute(self.gpos, self.vtens)
        self.acc = -self.gpos / self.masses.reshape(-1, 1)
        self.vel += 0.5 * self.acc * self.timestep
        self.time += self.timestep
        self.counter += 1
        self.compute_properties()
        for hook in self.hooks:
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
    """NVE velocity Verlet with positions, velocities, masses and the
    neighbour list resident in HBM (yg_md_* of libyaffgb.so).

    The same step as VerletIntegrator (yaff/sampling/verlet.py:339-367) and
    the same skin rule for rebuilding the list (yaff/pes/nlist.py:207-218),
    but the host only reads one scalar per step (the largest displacement
    since the last rebuild); the force evaluation and the second half kick
    are replayed from a CUDA graph when ``use_graph`` is set.  ``ff`` must run
    entirely on the fused device path (ForceField.device_md_terms).  The
    energy log holds (epot, ekin) of step 0 and of every step run since.
    """

    def __init__(self, ff, timestep, vel0=None, temp0=300.0, scalevel0=True, rng=None, max_steps=1000,
                 use_graph=True):
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
        vel0 = np.ascontiguousarray(vel0, dtype=np.float64)
        # one evaluation through the fused path builds the list and uploads
        # every parameter the device step needs
        ff.update_pos(system.pos)
        ff.compute(np.zeros((self.natom, 3)))
        self.dev, self.mask, self.const_energy = ff.device_md_terms()
        self.skin = float(ff.nlist.skin) if ff.nlist is not None else 0.0
        self.max_steps = int(max_steps)
        check(self.dev.lib.yg_md_setup(self.dev.ctx, ptr(self.masses), ptr(vel0), self.timestep, self.mask,
                                       self.const_energy, self.max_steps), 'yg_md_setup')
        self.counter = 0
        self.nrebuild = 0

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
