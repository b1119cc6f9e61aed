"""Many small systems on one GPU, stepped together (yg_fleet_* of libyaffgb.so).

``Fleet`` wraps one device fleet: fixed capacities (atoms, systems,
reciprocal vectors, neighbour slots per atom, steps per system) allocated
once, systems added and removed between steps, and one MD step of every
system in flight as eight kernel launches replayed from a CUDA graph --
the launch count per step does not grow with the number of systems.

``FleetEngine`` serves NVE requests (serve.Request: an LJ + EI + Ewald
system and a step count) from a fleet with continuous batching: requests
are admitted in arrival order as soon as a slot and contiguous atom and
k-vector ranges are free (the fleet's capacities are its device-memory
budget, allocated up front); every chunk of `chunk` steps advances all
systems in flight, and finished systems are read back and retired between
chunks.  A request larger than the whole fleet is rejected; a cancelled
request is withdrawn before admission or retired at the next chunk
boundary.  A system's trajectory is the same alone and in any mix.
"""
import ctypes
import time

import numpy as np

from . import _lib
from ._lib import check, ptr
from .units import femtosecond

__all__ = ['Fleet', 'FleetEngine', 'fleet_bytes']

NEIGHBOR_SLOTS = 512


def fleet_bytes(max_atoms, max_systems, max_k, max_neighbors=NEIGHBOR_SLOTS, max_steps=64):
    """Device memory a fleet of these capacities allocates."""
    per_atom = 6 * 24 + 3 * 8 + 3 * 4 + 5 * 16 + 2 * 4 + 64 * 8 + 16 * max_neighbors
    return int(max_atoms * per_atom + max_k * (16 + 8 + 4 + 16 + 8 + 16) + max_systems * (240 + 16 * (max_steps + 1)))


class Fleet(object):
    def __init__(self, max_atoms, max_systems, max_k, max_neighbors=NEIGHBOR_SLOTS, max_steps=64, stream=None):
        _lib.require_cuda()
        self.lib = _lib.load()
        self.max_systems = int(max_systems)
        self.max_steps = int(max_steps)
        h = ctypes.c_void_p()
        check(self.lib.yg_fleet_create(int(max_atoms), self.max_systems, int(max_k), int(max_neighbors),
                                       self.max_steps, None if stream is None else ctypes.c_void_p(stream),
                                       ctypes.byref(h)), 'yg_fleet_create')
        self.handle = h
        self.natom = {}

    def add(self, spec, vel, nsteps, dt):
        """Adds a configs.serving_request-style spec (LJ + EI + Ewald, no
        exclusions) with initial velocities; returns its slot, or None when
        the fleet has no room for it now."""
        pos = np.ascontiguousarray(spec['pos'], dtype=np.float64)
        n = len(pos)
        lj = [p for p in spec['pair'] if p['kind'] == 'lj']
        sig = np.ascontiguousarray(lj[0]['sigmas'] if lj else np.zeros(n), dtype=np.float64)
        eps = np.ascontiguousarray(lj[0]['epsilons'] if lj else np.zeros(n), dtype=np.float64)
        q = np.ascontiguousarray(spec['charges'], dtype=np.float64)
        m = np.ascontiguousarray(spec['masses'], dtype=np.float64)
        v = np.ascontiguousarray(vel, dtype=np.float64)
        rv = np.ascontiguousarray(spec['rvecs'], dtype=np.float64)
        ew = spec['ewald']
        slot = ctypes.c_int(-1)
        rc = self.lib.yg_fleet_add(self.handle, n, ptr(pos), ptr(v), ptr(m), ptr(q), ptr(sig), ptr(eps), ptr(rv),
                                   float(spec['rcut']), float(spec.get('skin', 0.0)), float(ew['alpha']),
                                   float(ew['gcut']), float(dt), int(nsteps), ctypes.byref(slot))
        if rc == _lib.YG_ERR_CAPACITY:
            return None
        check(rc, 'yg_fleet_add')
        self.natom[slot.value] = n
        return slot.value

    def step(self, nsteps):
        check(self.lib.yg_fleet_step(self.handle, int(nsteps)), 'yg_fleet_step')

    def poll(self):
        """(state, steps) per slot: 0 empty, 1 stepping, 2 done, 3 failed."""
        st = np.zeros(self.max_systems, np.int32)
        sp = np.zeros(self.max_systems, np.int32)
        check(self.lib.yg_fleet_poll(self.handle, ptr(st), ptr(sp)), 'yg_fleet_poll')
        return st, sp

    def get(self, slot):
        """(pos, vel, log, failed) of a slot; log rows (epot, ekin) from step 0."""
        n = self.natom[slot]
        pos = np.zeros((n, 3))
        vel = np.zeros((n, 3))
        log = np.zeros((self.max_steps + 1, 2))
        nlog = ctypes.c_int64()
        rc = self.lib.yg_fleet_get(self.handle, int(slot), ptr(pos), ptr(vel), ptr(log), ctypes.byref(nlog))
        if rc not in (_lib.YG_OK, _lib.YG_ERR_CAPACITY):
            check(rc, 'yg_fleet_get')
        return pos, vel, log[:nlog.value], rc == _lib.YG_ERR_CAPACITY

    def remove(self, slot):
        check(self.lib.yg_fleet_remove(self.handle, int(slot)), 'yg_fleet_remove')
        self.natom.pop(slot, None)

    def usage(self):
        a, n, k = ctypes.c_int64(), ctypes.c_int(), ctypes.c_int64()
        check(self.lib.yg_fleet_usage(self.handle, ctypes.byref(a), ctypes.byref(n), ctypes.byref(k)),
              'yg_fleet_usage')
        return a.value, n.value, k.value

    def launch_count(self):
        return int(self.lib.yg_fleet_launch_count(self.handle))

    def close(self):
        if getattr(self, 'handle', None) is not None and self.handle.value:
            self.lib.yg_fleet_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FleetEngine(object):
    """Continuous batching of NVE requests on one Fleet.

    max_atoms / max_systems / max_k: the fleet's capacities (its device
    memory, see fleet_bytes); chunk: steps between two admission / retirement
    points; dt, temp0: time step and initial temperature (seeded
    Maxwell-Boltzmann velocities per request, as serve.serve_request)."""

    def __init__(self, max_atoms=1 << 18, max_systems=256, max_k=1 << 20, chunk=5, dt=0.5 * femtosecond,
                 temp0=300.0, max_steps=64, max_neighbors=NEIGHBOR_SLOTS):
        self.fleet = Fleet(max_atoms, max_systems, max_k, max_neighbors=max_neighbors, max_steps=max_steps)
        self.max_atoms = int(max_atoms)
        self.chunk = int(chunk)
        self.dt = dt
        self.temp0 = temp0
        self.peak_inflight = 0
        self.peak_atoms = 0
        self.steps_run = 0

    def _velocities(self, req):
        from .verlet import get_random_vel
        return get_random_vel(self.temp0, True, np.asarray(req.spec['masses'], float),
                              rng=np.random.default_rng(req.seed))

    def run(self, requests, realtime=True):
        """Serves `requests` (sorted by arrival; with realtime, arrival times
        are offsets from the start, written back as absolute perf_counter
        times).  Returns wall seconds."""
        fl = self.fleet
        t0 = time.perf_counter()
        for r in requests:
            r.arrival = t0 + (r.arrival if realtime else 0.0)
        pending = list(requests)
        pending.reverse()   # pop() gives the earliest
        running = {}        # slot -> request
        while pending or running:
            now = time.perf_counter()
            # admission in arrival order (no overtaking)
            while pending and pending[-1].arrival <= now:
                r = pending[-1]
                if r.cancelled:
                    pending.pop()
                    r.error = 'cancelled'
                    r.t_done = time.perf_counter()
                    continue
                if r.natom > self.max_atoms:
                    pending.pop()
                    r.error = 'rejected: %d atoms, more than the whole fleet of %d' % (r.natom, self.max_atoms)
                    r.t_done = time.perf_counter()
                    continue
                if r.nsteps > fl.max_steps:
                    pending.pop()
                    r.error = 'rejected: %d steps, more than the fleet log of %d' % (r.nsteps, fl.max_steps)
                    r.t_done = time.perf_counter()
                    continue
                slot = fl.add(r.spec, self._velocities(r), r.nsteps, self.dt)
                if slot is None:
                    if not running:
                        pending.pop()
                        r.error = 'rejected: does not fit an empty fleet'
                        r.t_done = time.perf_counter()
                        continue
                    break
                pending.pop()
                r.t_admit = r.t_start = time.perf_counter()
                r.slot = slot
                running[slot] = r
            if not running:
                if pending:
                    wait = pending[-1].arrival - time.perf_counter()
                    if wait > 0:
                        time.sleep(min(wait, 0.05))
                continue
            self.peak_inflight = max(self.peak_inflight, len(running))
            self.peak_atoms = max(self.peak_atoms, fl.usage()[0])
            fl.step(self.chunk)
            self.steps_run += self.chunk
            state, _ = fl.poll()
            for slot in list(running):
                r = running[slot]
                if state[slot] in (2, 3) or r.cancelled:
                    if r.cancelled and state[slot] == 1:
                        r.error = 'cancelled'
                    else:
                        r.pos, r.vel, r.log, failed = fl.get(slot)
                        if failed:
                            r.error = 'neighbour rows overflowed'
                    fl.remove(slot)
                    r.t_done = time.perf_counter()
                    del running[slot]
        return time.perf_counter() - t0

    def close(self):
        self.fleet.close()
