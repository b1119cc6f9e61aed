"""Serving loop: many independent small systems, each a short NVE run.

A request carries one system (positions, cell, charges, LJ parameters) and
asks for ``nsteps`` velocity-Verlet steps; the answer is its energy log and
final positions and velocities.  The reference evaluates one ForceField per
process and step (yaff/pes/ff.py:226-245 inside yaff/sampling/verlet.py:
339-367); here many requests share one GPU:

* continuous batching: a fixed number of slots, each a worker thread with its
  own CUDA stream; a request enters the first free slot as soon as the
  admission rule lets it, without waiting for the others in flight;
* admission by device memory: a request is admitted only while the summed
  footprint estimate (``estimate_bytes``) of the requests in flight stays
  within ``budget_bytes``; requests are served in arrival order;
* each request runs device-resident (yg_md_*): positions, velocities and
  the neighbour list stay in HBM, the skin test and the rebuild run on the
  device, every step is replayed from a CUDA graph, and the library's
  stream-ordered allocator keeps context creation and destruction from
  synchronizing the device;
* library calls release the GIL (ctypes), so the GPU work of the slots
  overlaps.

Latency is arrival to completion (queueing included); throughput is requests
completed per second of wall time.
"""
import math
import queue
import threading
import time

import numpy as np

from . import configs
from .units import femtosecond

__all__ = ['Request', 'Cancelled', 'make_workload', 'estimate_bytes', 'serve_request', 'ServingEngine',
           'run_sequential', 'summarize']



class Request(object):
    def __init__(self, rid, natom, seed, arrival, nsteps):
        self.rid = rid
        self.natom = int(natom)
        self.seed = int(seed)
        self.arrival = float(arrival)
        self.nsteps = int(nsteps)
        self.spec = None
        # filled by the engine
        self.estimate = 0
        self.t_admit = self.t_start = self.t_done = None
        self.log = self.pos = self.vel = None
        self.nrebuild = 0
        self.bytes_high = 0
        self.slot = None
        self.error = None
        self.cancelled = False

    def cancel(self):
        """Withdraws the request: one still waiting for admission is never
        started; one in service stops at its next batch of MD steps and
        releases its device memory.  Its error reads 'cancelled'."""
        self.cancelled = True

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival


class Cancelled(Exception):
    """A request was withdrawn while in service."""


def request_spec(natom, seed, skin):
    """The system of one request: LJ + EI + Ewald at 0.064 atoms/A^3 with
    rcut 10 A (configs.serving_request) and a Verlet skin."""
    spec = configs.serving_request(natom, seed)
    spec['skin'] = skin
    return spec


def make_workload(nreq=4096, rate=200.0, seed=2024, nmin=64, nmax=4000, nsteps=50, skin=None):
    """nreq requests with log-uniform natom in [nmin, nmax] and Poisson
    arrivals at `rate` requests/s (seeded); specs are built up front (the
    client's payload exists before it arrives)."""
    from .units import angstrom
    skin = 1.0 * angstrom if skin is None else skin
    rng = np.random.default_rng(seed)
    natoms = np.exp(rng.uniform(math.log(nmin), math.log(nmax), nreq)).astype(int)
    natoms = np.clip(natoms, nmin, nmax)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq)) if rate > 0 else np.zeros(nreq)
    seeds = rng.integers(0, 2 ** 31 - 1, nreq)
    reqs = []
    for i in range(nreq):
        r = Request(i, natoms[i], seeds[i], arrivals[i], nsteps)
        r.spec = request_spec(r.natom, r.seed, skin)
        reqs.append(r)
    return reqs


def estimate_bytes(spec, precision='mixed', nsteps=50):
    """Upper estimate of the device memory one request's context holds at
    its peak: per-atom state, the neighbour slots (1.5x the mean count inside
    rcut + skin, the list's own first guess being 1.3x), the Ewald tables and
    structure-factor partials, the energy log; every buffer with the
    allocator's growth margin."""
    n = len(spec['pos'])
    rv = np.asarray(spec['rvecs'])
    vol = abs(np.linalg.det(rv))
    rc = spec['rcut'] + spec.get('skin', 0.0)
    fp64 = precision == 'fp64'
    grow = lambda b: int(b * 1.25) + 256  # noqa: E731  (yg_ensure's margin)
    per_atom = 172 + 144 + 24 + 240 + 32 + 24 + 8 + 72  # ... + integrator state and its snapshot
    total = per_atom * n + 16384
    est = n / vol * 4.0 / 3.0 * math.pi * rc ** 3
    cap = int(1.5 * est) + 128
    total += 8 * n * cap
    total += 65536 + 16 * n  # cell lists, stencil shifts, reductions
    ew = spec.get('ewald')
    if ew is not None:
        gsp = 1.0 / np.linalg.norm(rv, axis=1)
        gmax = np.ceil(ew['gcut'] / gsp - 0.5).astype(int)
        nm = int(gmax[2]) + 1
        ncol = (2 * int(gmax[0]) + 1) * (2 * int(gmax[1]) + 1)
        nkd = ncol * nm
        ct = 16 if fp64 else 8
        L = int(gmax.sum()) + 3
        nstile = (ncol + 127) // 128 + 1
        nslab = (nm + 31) // 32
        per = nstile * nslab * 128 * 32
        chunks = max(1, (n + 255) // 256)
        total += grow(n * L * ct) + grow(per * chunks * ct) + grow(3 * nkd * ct) + 8 * nkd + 48 * nkd + \
            16 * nstile * 128 + grow(24 * n) + grow(8 * (7 * (nkd // 256 + 2) + 71))
    total += 16 * (nsteps + 2) + 8 * (n * 3 // 256 + 2)
    return int(total * 1.1) + 65536


def serve_request(req, stream, precision='mixed', dt=0.5 * femtosecond, temp0=300.0, use_graph=True,
                  batch_steps=None):
    """Runs one request start to finish on `stream` (a cudaStream_t handle)
    through the C entry points directly: the same calls the ForceField path
    makes (cell, positions, charges, empty scaling table, the LJ and EI pair
    potentials, list build with rmax = ceil((rcut+skin)/spacing - 0.5),
    Ewald set-up with gmax = ceil(gcut/gspacing - 0.5), the neutralizing
    energy as a constant), without building the Python object graph, so
    that the per-request host work holding the GIL stays small.  Fills
    req.log / pos / vel / nrebuild / bytes_high.  With batch_steps the MD
    runs in batches of that many steps and a cancelled request stops between
    two of them (raising Cancelled after its context is destroyed)."""
    from ctypes import byref, c_int64, c_void_p
    from . import _lib
    from ._lib import check, ptr
    from .system import Cell
    from .verlet import get_random_vel
    lib = _lib.load()
    spec = req.spec
    n = len(spec['pos'])
    cell = Cell(np.asarray(spec['rvecs'], dtype=np.float64))
    prec = _lib.PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    h = c_void_p()
    tp = [time.perf_counter()]
    check(lib.yg_create(n, prec, c_void_p(stream), byref(h)), 'yg_create')
    try:
        rv = np.ascontiguousarray(cell.full_rvecs())
        gv = np.ascontiguousarray(cell.full_gvecs())
        check(lib.yg_set_cell(h, ptr(rv), ptr(gv), 3, float(cell.volume)), 'yg_set_cell')
        pos = np.ascontiguousarray(spec['pos'], dtype=np.float64)
        check(lib.yg_set_positions(h, ptr(pos), 0), 'yg_set_positions')
        q = np.ascontiguousarray(spec['charges'], dtype=np.float64)
        check(lib.yg_set_charges(h, ptr(q)), 'yg_set_charges')
        check(lib.yg_set_scalings(h, None, None, None, None, 0), 'yg_set_scalings')
        rcut = float(spec['rcut'])
        ew = spec['ewald']
        diel = float(spec.get('dielectric', 1.0))
        mask = 0
        for slot, p in enumerate(spec['pair']):
            if p['kind'] == 'lj':
                sg = np.ascontiguousarray(p['sigmas'], dtype=np.float64)
                ep = np.ascontiguousarray(p['epsilons'], dtype=np.float64)
                check(lib.yg_set_pair_pot(h, slot, _lib.POT_LJ, ptr(sg), ptr(ep), None, None, 0.0, 1.0, rcut,
                                          _lib.TR_NONE, 0.0), 'yg_set_pair_pot')
            elif p['kind'] == 'ei':
                check(lib.yg_set_pair_pot(h, slot, _lib.POT_EI, None, None, None, None, float(ew['alpha']), diel,
                                          rcut, _lib.TR_NONE, 0.0), 'yg_set_pair_pot')
            else:
                raise ValueError(p['kind'])
            mask |= 1 << slot
        skin = float(spec['skin'])
        rmax = np.ascontiguousarray(np.ceil((rcut + skin) / cell.rspacings - 0.5).astype(np.int64))
        nn = c_int64()
        tp.append(time.perf_counter())
        check(lib.yg_nlist_build(h, rcut + skin, ptr(rmax), 0, n, byref(nn)), 'yg_nlist_build')
        gmax = np.ascontiguousarray(np.ceil(ew['gcut'] / cell.gspacings - 0.5).astype(np.int64))
        tp.append(time.perf_counter())
        check(lib.yg_ewald_setup(h, float(ew['alpha']), float(ew['gcut']), ptr(gmax), diel, 0, n), 'yg_ewald_setup')
        tp.append(time.perf_counter())
        mask |= (1 << _lib.PART_EWALD_RECI) | (1 << _lib.PART_EWALD_CORR)
        # neutralizing background (yaff/pes/ff.py:640-669), position independent
        eneut = np.pi / (2.0 * diel * cell.volume) * q.sum() ** 2 / ew['alpha'] ** 2
        masses = np.ascontiguousarray(spec['masses'], dtype=np.float64)
        vel = np.ascontiguousarray(get_random_vel(temp0, True, masses, rng=np.random.default_rng(req.seed)))
        check(lib.yg_md_setup(h, ptr(masses), ptr(vel), float(dt), mask, float(eneut), req.nsteps), 'yg_md_setup')
        tp.append(time.perf_counter())
        nreb = c_int64()
        left = req.nsteps
        step = req.nsteps if not batch_steps else int(batch_steps)
        nrebuild = 0
        while left > 0:
            if req.cancelled:
                raise Cancelled()
            nb = min(step, left)
            check(lib.yg_md_run(h, nb, int(use_graph), skin, byref(nreb)), 'yg_md_run')
            nrebuild += nreb.value
            left -= nb
        nreb.value = nrebuild
        tp.append(time.perf_counter())
        req.pos = np.zeros((n, 3))
        req.vel = np.zeros((n, 3))
        log = np.zeros((req.nsteps + 1, 2))
        nlog = c_int64()
        check(lib.yg_md_get(h, ptr(req.pos), ptr(req.vel), ptr(log), byref(nlog)), 'yg_md_get')
        req.log = log[:nlog.value]
        req.nrebuild = nreb.value
        now, high = c_int64(), c_int64()
        check(lib.yg_mem_usage(h, byref(now), byref(high)), 'yg_mem_usage')
        req.bytes_high = high.value
    finally:
        lib.yg_destroy(h)
    tp.append(time.perf_counter())
    # seconds in: create + parameters, list build, Ewald set-up, MD set-up
    # (step-0 forces), the steps, readback + destroy
    req.phases = np.diff(tp)


class ServingEngine(object):
    """Continuous-batching server of NVE requests on one GPU.

    nslots: concurrent requests (worker threads, one CUDA stream each);
    budget_bytes: device-memory budget for the requests in flight;
    precision: 'mixed' or 'fp64'; use_graph: replay each request's step from
    a CUDA graph; dt: time step (0.5 fs: the 2.0-2.5 A lattice spacings of
    these LJ systems, far inside the LJ minimum, blow up within 50 steps of
    1 fs for a few sizes just above a cube number); temp0: initial
    temperature (seeded Maxwell-Boltzmann velocities per request).
    """

    def __init__(self, nslots=8, budget_bytes=8 << 30, precision='mixed', use_graph=True,
                 dt=0.5 * femtosecond, temp0=300.0, batch_steps=None):
        import torch
        self.nslots = int(nslots)
        self.budget = int(budget_bytes)
        self.precision = precision
        self.use_graph = use_graph
        self.dt = dt
        self.temp0 = temp0
        self.batch_steps = batch_steps
        self.streams = [torch.cuda.Stream() for _ in range(self.nslots)]
        self._lock = threading.Condition()
        self._inflight = 0
        self.peak_inflight_bytes = 0
        self.peak_inflight = 0
        self._busy = 0

    # one request, on one slot's stream
    def _serve(self, req, slot):
        req.t_start = time.perf_counter()
        req.slot = slot
        if req.cancelled:
            raise Cancelled()
        serve_request(req, self.streams[slot].cuda_stream, self.precision, self.dt, self.temp0, self.use_graph,
                      self.batch_steps)

    def _worker(self, slot, inbox, done):
        while True:
            req = inbox.get()
            if req is None:
                return
            try:
                self._serve(req, slot)
            except Cancelled:
                req.error = 'cancelled'
            except Exception as exc:  # reported per request, the server keeps going
                req.error = repr(exc)
            req.t_done = time.perf_counter()
            with self._lock:
                self._inflight -= req.estimate
                self._busy -= 1
                self._lock.notify_all()
            done.put(slot)

    def run(self, requests, realtime=True):
        """Serves `requests` (sorted by arrival); with realtime, a request is
        not admitted before its arrival time (offsets from the start of the
        run, written back as absolute perf_counter times).  Returns wall
        seconds.  A request whose footprint estimate exceeds the whole budget
        is rejected (its error says so) and the others are served; a request
        cancelled before admission is not started."""
        for r in requests:
            r.estimate = estimate_bytes(r.spec, self.precision, r.nsteps)
        inboxes = [queue.Queue() for _ in range(self.nslots)]
        done = queue.Queue()
        free = list(range(self.nslots))
        threads = [threading.Thread(target=self._worker, args=(s, inboxes[s], done), daemon=True)
                   for s in range(self.nslots)]
        for t in threads:
            t.start()
        t0 = time.perf_counter()
        for r in requests:
            r.arrival = t0 + (r.arrival if realtime else 0.0)
        try:
            for r in requests:
                if realtime:
                    wait = r.arrival - time.perf_counter()
                    if wait > 0:
                        time.sleep(wait)
                if r.estimate > self.budget:
                    r.error = 'rejected: needs %d bytes, more than the whole budget of %d' % (r.estimate, self.budget)
                    r.t_done = time.perf_counter()
                    continue
                if r.cancelled:
                    r.error = 'cancelled'
                    r.t_done = time.perf_counter()
                    continue
                # a free slot and room in the budget (arrival order: no overtaking)
                while True:
                    while not done.empty():
                        free.append(done.get())
                    with self._lock:
                        fits = self._inflight + r.estimate <= self.budget
                        if free and fits:
                            self._inflight += r.estimate
                            self._busy += 1
                            self.peak_inflight_bytes = max(self.peak_inflight_bytes, self._inflight)
                            self.peak_inflight = max(self.peak_inflight, self._busy)
                            break
                    free.append(done.get())
                slot = free.pop()
                r.t_admit = time.perf_counter()
                inboxes[slot].put(r)
        finally:
            for q in inboxes:
                q.put(None)
            for t in threads:
                t.join()
        return time.perf_counter() - t0


def run_sequential(requests, precision='fp64', dt=0.5 * femtosecond, temp0=300.0, mode='api'):
    """Per-system baselines: the same requests one after another, each its
    own context.  mode 'api': the drop-in use of the library, a ForceField
    driven by the host VerletIntegrator (one ForceField.compute per step, as
    yaff/sampling/verlet.py does); mode 'device': serve_request on the
    default stream, one request at a time.  Returns wall seconds."""
    from .builder import build_forcefield
    from .verlet import VerletIntegrator
    t0 = time.perf_counter()
    for r in requests:
        r.arrival = r.t_start = time.perf_counter()
        if mode == 'api':
            ff = build_forcefield(r.spec, precision=precision)
            vi = VerletIntegrator(ff, dt, temp0=temp0, rng=np.random.default_rng(r.seed))
            epot = [vi.epot]
            ekin = [vi.ekin]
            for _ in range(r.nsteps):
                vi.propagate()
                epot.append(vi.epot)
                ekin.append(vi.ekin)
            r.pos, r.vel, r.log = vi.pos.copy(), vi.vel.copy(), np.array([epot, ekin]).T
            ff.system._device.destroy()
        else:
            serve_request(r, 0, precision, dt, temp0, use_graph=True)
        r.t_done = time.perf_counter()
    return time.perf_counter() - t0


def summarize(requests, wall):
    lat = np.array([r.latency for r in requests if r.t_done is not None and r.error is None])
    svc = np.array([r.t_done - r.t_start for r in requests if r.t_done is not None and r.error is None])
    atoms_steps = sum(r.natom * r.nsteps for r in requests if r.error is None)
    return {
        'requests': len(requests),
        'errors': sum(1 for r in requests if r.error is not None),
        'wall_s': wall,
        'requests_per_s': len(lat) / wall if wall > 0 else None,
        'atom_steps_per_s': atoms_steps / wall if wall > 0 else None,
        'latency_p50_ms': float(np.percentile(lat, 50) * 1e3) if len(lat) else None,
        'latency_p99_ms': float(np.percentile(lat, 99) * 1e3) if len(lat) else None,
        'service_p50_ms': float(np.percentile(svc, 50) * 1e3) if len(svc) else None,
        'service_p99_ms': float(np.percentile(svc, 99) * 1e3) if len(svc) else None,
    }
