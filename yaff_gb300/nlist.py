"""Device neighbour list with the reference's NeighborList interface.

Same constructor, attributes and rebuild policy as yaff/pes/nlist.py:54-218:
``request_rcut`` raises the list radius to the largest pair cutoff,
``update_rmax`` recomputes the image range, and ``update`` rebuilds from
scratch unless the skin test (largest displacement since the last rebuild
times 2(rmax.max()+1) below the skin) allows the cheaper recompute path.  The
list itself stays on the GPU; ``neighs`` exports it in the reference's row
layout on demand (sorted by (a, b, r0, r1, r2)).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, ptr
from .device import device_of
from .system import as_system

__all__ = ['NeighborList', 'neigh_dtype']

neigh_dtype = _lib.neigh_dtype


class NeighborList(object):
    def __init__(self, system, skin=0, nlow=0, nhigh=-1):
        system = as_system(system)
        if skin < 0:
            raise ValueError('The skin parameter must be positive.')
        if nhigh == -1:
            nhigh = system.natom
        self.system = system
        self.skin = skin
        self.rcut = 0.0
        self._nneigh = 0
        self._pending = False   # a build was enqueued without waiting for its row count
        self.rmax = None
        if nlow < 0:
            raise ValueError('nlow must be a positive number, received %d.' % nlow)
        self.nlow = nlow
        if nhigh < self.nlow:
            raise ValueError('nhigh must not be smaller than nlow, received %d.' % nhigh)
        self.nhigh = nhigh
        self._built = False
        self._epoch = -1
        self.rebuild_next = False
        self._neighs_cache = None
        self.nrebuild = 0
        self.nrecompute = 0

    @property
    def device(self):
        return device_of(self.system)

    def request_rcut(self, rcut):
        """Make sure the internal rcut parameter is at least as high as rcut."""
        self.rcut = max(self.rcut, rcut)
        self.update_rmax()

    def update_rmax(self):
        """Recompute the image range rmax = ceil((rcut+skin)/rspacings - 0.5)."""
        self.rmax = np.ceil((self.rcut + self.skin) / self.system.cell.rspacings - 0.5).astype(int)
        self.rebuild_next = True

    def _need_rebuild(self):
        if self.skin <= 0 or not self._built or self.rebuild_next:
            return True
        if self._epoch != self.device.list_epoch:
            return True
        d2 = ctypes.c_double()
        check(self.device.lib.yg_nlist_max_disp2(self.device.ctx, ctypes.byref(d2)), 'yg_nlist_max_disp2')
        disp = np.sqrt(d2.value) * 2 * (self.rmax.max() + 1)
        return disp >= self.skin

    def set_capacity(self, slots):
        """Per-atom slot capacity of the device list's next builds (rounded
        up to 32); the current list is dropped and the next update rebuilds.
        Builds that need more slots regrow, as the reference's buffer does
        (yaff/pes/nlist.py:170-182)."""
        check(self.device.lib.yg_nlist_set_capacity(self.device.ctx, int(slots)), 'yg_nlist_set_capacity')
        self.rebuild_next = True
        self._neighs_cache = None

    @property
    def nneigh(self):
        """Number of rows of the list (the reference's half-list count)."""
        if self._pending:
            self.finish()
        return self._nneigh

    @nneigh.setter
    def nneigh(self, value):
        self._nneigh = value

    def finish(self):
        """Outcome of a build enqueued by update(defer=True): sets nneigh, or,
        when a row overflowed its slots, rebuilds the list now (the slot
        capacity has grown) and returns False: whatever was computed from the
        deferred build's rows must be recomputed."""
        if not self._pending:
            return True
        self._pending = False
        n = ctypes.c_int64()
        rc = self.device.lib.yg_nlist_build_wait(self.device.ctx, ctypes.byref(n))
        if rc == _lib.YG_ERR_CAPACITY:
            self.rebuild_next = True
            self.update(upload=False)
            return False
        check(rc, 'yg_nlist_build_wait')
        self._nneigh = n.value
        return True

    def update(self, upload=True, defer=False):
        """Rebuild or recompute the list for the current system positions.
        With defer, a rebuild is enqueued without waiting for its row count
        (the caller enqueues the pair terms behind it; finish() or any result
        readback reports an overflow)."""
        assert self.rcut > 0
        dev = self.device
        dev.sync_cell()
        if getattr(self, '_rmax_cell_key', None) != dev._cell_key:
            # the cell changed since rmax was last derived (the change may
            # have been synchronised to the device by another part)
            self.update_rmax()
            self._rmax_cell_key = dev._cell_key
        if upload:
            dev.upload_positions()
        self._neighs_cache = None
        if self._need_rebuild():
            if self.system.cell.volume != 0 and self.system.natom / self.system.cell.volume > 10:
                raise ValueError('Atom density too high')
            rmax = np.zeros(3, np.int64)
            rmax[:len(self.rmax)] = self.rmax
            if defer:
                check(dev.lib.yg_nlist_build_async(dev.ctx, self.rcut + self.skin, ptr(rmax), self.nlow,
                                                   self.nhigh), 'yg_nlist_build_async')
                self._pending = True
            else:
                self._pending = False
                n = ctypes.c_int64()
                check(dev.lib.yg_nlist_build(dev.ctx, self.rcut + self.skin, ptr(rmax), self.nlow, self.nhigh,
                                             ctypes.byref(n)), 'yg_nlist_build')
                self._nneigh = n.value
            self._built = True
            self._epoch = dev.list_epoch
            self.rebuild_next = False
            self.nrebuild += 1
            return True
        check(dev.lib.yg_nlist_recompute(dev.ctx), 'yg_nlist_recompute')
        self.nrecompute += 1
        return False

    @property
    def neighs(self):
        """The half list as reference rows (exported from the device)."""
        if self._neighs_cache is None:
            if not self._built:
                return np.zeros(0, neigh_dtype)
            dev = self.device
            rows = np.zeros(max(self.nneigh, 1), neigh_dtype)
            n = ctypes.c_int64()
            check(dev.lib.yg_nlist_export(dev.ctx, ptr(rows), len(rows), ctypes.byref(n)), 'yg_nlist_export')
            self._neighs_cache = rows[:n.value]
        return self._neighs_cache

    def to_dictionary(self):
        """{(a, b, r0, r1, r2): [d, dx, dy, dz]} of the current list (slow)."""
        nb = self.neighs
        return dict(((int(r['a']), int(r['b']), int(r['r0']), int(r['r1']), int(r['r2'])),
                     np.array([r['d'], r['dx'], r['dy'], r['dz']])) for r in nb)

    def check(self):
        """Slow brute-force consistency test on the host (small systems only),
        the enumeration of yaff/pes/nlist.py:240-350."""
        actual = self.to_dictionary()
        cell = self.system.cell
        pos = self.system.pos
        rmax = np.zeros(3, int)
        rmax[:len(self.rmax)] = self.rmax
        expected = {}
        rc = self.rcut + self.skin
        for r2 in range(0, rmax[2] + 1):
            for r1 in range(0 if r2 == 0 else -rmax[1], rmax[1] + 1):
                for r0 in range(0 if (r2 == 0 and r1 == 0) else -rmax[0], rmax[0] + 1):
                    for a in range(self.system.natom):
                        for b in range(a + 1):
                            if not ((a >= self.nlow and b < self.nhigh) or (b >= self.nlow and a < self.nhigh)):
                                continue
                            image = (r0, r1, r2) != (0, 0, 0)
                            signs = [1, -1] if image else ([1] if a > b else [])
                            if image and a == b:
                                signs = [1]
                            for sign in signs:
                                delta = pos[b] - pos[a]
                                cell.mic(delta)
                                delta *= sign
                                cell.add_vec(delta, np.array([r0, r1, r2]))
                                d = np.linalg.norm(delta)
                                if d < rc:
                                    key = (a, b, r0, r1, r2) if sign == 1 else (b, a, r0, r1, r2)
                                    expected[key] = np.array([d, delta[0], delta[1], delta[2]])
        missing = set(expected) - set(actual)
        extra = set(actual) - set(expected)
        assert not missing and not extra, 'neighbour list mismatch: %d missing, %d redundant' % (
            len(missing), len(extra))
        for k, v in expected.items():
            assert abs(actual[k] - v).max() < 1e-10, k
