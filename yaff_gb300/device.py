"""Device-resident state of one system (wraps a yg_ctx of libyaffgb.so).

One ``DeviceSystem`` is attached to each ``System`` the first time a GPU part
or neighbour list needs it; the neighbour list, the pair parts, the Ewald
parts and the valence part of that system all share it, so positions are
uploaded once per evaluation and every kernel works on the same resident
copy.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, ptr

__all__ = ['DeviceSystem', 'device_of', 'set_default_precision', 'get_default_precision']

_default_precision = _lib.FP64


def set_default_precision(precision):
    """'fp64' (plain, the default), 'mixed' or 'mixed_kahan'."""
    global _default_precision
    _default_precision = _lib.PRECISIONS[precision] if isinstance(precision, str) else int(precision)


def get_default_precision():
    return _default_precision


def _pinned(shape):
    """(array, owner): a zero-filled float64 host array in page-locked
    memory (host-to-device copies from it are asynchronous DMA) and the
    tensor that owns the memory (keep it alive as long as the array)."""
    import torch
    t = torch.zeros(shape, dtype=torch.float64, pin_memory=True)
    return t.numpy(), t


def device_of(system, precision=None, stream=None):
    """The DeviceSystem of a System, created on first use (on `stream`, a
    cudaStream_t handle as int, default: the legacy default stream)."""
    dev = getattr(system, '_device', None)
    if dev is None:
        dev = DeviceSystem(system, _default_precision if precision is None else precision, stream=stream)
        system._device = dev
    elif precision is not None:
        dev.set_precision(precision)
    return dev


class DeviceSystem(object):
    def __init__(self, system, precision=_lib.FP64, stream=None):
        _lib.require_cuda()
        self.lib = _lib.load()
        self.system = system
        self.natom = system.natom
        if isinstance(precision, str):
            precision = _lib.PRECISIONS[precision]
        self.precision = precision
        handle = ctypes.c_void_p()
        self.stream = stream
        check(self.lib.yg_create(self.natom, precision, None if stream is None else ctypes.c_void_p(stream),
                                 ctypes.byref(handle)), 'yg_create')
        self.ctx = handle
        self._cell_key = None
        self._charges_key = None
        self.pair_slots = []          # ForcePartPair objects in slot order
        self.scalings_obj = None
        self.ewald_key = None
        self.valence_key = None
        self._pos_staging, self._pos_owner = _pinned((self.natom, 3))
        # the system's positions move into the page-locked buffer (same
        # values): ForceField.update_pos then writes straight into the memory
        # the host->device copy reads, one host copy per step instead of two
        self._pos_staging[:] = system.pos
        system.pos = self._pos_staging
        self._parts_buf = np.zeros(_lib.NPART)
        self._vt_buf = np.zeros(9)
        # bumped whenever the device list is invalidated (cell or scalings)
        self.list_epoch = 0
        self.sync_cell()
        if system.charges is not None:
            self.sync_charges()

    def __del__(self):
        ctx = getattr(self, 'ctx', None)
        if ctx is not None and ctx.value:
            try:
                self.lib.yg_destroy(ctx)
            except Exception:
                pass
            self.ctx = None

    # -- state --
    def set_precision(self, precision):
        if isinstance(precision, str):
            precision = _lib.PRECISIONS[precision]
        if precision != self.precision:
            check(self.lib.yg_set_precision(self.ctx, precision), 'yg_set_precision')
            self.precision = precision

    def sync_cell(self):
        cell = self.system.cell
        key = (cell.nvec, cell.full_rvecs().tobytes())
        if key == self._cell_key:
            return False
        if cell.nvec != 3:
            raise NotImplementedError('the device force path needs a 3D periodic cell (nvec == 3)')
        rv = np.ascontiguousarray(cell.full_rvecs())
        gv = np.ascontiguousarray(cell.full_gvecs())
        check(self.lib.yg_set_cell(self.ctx, ptr(rv), ptr(gv), cell.nvec, float(cell.volume)), 'yg_set_cell')
        self._cell_key = key
        self.list_epoch += 1
        return True

    def sync_charges(self):
        """Uploads the system's charges when they differ from the last upload
        (an element-wise comparison: charges may be changed in place).  Inside
        one ForceField evaluation (call_key set) the comparison runs once."""
        ck = getattr(self, 'call_key', None)
        if ck is not None and ck == getattr(self, '_charges_call', None):
            return
        self._charges_call = ck
        q = self.system.charges
        if self._charges_key is not None and q.shape == self._charges_key.shape and np.array_equal(q, self._charges_key):
            return
        q = np.ascontiguousarray(q, dtype=np.float64)
        check(self.lib.yg_set_charges(self.ctx, ptr(q)), 'yg_set_charges')
        self._charges_key = q.copy()

    def upload_positions(self, pos=None, wait=True):
        """Copies the current positions (host array) to the device.  The copy
        reads the system's own (user-visible, page-locked) positions
        asynchronously; wait=True returns only when it is done, so that the
        caller may write them again.  wait=False is for callers that
        synchronize with the device before returning to user code."""
        src = self.system.pos if pos is None else pos
        if src is not self._pos_staging:
            self._pos_staging[:] = src
        check(self.lib.yg_set_positions(self.ctx, ptr(self._pos_staging), 0), 'yg_set_positions')
        if wait:
            check(self.lib.yg_sync(self.ctx), 'yg_sync')

    def upload_positions_device(self, dptr):
        check(self.lib.yg_set_positions(self.ctx, ctypes.c_void_p(dptr), 1), 'yg_set_positions')

    def set_scalings(self, scalings):
        if self.scalings_obj is scalings:
            return
        st = scalings.stab
        a = np.ascontiguousarray(st['a'], dtype=np.int64)
        b = np.ascontiguousarray(st['b'], dtype=np.int64)
        s = np.ascontiguousarray(st['scale'], dtype=np.float64)
        nb = np.ascontiguousarray(st['nbond'], dtype=np.int64)
        check(self.lib.yg_set_scalings(self.ctx, ptr(a), ptr(b), ptr(s), ptr(nb), len(st)), 'yg_set_scalings')
        self.scalings_obj = scalings
        self.list_epoch += 1

    def register_pair(self, part):
        if part in self.pair_slots:
            return self.pair_slots.index(part)
        if len(self.pair_slots) >= 3:
            raise NotImplementedError('at most three pair potentials per system on the device')
        slot = len(self.pair_slots)
        self.pair_slots.append(part)
        pp = part.pair_pot
        tr = pp.get_truncation()
        trk, trp = (_lib.TR_NONE, 0.0) if tr is None else (tr.kind, tr.par)
        if getattr(pp, 'type_table', False):
            t = pp._device_table(self.natom)
            check(self.lib.yg_set_pair_table(self.ctx, slot, pp.kind, len(t['cross0']), ptr(t['ffatype_ids']),
                                             ptr(t['cross0']), ptr(t['cross1']), ptr(t['cross2']),
                                             int(t['power']), ptr(t['scales']), float(pp.rcut), trk, float(trp)),
                  'yg_set_pair_table')
        else:
            arrs = pp._device_arrays(self.natom)
            check(self.lib.yg_set_pair_pot(self.ctx, slot, pp.kind, ptr(arrs['sigma']), ptr(arrs['epsilon']),
                                           ptr(arrs['onlypauli']), ptr(arrs['radii']), float(arrs['alpha']),
                                           float(arrs['dielectric']), float(pp.rcut), trk, float(trp)),
                  'yg_set_pair_pot')
        if pp.kind == _lib.POT_EI:
            self.sync_charges()
        return slot

    # -- readback --
    def get_part(self, slot, gpos=None, vtens=None):
        e = ctypes.c_double()
        g = None
        if gpos is not None:
            g = gpos if (gpos.flags['C_CONTIGUOUS'] and gpos.dtype == np.float64) else np.zeros((self.natom, 3))
        v = None
        if vtens is not None:
            v = np.zeros(9)
        check(self.lib.yg_get_part(self.ctx, slot, ctypes.byref(e), ptr(g), ptr(v)), 'yg_get_part')
        if gpos is not None and g is not gpos:
            gpos[:] = g
        if vtens is not None:
            vtens[:] = v.reshape(3, 3)
        return e.value

    def get_total(self, mask, gpos=None, vtens=None):
        e = ctypes.c_double()
        parts = np.zeros(_lib.NPART)
        g = None if gpos is None else np.zeros((self.natom, 3))
        v = None if vtens is None else np.zeros(9)
        check(self.lib.yg_get_total(self.ctx, mask, ctypes.byref(e), ptr(g), ptr(v), ptr(parts)), 'yg_get_total')
        return e.value, g, None if v is None else v.reshape(3, 3), parts

    def get_total_into(self, mask, gpos=None, vtens=None):
        """(energy, part energies); the summed gradient is written into gpos
        and the virial into vtens (overwritten, float64 C-contiguous), each
        skipped when None.  Raises ValueError on NaN energy or gradient."""
        e = ctypes.c_double()
        parts = self._parts_buf
        g = gpos
        if g is not None and not (g.flags['C_CONTIGUOUS'] and g.dtype == np.float64):
            g = np.zeros((self.natom, 3))
        v = self._vt_buf if vtens is not None else None
        check(self.lib.yg_get_total(self.ctx, mask, ctypes.byref(e), ptr(g), ptr(v), ptr(parts)), 'yg_get_total')
        if gpos is not None and g is not gpos:
            gpos[:] = g
        if vtens is not None:
            vtens[:] = v.reshape(3, 3)
        return e.value, parts.copy()

    def get_total_add(self, mask, gpos=None, vtens=None):
        """(energy, part energies); the summed gradient is ADDED to gpos and
        the virial to vtens (float64 C-contiguous arrays are added to in
        place by the library), each skipped when None.  Raises ValueError on
        NaN energy or gradient."""
        e = ctypes.c_double()
        parts = self._parts_buf
        g = gpos
        if g is not None and not (g.flags['C_CONTIGUOUS'] and g.dtype == np.float64):
            g = np.zeros((self.natom, 3))
        v = vtens
        if v is not None and not (v.flags['C_CONTIGUOUS'] and v.dtype == np.float64):
            v = np.zeros((3, 3))
        check(self.lib.yg_get_total_add(self.ctx, mask, ctypes.byref(e), ptr(g), ptr(v), ptr(parts)),
              'yg_get_total')
        if gpos is not None and g is not gpos:
            gpos += g
        if vtens is not None and v is not vtens:
            vtens += v
        return e.value, parts.copy()

    def launch_count(self):
        return int(self.lib.yg_launch_count(self.ctx))

    def mem_usage(self):
        """(bytes now, high-water bytes) of device memory this system holds."""
        now, high = ctypes.c_int64(), ctypes.c_int64()
        check(self.lib.yg_mem_usage(self.ctx, ctypes.byref(now), ctypes.byref(high)), 'yg_mem_usage')
        return now.value, high.value

    def destroy(self):
        """Releases the device state now (stream-ordered; no device sync)."""
        ctx = getattr(self, 'ctx', None)
        if ctx is not None and ctx.value:
            check(self.lib.yg_destroy(ctx), 'yg_destroy')
        self.ctx = None

    def sync(self):
        check(self.lib.yg_sync(self.ctx), 'yg_sync')
