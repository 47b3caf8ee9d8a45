"""BatchTracker: several lattices that share one element sequence (error
seeds of one ring) tracked in one persistent launch.

The reference tracks each seed with its own ``Line`` and ``Tracker``
(xtrack/tracker.py:1270-1436 per seed, one kernel launch per seed and turn
range). Here every particle carries the index of its seed's lattice and a
single call of ``xtg_track_batch`` pushes all of them: the device work queue
hands out items of one lattice each, so a block stages one lattice's
element table at a time. The turn split, monitor and flags are those of
``Tracker._track``; the result for each particle is the one its seed's own
``Tracker`` gives (same packed records, same kernels).
"""
import ctypes

import numpy as np
import torch

from . import _abi
from .tracker import Tracker


class BatchTracker(Tracker):
    def __init__(self, lines, device=None, arith="exact"):
        lines = list(lines)
        if not lines:
            raise ValueError("BatchTracker needs at least one line")
        n0 = len(lines[0].element_names)
        for k, ln in enumerate(lines):
            if len(ln.element_names) != n0:
                raise ValueError(f"line {k} has {len(ln.element_names)} elements, line 0 {n0}")
        # one lattice per seed; the batch keeps its own copy of their tables
        self._seeds = [Tracker(ln, device=device, arith=arith) for ln in lines]
        first = self._seeds[0]
        for k, t in enumerate(self._seeds[1:], start=1):
            if bytes(t._cfg) != bytes(first._cfg):
                raise ValueError(f"line {k} has a different tracker configuration")
            if not np.isclose(t.line_length, first.line_length, rtol=0, atol=1e-9):
                raise ValueError(f"line {k} has length {t.line_length}, line 0 {first.line_length}")
        self.lines = lines
        self.line = lines[0]
        self.arith = arith
        self.device = first.device
        self._lib = first._lib
        self.track_flags = first.track_flags
        self.frozen_longitudinal = False
        self.num_elements = n0
        self._records = None
        self._cfg = first._cfg
        self.line_length = first.line_length
        arr = (ctypes.c_void_p * len(self._seeds))(*[t._handle.value for t in self._seeds])
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _abi.check(self._lib.xtg_batch_create(arr, len(self._seeds), ctypes.byref(handle)),
                       self._lib)
        self._handle = handle
        self._lattice_index = None
        self.record_last_track = None
        self.time_last_track = None

    @property
    def num_lattices(self):
        return len(self._seeds)

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                self._lib.xtg_batch_destroy(h)
            except Exception:
                pass
            self._handle = None

    def flops_per_particle(self, ele_start=0, num_elements=None):
        return self._seeds[0].flops_per_particle(ele_start, num_elements)

    def get_tuning(self):
        t = _abi.XtgTuning()
        _abi.check(self._lib.xtg_batch_get_tuning(self._handle, ctypes.byref(t)), self._lib)
        return {f: getattr(t, f) for f, _ in _abi.XtgTuning._fields_}

    def set_tuning(self, **kw):
        cur = self.get_tuning()
        unknown = set(kw) - set(cur)
        if unknown:
            raise KeyError(f"unknown tuning keys {unknown}")
        cur.update(kw)
        t = _abi.XtgTuning(**{k: int(v) for k, v in cur.items()})
        _abi.check(self._lib.xtg_batch_set_tuning(self._handle, ctypes.byref(t)), self._lib)
        return cur

    def device_status(self):
        _abi.check(self._lib.xtg_batch_device_status(self._handle), self._lib)

    def _launch(self, pstruct, num_turns, ele_start, num_ele_track, flag_end, flag_monitor,
                mstruct, flags, stream):
        idx = self._lattice_index
        st = self._lib.xtg_track_batch(
            self._handle, ctypes.byref(pstruct), ctypes.c_void_p(idx.data_ptr()),
            int(num_turns), int(ele_start), int(num_ele_track), int(flag_end),
            int(1 if self.line.reset_s_at_end_turn else 0), int(flag_monitor),
            int(self.num_elements), self.line_length,
            ctypes.byref(mstruct) if mstruct is not None else None,
            int(flags), ctypes.c_void_p(stream))
        _abi.check(st, self._lib)

    def track(self, particles, lattice_index, **kwargs):
        """Tracks ``particles``; particle slot i through lattice
        ``lattice_index[i]`` (the seed's position in ``lines``). Takes the
        keyword arguments of ``Line.track``."""
        if kwargs.get("multi_element_monitor_at"):
            raise NotImplementedError("multi_element_monitor_at is not supported for batches")
        idx = torch.as_tensor(lattice_index, dtype=torch.int32, device=particles.device)
        if idx.dim() != 1 or idx.numel() != particles._capacity:
            raise ValueError("lattice_index needs one entry per particle slot "
                             f"({particles._capacity})")
        if idx.numel() and (int(idx.min()) < 0 or int(idx.max()) >= self.num_lattices):
            raise ValueError(f"lattice_index outside [0, {self.num_lattices})")
        self._lattice_index = idx.contiguous()
        try:
            return self._track(particles, **kwargs)
        finally:
            self._lattice_index = None
