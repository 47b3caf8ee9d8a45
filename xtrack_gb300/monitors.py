"""Turn-by-turn ParticlesMonitor (xtrack/monitors/particles_monitor.py).

Record layout and reshaping follow the reference: ``n_records =
(stop_at_turn-start_at_turn) * (part_id_end-part_id_start) * n_repetitions``
records, zero-initialised (particles_monitor.py:101-104), accessed as
``monitor.x[particle, turn]`` (or ``[frame, particle, turn]`` with
repetitions, particles_monitor.py:153-177). The record of a particle at a
turn is written by the push at the start of that turn
(particles_monitor.h:12-77).

``fields`` selects the recorded arrays (default: all of them, as the
reference does); unrecorded fields read back as zeros.
"""
import numpy as np
import torch

from . import _abi
from .particles import DOUBLE_FIELDS, INT_FIELDS, default_device

_RECORDABLE = _abi.PARTICLE_DOUBLE_FIELDS + _abi.PARTICLE_INT_FIELDS


class ParticlesMonitor:
    def __init__(self, start_at_turn=0, stop_at_turn=1, num_particles=None,
                 particle_id_range=None, n_repetitions=None, repetition_period=None,
                 auto_to_numpy=True, fields=None, device=None, ebe_mode=0):
        if particle_id_range is not None:
            if num_particles is not None:
                raise ValueError("give either num_particles or particle_id_range")
            part_id_start, part_id_end = int(particle_id_range[0]), int(particle_id_range[1])
        else:
            if num_particles is None:
                raise ValueError("num_particles or particle_id_range is required")
            part_id_start, part_id_end = 0, int(num_particles)
        if part_id_end - part_id_start < 0:
            raise ValueError("empty particle id range")
        if (repetition_period is None) != (n_repetitions is None):
            raise ValueError("n_repetitions and repetition_period go together")
        if repetition_period is None:
            repetition_period, n_repetitions = -1, 1
        self.start_at_turn = int(start_at_turn)
        self.stop_at_turn = int(stop_at_turn)
        self.part_id_start = part_id_start
        self.part_id_end = part_id_end
        self.n_repetitions = int(n_repetitions)
        self.repetition_period = int(repetition_period)
        self.ebe_mode = int(ebe_mode)
        n_turns = self.stop_at_turn - self.start_at_turn
        self.n_records = n_turns * (part_id_end - part_id_start) * self.n_repetitions
        self.auto_to_numpy = bool(auto_to_numpy)
        self.device = torch.device(device) if device is not None else default_device()
        if fields is None:
            fields = _RECORDABLE
        bad = set(fields) - set(_RECORDABLE)
        if bad:
            raise ValueError(f"fields that cannot be recorded: {bad}")
        self.fields = tuple(fields)
        self.data = {}
        for f in self.fields:
            dtype = torch.int64 if f in INT_FIELDS else torch.float64
            self.data[f] = torch.zeros(self.n_records, dtype=dtype, device=self.device)

    def _xtg_struct(self):
        m = _abi.XtgMonitor()
        m.start_at_turn = self.start_at_turn
        m.stop_at_turn = self.stop_at_turn
        m.part_id_start = self.part_id_start
        m.part_id_end = self.part_id_end
        m.ebe_mode = self.ebe_mode
        m.n_repetitions = self.n_repetitions
        m.repetition_period = self.repetition_period
        m.n_records = self.n_records
        ptrs = {f: t.data_ptr() for f, t in self.data.items()}
        m.data = _abi.particles_struct_from_ptrs(self.n_records, 0.0, 0.0, 0.0, ptrs)
        return m

    def _get(self, name):
        if name in self.data:
            v = self.data[name]
        else:
            dtype = torch.int64 if name in INT_FIELDS else torch.float64
            v = torch.zeros(self.n_records, dtype=dtype, device=self.device)
        if self.auto_to_numpy:
            v = v.cpu().numpy()
        n_cols = self.stop_at_turn - self.start_at_turn
        if n_cols == 0:
            return v.reshape(0, 0) if self.n_repetitions == 1 else v.reshape(self.n_repetitions, 0, 0)
        if self.n_repetitions == 1:
            return v.reshape(self.n_records // n_cols, n_cols)
        n_rows = self.n_records // n_cols // self.n_repetitions
        return v.reshape(self.n_repetitions, n_rows, n_cols)

    def __getattr__(self, name):
        if name in DOUBLE_FIELDS or name in INT_FIELDS:
            return self._get(name)
        raise AttributeError(name)
