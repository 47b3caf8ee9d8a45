"""Monitors: the turn-by-turn ParticlesMonitor
(xtrack/monitors/particles_monitor.py), usable as the tracker's
``turn_by_turn_monitor`` or placed in the line as an element, and the
LastTurnsMonitor and BeamPositionMonitor elements
(xtrack/monitors/last_turns_monitor.py, beam_position_monitor.py).

ParticlesMonitor:

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
import ctypes

import numpy as np
import torch

from . import _abi
from .particles import DOUBLE_FIELDS, INT_FIELDS, default_device

_RECORDABLE = _abi.PARTICLE_DOUBLE_FIELDS + _abi.PARTICLE_INT_FIELDS


class _MonitorElement:
    """Line-element side of a monitor: the record carries the address of an
    xtg_element_monitor descriptor (kept alive by the element) whose buffers
    live on the monitor's device."""
    isthick = False
    _cls = _abi.CLS_MONITOR

    def _descriptor(self):
        raise NotImplementedError

    def to_record(self):
        rec = np.zeros(1, dtype=_abi.ELEMENT_DTYPE)[0]
        rec["weight"] = 1.0
        rec["order_rel"] = -1
        rec["cls"] = _abi.CLS_MONITOR
        desc = self._descriptor()
        # every descriptor handed out stays alive with the element: records
        # built earlier keep pointing at valid memory
        self.__dict__.setdefault("_descs", []).append(desc)
        rec["aux"] = ctypes.addressof(desc)
        return rec

    def copy(self):
        import copy
        return copy.deepcopy(self)


class ParticlesMonitor(_MonitorElement):
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

    def _descriptor(self):
        d = _abi.XtgElementMonitor()
        d.kind = _abi.MON_PARTICLES
        d.particles = self._xtg_struct()
        return d

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


class LastTurnsMonitor(_MonitorElement):
    """Rolling buffer of the last ``n_last_turns`` passes (every
    ``every_n_turns`` turns) of the particles with ids in
    ``particle_id_range`` (last_turns_monitor.py:31-111). ``x``, ``px``,
    ``y``, ``py``, ``delta``, ``zeta`` (float32), ``particle_id`` and
    ``at_turn`` (uint32 in the buffers) read back as arrays of shape
    (num_particles, n_last_turns), oldest pass first."""
    properties = ("particle_id", "at_turn", "x", "px", "y", "py", "delta", "zeta")

    def __init__(self, *, n_last_turns=None, num_particles=None, particle_id_range=None,
                 every_n_turns=1, device=None):
        if num_particles is not None and particle_id_range is None:
            particle_id_start = 0
        elif particle_id_range is not None and num_particles is None:
            particle_id_start = particle_id_range[0]
            num_particles = particle_id_range[1] - particle_id_range[0]
        else:
            raise ValueError("Exactly one of `num_particles` or `particle_id_range` parameters "
                             "must be specified")
        if n_last_turns is None or n_last_turns < 1:
            raise ValueError("n_last_turns must be >= 1")
        self.n_last_turns = int(n_last_turns)
        self.particle_id_start = int(particle_id_start)
        self.num_particles = int(num_particles)
        self.every_n_turns = int(every_n_turns)
        self.device = torch.device(device) if device is not None else default_device()
        size = self.num_particles * self.n_last_turns
        # uint32 in the reference; torch keeps them as int32 bit patterns
        self._buf = {f: torch.zeros(size, dtype=torch.int32 if f in ("particle_id", "at_turn")
                                    else torch.float32, device=self.device)
                     for f in self.properties}
        self._buf["lost_at_offset"] = torch.zeros(self.num_particles, dtype=torch.int32,
                                                  device=self.device)

    def _descriptor(self):
        d = _abi.XtgElementMonitor()
        d.kind = _abi.MON_LAST_TURNS
        d.particle_id_start = self.particle_id_start
        d.num_particles = self.num_particles
        d.n_last_turns = self.n_last_turns
        d.every_n_turns = self.every_n_turns
        b = self._buf
        d.lost_at_offset = b["lost_at_offset"].data_ptr()
        d.lt_particle_id = b["particle_id"].data_ptr()
        d.lt_at_turn = b["at_turn"].data_ptr()
        for f in ("x", "px", "y", "py", "delta", "zeta"):
            setattr(d, "lt_" + f, b[f].data_ptr())
        return d

    def __getattr__(self, attr):
        if attr in LastTurnsMonitor.properties:
            val = self._buf[attr].cpu().numpy()
            if attr in ("particle_id", "at_turn"):
                val = val.view(np.uint32)
            val = val.reshape(self.num_particles, self.n_last_turns)
            off = self._buf["lost_at_offset"].cpu().numpy().view(np.uint32).astype(np.int64) + 1
            r, c = np.ogrid[:val.shape[0], :val.shape[1]]
            c = (c + off[:, np.newaxis]) % val.shape[1]
            return val[r, c]
        raise AttributeError(attr)


def _id_range(particle_id_range, particle_id_start, num_particles):
    if particle_id_range is None:
        return (0 if particle_id_start is None else int(particle_id_start),
                -1 if num_particles is None else int(num_particles))
    if particle_id_start is None and num_particles is None:
        return int(particle_id_range[0]), int(particle_id_range[1] - particle_id_range[0])
    raise ValueError("Parameter `particle_id_range` must not be used together with "
                     "`num_particles` and/or `particle_id_start`")


class BeamPositionMonitor(_MonitorElement):
    """Centroid recorder (beam_position_monitor.py:25-137): per sample slot
    i = round(sampling_frequency * ((at_turn - start_at_turn)/frev -
    zeta/beta0/c)), the count and the sums of x and y of the particles that
    pass; ``x_mean`` / ``y_mean`` are sum / count."""
    properties = ("count", "x_sum", "y_sum")

    def __init__(self, *, particle_id_range=None, particle_id_start=None, num_particles=None,
                 start_at_turn=None, stop_at_turn=None, frev=None, sampling_frequency=None,
                 device=None):
        if particle_id_range is None:
            particle_id_start = 0 if particle_id_start is None else particle_id_start
            num_particles = -1 if num_particles is None else num_particles
        elif particle_id_start is None and num_particles is None:
            particle_id_start = particle_id_range[0]
            num_particles = particle_id_range[1] - particle_id_range[0]
        else:
            raise ValueError("Parameter `particle_id_range` must not be used together with "
                             "`num_particles` and/or `particle_id_start`")
        self.particle_id_start = int(particle_id_start)
        self.num_particles = int(num_particles)
        self.start_at_turn = int(start_at_turn or 0)
        self.stop_at_turn = int(stop_at_turn or 0)
        self.frev = float(frev or 1)
        self.sampling_frequency = float(sampling_frequency or 1)
        self.device = torch.device(device) if device is not None else default_device()
        size = int(round((self.stop_at_turn - self.start_at_turn) * self.sampling_frequency
                         / self.frev))
        self.n_slots = size
        self._buf = {f: torch.zeros(size, dtype=torch.float64, device=self.device)
                     for f in self.properties}

    def _descriptor(self):
        d = _abi.XtgElementMonitor()
        d.kind = _abi.MON_BEAM_POSITION
        d.particle_id_start = self.particle_id_start
        d.num_particles = self.num_particles
        d.start_at_turn = self.start_at_turn
        d.n_slots = self.n_slots
        d.frev = self.frev
        d.sampling_frequency = self.sampling_frequency
        d.count = self._buf["count"].data_ptr()
        d.x_sum = self._buf["x_sum"].data_ptr()
        d.y_sum = self._buf["y_sum"].data_ptr()
        return d

    def __getattr__(self, attr):
        if attr in BeamPositionMonitor.properties:
            return self._buf[attr].cpu().numpy()
        if attr in ("x_mean", "y_mean", "x_cen", "y_cen", "x_centroid", "y_centroid"):
            with np.errstate(invalid="ignore", divide="ignore"):
                return self._buf[attr[0] + "_sum"].cpu().numpy() / self._buf["count"].cpu().numpy()
        raise AttributeError(attr)


class BeamSizeMonitor(BeamPositionMonitor):
    """Beam size recorder (beam_size_monitor.py): the beam position
    monitor's sums plus those of x^2 and y^2 per sample slot; ``x_std`` /
    ``y_std`` from them."""
    properties = ("count", "x_sum", "y_sum", "x2_sum", "y2_sum")

    def __init__(self, **kwargs):
        super().__init__(**kwargs)
        for f in ("x2_sum", "y2_sum"):
            self._buf[f] = torch.zeros(self.n_slots, dtype=torch.float64, device=self.device)

    def _descriptor(self):
        d = super()._descriptor()
        d.kind = _abi.MON_BEAM_SIZE
        d.x2_sum = self._buf["x2_sum"].data_ptr()
        d.y2_sum = self._buf["y2_sum"].data_ptr()
        return d

    def __getattr__(self, attr):
        if attr in BeamSizeMonitor.properties:
            return self._buf[attr].cpu().numpy()
        if attr in ("x_var", "y_var", "x_std", "y_std"):
            c = attr[0]
            with np.errstate(invalid="ignore", divide="ignore"):
                n = self._buf["count"].cpu().numpy()
                mean = self._buf[c + "_sum"].cpu().numpy() / n
                var = self._buf[c + "2_sum"].cpu().numpy() / n - mean ** 2
            return var if attr.endswith("var") else np.sqrt(var)
        return super().__getattr__(attr)


class BeamProfileMonitor(_MonitorElement):
    """Transverse profile recorder (beam_profile_monitor.py): per sample,
    particle counts in ``nx`` bins over ``x_range`` and ``ny`` bins over
    ``y_range``; ``x_intensity`` / ``y_intensity`` have shape
    (sample_size, n)."""
    properties = ("counts_x", "counts_y")

    def __init__(self, *, particle_id_range=None, particle_id_start=None, num_particles=None,
                 start_at_turn=None, stop_at_turn=None, frev=None, sampling_frequency=None,
                 nx=None, x_range=None, ny=None, y_range=None, n=None, range=None, device=None):
        self.particle_id_start, self.num_particles = _id_range(particle_id_range,
                                                               particle_id_start, num_particles)
        self.start_at_turn = int(start_at_turn or 0)
        self.stop_at_turn = int(stop_at_turn or 0)
        self.frev = float(frev or 1)
        self.sampling_frequency = float(sampling_frequency or 1)

        def axis(nv, rv):
            nv = int(nv if nv is not None else (n or 128))
            if rv is None:
                if range is None:
                    raise ValueError("Either `x_range`/`y_range` or `range` must be provided")
                rv = range
            if np.isscalar(rv):
                rv = (-rv / 2, rv / 2)
            return nv, float(rv[0]), (rv[1] - rv[0]) / nv

        self.nx, self.x_min, self.dx = axis(nx, x_range)
        self.ny, self.y_min, self.dy = axis(ny, y_range)
        self.sample_size = int(round((self.stop_at_turn - self.start_at_turn)
                                     * self.sampling_frequency / self.frev))
        self.device = torch.device(device) if device is not None else default_device()
        self._buf = {"counts_x": torch.zeros(self.sample_size * self.nx, dtype=torch.float64,
                                             device=self.device),
                     "counts_y": torch.zeros(self.sample_size * self.ny, dtype=torch.float64,
                                             device=self.device)}

    def _descriptor(self):
        d = _abi.XtgElementMonitor()
        d.kind = _abi.MON_BEAM_PROFILE
        d.particle_id_start = self.particle_id_start
        d.num_particles = self.num_particles
        d.start_at_turn = self.start_at_turn
        d.n_slots = self.sample_size
        d.frev = self.frev
        d.sampling_frequency = self.sampling_frequency
        d.nx, d.ny = self.nx, self.ny
        d.x_min, d.dx, d.y_min, d.dy = self.x_min, self.dx, self.y_min, self.dy
        d.counts_x = self._buf["counts_x"].data_ptr()
        d.counts_y = self._buf["counts_y"].data_ptr()
        return d

    def __getattr__(self, attr):
        if attr in BeamProfileMonitor.properties:
            return self._buf[attr].cpu().numpy()
        if attr in ("x_intensity", "y_intensity"):
            c = attr[0]
            nb = self.nx if c == "x" else self.ny
            return self._buf["counts_" + c].cpu().numpy().reshape(self.sample_size, nb)
        if attr in ("x_edges", "y_edges"):
            c = attr[0]
            nb, lo, d = (self.nx, self.x_min, self.dx) if c == "x" else (self.ny, self.y_min, self.dy)
            return lo + d * np.arange(nb + 1)
        if attr in ("x_grid", "y_grid"):
            e = self.__getattr__(attr[0] + "_edges")
            return 0.5 * (e[1:] + e[:-1])
        raise AttributeError(attr)


class MultiElementMonitor:
    """Coordinates at several elements of the line, every turn
    (multi_element_monitor.py): ``data[turn, particle, coordinate, obs]``
    with coordinates x, px, y, py, zeta, delta, s, filled before each
    observed element. Built by ``Line.track(..., multi_element_monitor_at=
    [...])``."""
    _coord_name_to_index = {"x": 0, "px": 1, "y": 2, "py": 3, "zeta": 4, "delta": 5, "s": 6}

    def __init__(self, start_at_turn, stop_at_turn, part_id_start, part_id_end,
                 at_element_mapping, obs_names, device=None):
        self.start_at_turn = int(start_at_turn)
        self.stop_at_turn = int(stop_at_turn)
        self.part_id_start = int(part_id_start)
        self.part_id_end = int(part_id_end)
        self.obs_names = list(obs_names)
        self._name_to_index = {n: k for k, n in enumerate(self.obs_names)}
        self.device = torch.device(device) if device is not None else default_device()
        self._mapping = torch.as_tensor(np.asarray(at_element_mapping, dtype=np.int64),
                                        device=self.device)
        shape = (self.stop_at_turn - self.start_at_turn, self.part_id_end - self.part_id_start,
                 7, len(self.obs_names))
        self._data = torch.zeros(shape, dtype=torch.float64, device=self.device)

    def _xtg_struct(self):
        m = _abi.XtgMultiElementMonitor()
        m.start_at_turn = self.start_at_turn
        m.stop_at_turn = self.stop_at_turn
        m.part_id_start = self.part_id_start
        m.part_id_end = self.part_id_end
        m.mapping_len = self._mapping.numel()
        m.n_obs = len(self.obs_names)
        m.at_element_mapping = self._mapping.data_ptr()
        m.data = self._data.data_ptr()
        return m

    @property
    def data(self):
        return self._data.cpu().numpy()

    def get(self, coordinate, obs_name=None, particle_id=None, turn=None):
        c = self._coord_name_to_index[coordinate]
        o = slice(None) if obs_name is None else self._name_to_index[obs_name]
        pi = slice(None) if particle_id is None else particle_id - self.part_id_start
        ti = slice(None) if turn is None else turn - self.start_at_turn
        return self.data[ti, pi, c, o]

    def __repr__(self):
        names = self.obs_names if len(self.obs_names) < 5 else self.obs_names[:5] + ["..."]
        return f"MultiElementMonitor(obs_names=[{', '.join(names)}])"
