"""Line: an ordered sequence of named elements (the part of xtrack/line.py
that the push uses).

Covers ``Line(elements=..., element_names=...)`` (line.py:144-351),
``build_tracker`` (line.py:1537-1620), ``track`` (line.py:1902-1994),
``slice_thick_elements`` (line.py:2232-2274), the tracker config
(line.py:283-287) and ``reset_s_at_end_turn`` / ``skip_end_turn_actions``
(line.py:6817-6851), plus ``to_dict`` / ``from_dict`` for the elements built
here.
"""
import contextlib

import numpy as np

from . import _abi
from . import elements as el
from .particles import Particles
from .slicing import slice_line
from .tracker import Tracker


class TrackerConfig:
    """Compile-time configuration of the reference tracker
    (tracker.py:1696-1728), restricted to the switches the push honours."""

    def __init__(self):
        object.__setattr__(self, "_v", {
            "XTRACK_MULTIPOLE_NO_SYNRAD": True,
            "XTRACK_GLOBAL_XY_LIMIT": 1.0,
            "XTRACK_USE_EXACT_DRIFTS": False,
            "XTRACK_CAVITY_PRESERVE_ANGLE": False,
            "XFIELDS_BB3D_NO_BEAMSTR": True,
            "XFIELDS_BB3D_NO_BHABHA": True,
        })

    def __getattr__(self, k):
        v = object.__getattribute__(self, "_v")
        if k in v:
            return v[k]
        return False

    def __setattr__(self, k, value):
        if k == "XTRACK_MULTIPOLE_NO_SYNRAD" and not value:
            raise NotImplementedError("synchrotron radiation is not supported")
        self._v[k] = value


class Line:
    def __init__(self, elements=None, element_names=None):
        if elements is None:
            elements = []
        if isinstance(elements, dict):
            element_dict = dict(elements)
            if element_names is None:
                element_names = list(element_dict.keys())
        else:
            elements = list(elements)
            if element_names is None:
                element_names = [f"e{ii}" for ii in range(len(elements))]
            if len(element_names) != len(elements):
                raise ValueError("`elements` and `element_names` should have the same length")
            element_dict = {}
            for nn, ee in zip(element_names, elements):
                if nn in element_dict and element_dict[nn] is not ee:
                    raise ValueError(f"duplicate element name {nn}")
                element_dict[nn] = ee
        self.element_dict = element_dict
        self.element_names = list(element_names)
        self.config = TrackerConfig()
        self._extra_config = {"skip_end_turn_actions": False, "reset_s_at_end_turn": True}
        self.particle_ref = None
        self.tracker = None

    # ------------------------------------------------------------------
    @property
    def elements(self):
        return [self.element_dict[n] for n in self.element_names]

    def __getitem__(self, key):
        if isinstance(key, (int, np.integer)):
            return self.element_dict[self.element_names[key]]
        return self.element_dict[key]

    def __len__(self):
        return len(self.element_names)

    @property
    def reset_s_at_end_turn(self):
        return self._extra_config["reset_s_at_end_turn"]

    @reset_s_at_end_turn.setter
    def reset_s_at_end_turn(self, v):
        self._extra_config["reset_s_at_end_turn"] = bool(v)

    @property
    def skip_end_turn_actions(self):
        return self._extra_config["skip_end_turn_actions"]

    @skip_end_turn_actions.setter
    def skip_end_turn_actions(self, v):
        self._extra_config["skip_end_turn_actions"] = bool(v)

    def get_length(self):
        tot = 0.0
        for e in self.elements:
            tot += _element_length(e)
        return tot

    def get_s_elements(self, mode="upstream"):
        s = [0.0]
        for e in self.elements:
            s.append(s[-1] + _element_length(e))
        return s[:-1] if mode == "upstream" else s[1:]

    # ------------------------------------------------------------------
    def _element_records(self):
        recs = np.zeros(len(self.element_names), dtype=_abi.ELEMENT_DTYPE)
        recs["weight"] = 1.0
        recs["order_rel"] = -1
        cache = {}
        for i, name in enumerate(self.element_names):
            e = self.element_dict[name]
            key = id(e)
            if key not in cache:
                cache[key] = e.to_record()
            recs[i] = cache[key]
        return recs

    def build_tracker(self, device=None, arith="exact"):
        """Builds the device lattice (line.py:1537-1620). ``arith``: 'exact'
        (reference operation order) or 'fast' (merged kicks with FMA)."""
        self.tracker = Tracker(self, device=device, arith=arith)
        return self.tracker

    def discard_tracker(self):
        self.tracker = None

    def freeze_longitudinal(self, state=True):
        """Freezes (True) or unfreezes (False) the longitudinal coordinates
        zeta, ptau, delta, rpp and rvv in every following track call
        (line.py:4446-4469: the tracker's FREEZE_VAR_<name> config, whose
        setters become no-ops)."""
        if state not in (True, False):
            raise ValueError("state must be True or False")
        if not self._has_valid_tracker():
            self.build_tracker()
        self.tracker.frozen_longitudinal = state

    def _has_valid_tracker(self):
        return self.tracker is not None and self.tracker.num_elements == len(self.element_names)

    def track(self, particles, ele_start=0, ele_stop=None, num_elements=None, num_turns=None,
              turn_by_turn_monitor=None, freeze_longitudinal=False, time=False,
              with_progress=False, backtrack=False, **kwargs):
        """Tracks ``particles`` in place (line.py:1902-1994).
        ``multi_element_monitor_at``: element names (or '_all_') at which
        x, px, y, py, zeta, delta, s are recorded before the element, every
        turn (tracker.py:1482-1525); the record is
        ``line.record_multi_element_last_track``."""
        unknown = set(kwargs) - {"multi_element_monitor_at"}
        if unknown:
            raise TypeError(f"unexpected arguments {unknown}")
        if not self._has_valid_tracker():
            self.build_tracker(device=particles.device)
        return self.tracker._track(particles, ele_start=ele_start, ele_stop=ele_stop,
                                   num_elements=num_elements, num_turns=num_turns,
                                   turn_by_turn_monitor=turn_by_turn_monitor,
                                   freeze_longitudinal=freeze_longitudinal, time=time,
                                   with_progress=with_progress, backtrack=backtrack,
                                   multi_element_monitor_at=kwargs.get("multi_element_monitor_at"))

    @property
    def record_last_track(self):
        return self.tracker.record_last_track if self.tracker else None

    @property
    def time_last_track(self):
        return self.tracker.time_last_track if self.tracker else None

    @property
    def record_multi_element_last_track(self):
        return self.tracker.record_multi_element_last_track if self.tracker else None

    @property
    def track_flags(self):
        if self.tracker is None:
            raise RuntimeError("build the tracker first")
        return self.tracker.track_flags

    def slice_thick_elements(self, slicing_strategies, _edge_markers=True):
        """Slices thick elements in place (line.py:2232-2274)."""
        self.discard_tracker()
        return slice_line(self, slicing_strategies, _edge_markers=_edge_markers)

    def build_particles(self, particle_ref=None, device=None, **coords):
        """Particles with the reference particle's p0c, mass0 and q0 and the
        given coordinates (the twiss-free part of line.py:2277-...)."""
        ref = particle_ref if particle_ref is not None else self.particle_ref
        if ref is None:
            raise ValueError("particle_ref is required")
        return Particles(p0c=float(ref.p0c[0].item()), mass0=ref.mass0, q0=ref.q0,
                         device=device, **coords)

    # ------------------------------------------------------------------
    def to_dict(self):
        """xtrack-format line dict (serialization.py)."""
        from .serialization import line_to_dict
        return line_to_dict(self)

    @classmethod
    def from_dict(cls, dct):
        """Line from an xtrack-format line dict (as xtrack's Line.to_dict
        writes it, line.py:384-508)."""
        from .serialization import line_from_dict
        return line_from_dict(dct)

    def to_json(self, path):
        from .serialization import save_json
        save_json(self, path)

    @classmethod
    def from_json(cls, path):
        from .serialization import load
        return load(path)


def _element_length(e):
    if isinstance(e, el._Slice):
        if e._kind in (_abi.SLICE_THICK, _abi.SLICE_DRIFT):
            return e._parent.length * e.weight
        return 0.0
    if isinstance(e, el.Multipole):
        return e.length if e.isthick else 0.0
    if getattr(e, "isthick", False):
        return float(getattr(e, "length", 0.0))
    return 0.0


@contextlib.contextmanager
def freeze_longitudinal(line_or_tracker):
    """Context manager that freezes the longitudinal coordinates of a line
    (or tracker) and restores the previous state on exit (line.py:7673-7684)."""
    tr = line_or_tracker
    if isinstance(line_or_tracker, Line):
        if not line_or_tracker._has_valid_tracker():
            line_or_tracker.build_tracker()
        tr = line_or_tracker.tracker
    previous = tr.frozen_longitudinal
    tr.frozen_longitudinal = True
    try:
        yield None
    finally:
        tr.frozen_longitudinal = previous
