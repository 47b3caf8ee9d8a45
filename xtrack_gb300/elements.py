"""Beam elements of the push, with xtrack's constructors and defaults.

Each class keeps the parameters of its xtrack counterpart
(xtrack/beam_elements/*.py ``_xofields``) and fills one raw C-ABI record
(``xtg_element``); the library packs the records into the device table.
Parameter handling follows the reference:
  * knl/ksl padding and ``order`` / ``inv_factorial_order``:
    _common.py:481-546 (``_prepare_multipolar_params``), default order 5
    for the thick magnets (_common.py:18, 426);
  * knl_rel/ksl_rel default ``[0]`` and equal-length padding:
    _common.py:548-557;
  * Bend ``angle``/``length`` -> ``h``, ``k0='from_h'``: _common.py:619-690;
  * model / integrator / edge-model names: _common.py:20-80;
  * LimitEllipse a, b -> a_squ, b_squ, a_b_squ: limit_ellipse.py:45-64.
"""
import math

import numpy as np

from . import _abi

DEFAULT_MULTIPOLE_ORDER = 5
UNLIMITED = 1e10                        # beam_elements/_aperture_common.py:6

MODEL_CURVED = {
    "adaptive": 0, "full": 1, "bend-kick-bend": 2, "rot-kick-rot": 3,
    "mat-kick-mat": 4, "drift-kick-drift-exact": 5, "drift-kick-drift-expanded": 6,
    "rot-kick-rot-low-order": 7, "rot-kick-rot-high-order": 8, "expanded": 4,
}
MODEL_STRAIGHT = {k: v for k, v in MODEL_CURVED.items() if v not in (2, 3)}
MODEL_RF = {k: v for k, v in MODEL_STRAIGHT.items() if v not in (1, 4)}
MODEL_DRIFT = {"adaptive": 0, "expanded": 1, "exact": 2}
INTEGRATORS = {"adaptive": 0, "teapot": 1, "yoshida4": 2, "uniform": 3}
EDGE_MODELS = {"suppressed": -1, "linear": 0, "full": 1, "dipole-only": 2}


def _index(table, value, what):
    if isinstance(value, (int, np.integer)):
        return int(value)
    try:
        return table[value]
    except KeyError:
        raise ValueError(f"Invalid {what}: {value}") from None


def _name_of(table, index):
    for k, v in table.items():
        if v == index and k != "expanded":
            return k
    return index


class BeamElement:
    """Base of all elements: holds parameters, fills a C-ABI record."""
    isthick = False
    _cls = None

    def _fill(self, rec):
        raise NotImplementedError

    def to_record(self):
        rec = np.zeros(1, dtype=_abi.ELEMENT_DTYPE)[0]
        rec["weight"] = 1.0
        rec["order_rel"] = -1
        self._fill(rec)
        # transverse shift and tilt (apertures, thin multipoles, dipole
        # edges: track_local_particle_with_transformations.h)
        for f in ("shift_x", "shift_y", "rot_s_rad", "rot_s_rad_no_frame"):
            rec[f] = getattr(self, f, 0.0)
        return rec

    def copy(self):
        import copy
        return copy.deepcopy(self)

    def __repr__(self):
        return f"{type(self).__name__}({', '.join(f'{k}={v!r}' for k, v in self._repr_items())})"

    def _repr_items(self):
        return []


class Marker(BeamElement):
    """Marker (beam_elements/marker.py): no effect, counts as an element."""
    _cls = _abi.CLS_MARKER

    def _fill(self, rec):
        rec["cls"] = self._cls


class Drift(BeamElement):
    """Drift (drift.py:14-76). ``model``: 'adaptive' (-> expanded), 'expanded', 'exact'."""
    isthick = True
    _cls = _abi.CLS_DRIFT

    def __init__(self, length=0.0, model="adaptive"):
        self.length = float(length)
        self.model = model

    @property
    def model(self):
        return _name_of(MODEL_DRIFT, self._model)

    @model.setter
    def model(self, value):
        self._model = _index(MODEL_DRIFT, value, "drift model")

    def _fill(self, rec):
        rec["cls"] = self._cls
        rec["length"] = self.length
        rec["model"] = self._model

    def _repr_items(self):
        return [("length", self.length)]


def _multipolar(order, knl, ksl, default_order):
    """_common.py:481-546 (_prepare_multipolar_params)."""
    order = order if order else default_order
    order = order or 0
    lengths = [len(v) for v in (knl, ksl) if v is not None]
    target_len = max([order + 1] + lengths)
    out = []
    for v in (knl, ksl):
        a = np.zeros(target_len, dtype=np.float64)
        if v is not None:
            a[:len(v)] = np.asarray(v, dtype=np.float64)
        out.append(a)
    order = target_len - 1
    return order, out[0], out[1], 1.0 / math.factorial(order)


def _rel(knl_rel, ksl_rel):
    """_common.py:548-557 (_handle_knl_ksl_rel_kwargs)."""
    knl_rel = [0.0] if knl_rel is None else list(knl_rel)
    ksl_rel = [0.0] if ksl_rel is None else list(ksl_rel)
    n = max(len(knl_rel), len(ksl_rel))
    knl_rel = knl_rel + [0.0] * (n - len(knl_rel))
    ksl_rel = ksl_rel + [0.0] * (n - len(ksl_rel))
    return np.asarray(knl_rel, dtype=np.float64), np.asarray(ksl_rel, dtype=np.float64)


class _Magnet(BeamElement):
    """Common part of the magnet classes (knl/ksl, knl_rel/ksl_rel, model,
    integrator, number of kicks)."""
    _models = MODEL_STRAIGHT

    def _init_common(self, order, knl, ksl, knl_rel, ksl_rel, model, integrator,
                     num_multipole_kicks, default_order):
        self._order, self.knl, self.ksl, self.inv_factorial_order = _multipolar(
            order, knl, ksl, default_order)
        self.knl_rel, self.ksl_rel = _rel(knl_rel, ksl_rel)
        self.model = model
        self.integrator = integrator
        self.num_multipole_kicks = int(num_multipole_kicks)

    @property
    def order(self):
        return self._order

    @property
    def model(self):
        return _name_of(self._models, self._model)

    @model.setter
    def model(self, value):
        self._model = _index(self._models, value, "model")

    @property
    def integrator(self):
        return _name_of(INTEGRATORS, self._integrator)

    @integrator.setter
    def integrator(self, value):
        self._integrator = _index(INTEGRATORS, value, "integrator")

    def _fill_common(self, rec):
        rec["cls"] = self._cls
        rec["model"] = self._model
        rec["integrator"] = self._integrator
        rec["num_multipole_kicks"] = self.num_multipole_kicks
        rec["order"] = self._order
        rec["inv_factorial_order"] = self.inv_factorial_order
        if self._order + 1 > _abi.XTG_MAX_KNL or len(self.knl_rel) > 20:
            raise ValueError("multipole order above the supported maximum "
                             f"(knl up to {_abi.XTG_MAX_KNL - 1}, knl_rel up to 19)")
        rec["knl"][:self._order + 1] = self.knl
        rec["ksl"][:self._order + 1] = self.ksl
        rec["order_rel"] = len(self.knl_rel) - 1
        rec["knl_rel"][:len(self.knl_rel)] = self.knl_rel
        rec["ksl_rel"][:len(self.ksl_rel)] = self.ksl_rel


class Multipole(_Magnet):
    """Multipole (multipole.py:26-206). Thin (kick only) unless ``isthick``."""
    _cls = _abi.CLS_MULTIPOLE

    def __init__(self, knl=None, ksl=None, order=None, hxl=0.0, length=0.0, isthick=False,
                 knl_rel=None, ksl_rel=None, main_order=0, main_is_skew=False,
                 num_multipole_kicks=0, model="adaptive", integrator="adaptive", shift_x=0.0,
                 shift_y=0.0, rot_s_rad=0.0, rot_s_rad_no_frame=0.0):
        self._init_common(order, knl, ksl, knl_rel, ksl_rel, model, integrator,
                          num_multipole_kicks, default_order=0)
        # transverse shift and tilt: thin multipoles only (a thick one is
        # rejected when the tracker is built)
        self.shift_x = float(shift_x)
        self.shift_y = float(shift_y)
        self.rot_s_rad = float(rot_s_rad)
        self.rot_s_rad_no_frame = float(rot_s_rad_no_frame)
        self.hxl = float(hxl)
        self.length = float(length)
        self._isthick = bool(isthick)
        self.main_order = int(main_order)
        self.main_is_skew = bool(main_is_skew)

    @property
    def isthick(self):
        return self._isthick

    @isthick.setter
    def isthick(self, value):
        self._isthick = bool(value)

    def _fill(self, rec):
        self._fill_common(rec)
        rec["hxl"] = self.hxl
        rec["length"] = self.length
        rec["isthick"] = 1 if self._isthick else 0
        rec["main_order"] = self.main_order
        rec["main_is_skew"] = 1 if self.main_is_skew else 0

    def _repr_items(self):
        return [("knl", self.knl.tolist()), ("ksl", self.ksl.tolist())]


class Bend(_Magnet):
    """Sector bend (bend.py:24-124, fields _common.py:561-690).

    ``k0`` defaults to 'from_h' (k0 = h = angle/length). Edges are active
    with the linear model by default (only 'linear' and 'suppressed' edge
    models are built)."""
    isthick = True
    _cls = _abi.CLS_BEND
    _models = MODEL_CURVED

    def __init__(self, length=0.0, angle=0.0, k0="from_h", k1=0.0, k2=0.0, knl=None, ksl=None,
                 order=None, knl_rel=None, ksl_rel=None, model="adaptive",
                 integrator="adaptive", num_multipole_kicks=0,
                 edge_entry_active=True, edge_exit_active=True,
                 edge_entry_model="linear", edge_exit_model="linear",
                 edge_entry_angle=0.0, edge_exit_angle=0.0,
                 edge_entry_angle_fdown=0.0, edge_exit_angle_fdown=0.0,
                 edge_entry_fint=0.0, edge_exit_fint=0.0,
                 edge_entry_hgap=0.0, edge_exit_hgap=0.0):
        self._init_common(order, knl, ksl, knl_rel, ksl_rel, model, integrator,
                          num_multipole_kicks, default_order=DEFAULT_MULTIPOLE_ORDER)
        self.k1 = float(k1)
        self.k2 = float(k2)
        self._length = float(length)
        self._angle = float(angle)
        self._k0_from_h = True
        self._k0 = 0.0
        self._update_h()
        self.k0 = k0
        self.edge_entry_active = int(bool(edge_entry_active))
        self.edge_exit_active = int(bool(edge_exit_active))
        self.edge_entry_model = edge_entry_model
        self.edge_exit_model = edge_exit_model
        self.edge_entry_angle = float(edge_entry_angle)
        self.edge_exit_angle = float(edge_exit_angle)
        self.edge_entry_angle_fdown = float(edge_entry_angle_fdown)
        self.edge_exit_angle_fdown = float(edge_exit_angle_fdown)
        self.edge_entry_fint = float(edge_entry_fint)
        self.edge_exit_fint = float(edge_exit_fint)
        self.edge_entry_hgap = float(edge_entry_hgap)
        self.edge_exit_hgap = float(edge_exit_hgap)

    def _update_h(self):
        self._h = self._angle / self._length if self._length != 0 else 0.0
        if self._k0_from_h:
            self._k0 = self._h

    @property
    def length(self):
        return self._length

    @length.setter
    def length(self, v):
        self._length = float(v)
        self._update_h()

    @property
    def angle(self):
        return self._angle

    @angle.setter
    def angle(self, v):
        self._angle = float(v)
        self._update_h()

    @property
    def h(self):
        return self._h

    @property
    def k0(self):
        return "from_h" if self._k0_from_h else self._k0

    @k0.setter
    def k0(self, value):
        if isinstance(value, str):
            if value != "from_h":
                raise ValueError("k0 can only be set to 'from_h' as a string")
            self._k0_from_h = True
            self._k0 = self._h
        else:
            self._k0_from_h = False
            self._k0 = float(value)

    @property
    def edge_entry_model(self):
        return _name_of(EDGE_MODELS, self._edge_entry_model)

    @edge_entry_model.setter
    def edge_entry_model(self, v):
        self._edge_entry_model = _index(EDGE_MODELS, v, "edge model")

    @property
    def edge_exit_model(self):
        return _name_of(EDGE_MODELS, self._edge_exit_model)

    @edge_exit_model.setter
    def edge_exit_model(self, v):
        self._edge_exit_model = _index(EDGE_MODELS, v, "edge model")

    def _fill(self, rec):
        self._fill_common(rec)
        rec["length"] = self._length
        rec["h"] = self._h
        rec["k0"] = self._k0
        rec["k1"] = self.k1
        rec["k2"] = self.k2
        rec["edge_entry_active"] = self.edge_entry_active
        rec["edge_exit_active"] = self.edge_exit_active
        rec["edge_entry_model"] = self._edge_entry_model
        rec["edge_exit_model"] = self._edge_exit_model
        for f in ("edge_entry_angle", "edge_exit_angle", "edge_entry_angle_fdown",
                  "edge_exit_angle_fdown", "edge_entry_fint", "edge_exit_fint",
                  "edge_entry_hgap", "edge_exit_hgap"):
            rec[f] = getattr(self, f)

    def _repr_items(self):
        return [("length", self._length), ("angle", self._angle), ("k0", self.k0)]


class _StraightMagnet(_Magnet):
    isthick = True
    _main = None

    def __init__(self, length=0.0, knl=None, ksl=None, order=None, knl_rel=None, ksl_rel=None,
                 main_is_skew=False, model="adaptive", integrator="adaptive",
                 num_multipole_kicks=0, edge_entry_active=False, edge_exit_active=False, **k):
        self._init_common(order, knl, ksl, knl_rel, ksl_rel, model, integrator,
                          num_multipole_kicks, default_order=DEFAULT_MULTIPOLE_ORDER)
        self.length = float(length)
        self.main_is_skew = bool(main_is_skew)
        self.edge_entry_active = int(bool(edge_entry_active))
        self.edge_exit_active = int(bool(edge_exit_active))
        n, s = self._main
        setattr(self, n, float(k.pop(n, 0.0)))
        setattr(self, s, float(k.pop(s, 0.0)))
        if k:
            raise NameError(f"Invalid argument(s): {set(k)}")

    def _fill(self, rec):
        self._fill_common(rec)
        rec["length"] = self.length
        rec["main_is_skew"] = 1 if self.main_is_skew else 0
        rec["edge_entry_active"] = self.edge_entry_active
        rec["edge_exit_active"] = self.edge_exit_active
        n, s = self._main
        rec[n] = getattr(self, n)
        rec[s] = getattr(self, s)

    def _repr_items(self):
        n, _ = self._main
        return [("length", self.length), (n, getattr(self, n))]


class Quadrupole(_StraightMagnet):
    """Quadrupole (quadrupole.py:24-146): k1, k1s; default model mat-kick-mat."""
    _cls = _abi.CLS_QUADRUPOLE
    _main = ("k1", "k1s")


class Sextupole(_StraightMagnet):
    """Sextupole (sextupole.py): k2, k2s; default drift-kick-drift-expanded."""
    _cls = _abi.CLS_SEXTUPOLE
    _main = ("k2", "k2s")


class Octupole(_StraightMagnet):
    """Octupole (octupole.py): k3, k3s; default drift-kick-drift-expanded."""
    _cls = _abi.CLS_OCTUPOLE
    _main = ("k3", "k3s")


class Cavity(BeamElement):
    """Cavity (cavity.py:24-200). ``frequency`` [Hz] or ``harmonic``, ``lag``
    [deg], ``phase`` [rad], ``voltage`` [V]."""
    isthick = True
    _cls = _abi.CLS_CAVITY

    def __init__(self, voltage=0.0, frequency=0.0, lag=0.0, phase=0.0, harmonic=0.0,
                 length=0.0, absolute_time=0, num_kicks=0, model="adaptive",
                 integrator="adaptive"):
        if frequency != 0 and harmonic != 0:
            raise ValueError("Cannot set non-zero frequency when harmonic is not zero.")
        self.voltage = float(voltage)
        self.frequency = float(frequency)
        self.harmonic = float(harmonic)
        self.lag = float(lag)
        self.phase = float(phase)
        self.length = float(length)
        self.absolute_time = int(absolute_time)
        self.num_kicks = int(num_kicks)
        self.model = model
        self.integrator = integrator

    @property
    def model(self):
        return _name_of(MODEL_RF, self._model)

    @model.setter
    def model(self, value):
        self._model = _index(MODEL_RF, value, "model")

    @property
    def integrator(self):
        return _name_of(INTEGRATORS, self._integrator)

    @integrator.setter
    def integrator(self, value):
        self._integrator = _index(INTEGRATORS, value, "integrator")

    def _fill(self, rec):
        rec["cls"] = self._cls
        rec["length"] = self.length
        rec["voltage"] = self.voltage
        rec["frequency"] = self.frequency
        rec["harmonic"] = self.harmonic
        rec["lag"] = self.lag
        rec["phase"] = self.phase
        rec["absolute_time"] = self.absolute_time
        rec["num_multipole_kicks"] = self.num_kicks
        rec["model"] = self._model
        rec["integrator"] = self._integrator

    def _repr_items(self):
        return [("voltage", self.voltage), ("frequency", self.frequency), ("lag", self.lag)]


class LimitEllipse(BeamElement):
    """Elliptical aperture (limit_ellipse.py:12-94)."""
    _cls = _abi.CLS_LIMIT_ELLIPSE

    def __init__(self, a=None, b=None, a_squ=None, b_squ=None, a_b_squ=None, shift_x=0.0,
                 shift_y=0.0, rot_s_rad=0.0,
                 rot_s_rad_no_frame=0.0):
        self.shift_x = float(shift_x)
        self.shift_y = float(shift_y)
        self.rot_s_rad = float(rot_s_rad)
        self.rot_s_rad_no_frame = float(rot_s_rad_no_frame)
        if a is None and a_squ is None:
            a = UNLIMITED
        if b is None and b_squ is None:
            b = UNLIMITED
        if a is not None:
            a_squ = a * a
        if b is not None:
            b_squ = b * b
        if a_b_squ is None:
            a_b_squ = a_squ * b_squ
        if not (a_squ > 0.0 and b_squ > 0.0):
            raise ValueError("a_squ and b_squ have to be positive definite")
        self.a_squ = float(a_squ)
        self.b_squ = float(b_squ)
        self.a_b_squ = float(a_b_squ)

    @property
    def a(self):
        return math.sqrt(self.a_squ)

    @property
    def b(self):
        return math.sqrt(self.b_squ)

    def _fill(self, rec):
        rec["cls"] = self._cls
        rec["a_squ"] = self.a_squ
        rec["b_squ"] = self.b_squ
        rec["a_b_squ"] = self.a_b_squ

    def _repr_items(self):
        return [("a", self.a), ("b", self.b)]


class LimitRectEllipse(BeamElement):
    """Intersection of a symmetric rectangle and an ellipse
    (limit_rect_ellipse.py; limitrectellipse.h:14-44): lost outside
    |x| <= max_x, |y| <= max_y or x^2 b^2 + y^2 a^2 <= a^2 b^2."""
    _cls = _abi.CLS_LIMIT_RECT_ELLIPSE

    def __init__(self, max_x=UNLIMITED, max_y=UNLIMITED, a_squ=None, b_squ=None, a=None, b=None,
                 a_b_squ=None, shift_x=0.0, shift_y=0.0, rot_s_rad=0.0,
                 rot_s_rad_no_frame=0.0):
        self.shift_x = float(shift_x)
        self.shift_y = float(shift_y)
        self.rot_s_rad = float(rot_s_rad)
        self.rot_s_rad_no_frame = float(rot_s_rad_no_frame)
        if a is None and a_squ is None:
            a = UNLIMITED
        if b is None and b_squ is None:
            b = UNLIMITED
        if a is not None:
            a_squ = a * a
        if b is not None:
            b_squ = b * b
        if max_x < 0.0 or max_y < 0.0:
            raise ValueError("max_x and max_y have to be positive definite")
        if a_squ < 0.0 or b_squ < 0.0:
            raise ValueError("a_squ and b_squ have to be positive definite")
        self.max_x = float(max_x)
        self.max_y = float(max_y)
        self.a_squ = float(a_squ)
        self.b_squ = float(b_squ)
        self.a_b_squ = float(a_squ * b_squ if a_b_squ is None else a_b_squ)

    @property
    def a(self):
        return math.sqrt(self.a_squ)

    @property
    def b(self):
        return math.sqrt(self.b_squ)

    def _fill(self, rec):
        rec["cls"] = self._cls
        for f in ("max_x", "max_y", "a_squ", "b_squ", "a_b_squ"):
            rec[f] = getattr(self, f)

    def _repr_items(self):
        return [("max_x", self.max_x), ("max_y", self.max_y), ("a", self.a), ("b", self.b)]


class LimitRect(BeamElement):
    """Rectangular aperture (limit_rect.py)."""
    _cls = _abi.CLS_LIMIT_RECT

    def __init__(self, min_x=-UNLIMITED, max_x=UNLIMITED, min_y=-UNLIMITED, max_y=UNLIMITED,
                 shift_x=0.0, shift_y=0.0, rot_s_rad=0.0,
                 rot_s_rad_no_frame=0.0):
        self.shift_x = float(shift_x)
        self.shift_y = float(shift_y)
        self.rot_s_rad = float(rot_s_rad)
        self.rot_s_rad_no_frame = float(rot_s_rad_no_frame)
        self.min_x = float(min_x)
        self.max_x = float(max_x)
        self.min_y = float(min_y)
        self.max_y = float(max_y)

    def _fill(self, rec):
        rec["cls"] = self._cls
        for f in ("min_x", "max_x", "min_y", "max_y"):
            rec[f] = getattr(self, f)

    def _repr_items(self):
        return [("min_x", self.min_x), ("max_x", self.max_x),
                ("min_y", self.min_y), ("max_y", self.max_y)]


class DipoleEdge(BeamElement):
    """Thin dipole edge (dipole_edge.py; dipoleedge.h:14-71). ``model``:
    'linear' (px += chi r21 x, py += chi r43 y), 'full' (y-rotation by the
    face angle, dipole fringe, wedge; backtracking kills) or 'suppressed';
    ``side``: 'entry' or 'exit'. r21 and r43 follow the class's own
    _update_r21_r43 (numpy, from k, e1, e1_fd, hgap, fint) and are
    recomputed whenever one of those changes."""
    _cls = _abi.CLS_DIPOLE_EDGE
    _MODELS = {"linear": 0, "full": 1, "suppressed": -1}
    _SIDES = {"entry": 0, "exit": 1}

    def __init__(self, k=None, e1=None, e1_fd=None, hgap=None, fint=None, model=None,
                 side=None, h=None, shift_x=0.0, shift_y=0.0, rot_s_rad=0.0,
                 rot_s_rad_no_frame=0.0):
        self.shift_x = float(shift_x)
        self.shift_y = float(shift_y)
        self.rot_s_rad = float(rot_s_rad)
        self.rot_s_rad_no_frame = float(rot_s_rad_no_frame)
        if h is not None:
            if k is not None:
                raise ValueError("give k or its older name h, not both")
            k = h
        self._k = float(k) if k is not None else 0.0
        self._e1 = float(e1) if e1 is not None else 0.0
        self._e1_fd = float(e1_fd) if e1_fd is not None else 0.0
        self._hgap = float(hgap) if hgap is not None else 0.0
        self._fint = float(fint) if fint is not None else 0.0
        self._model = 0
        self._side = 0
        if model is not None:
            self.model = model
        if side is not None:
            self.side = side
        self._update_r21_r43()

    def _update_r21_r43(self):
        k, e1 = np.float64(self._k), np.float64(self._e1)
        corr = np.float64(2.0) * k * np.float64(self._hgap) * np.float64(self._fint)
        r21 = k * np.tan(e1)
        e1_v = e1 + np.float64(self._e1_fd)
        temp = corr / np.cos(e1_v) * (np.float64(1) + np.sin(e1_v) * np.sin(e1_v))
        r43 = -k * np.tan(e1_v - temp)
        self.r21 = float(r21)
        self.r43 = float(r43)

    def _param(name):
        def get(self):
            return getattr(self, "_" + name)

        def set_(self, value):
            setattr(self, "_" + name, float(value))
            self._update_r21_r43()
        return property(get, set_)

    k = _param("k")
    e1 = _param("e1")
    e1_fd = _param("e1_fd")
    hgap = _param("hgap")
    fint = _param("fint")
    del _param

    @property
    def model(self):
        return {v: k for k, v in self._MODELS.items()}[self._model]

    @model.setter
    def model(self, value):
        if isinstance(value, str):
            if value not in self._MODELS:
                raise ValueError(f"model must be one of {list(self._MODELS)}")
            value = self._MODELS[value]
        if int(value) not in self._MODELS.values():
            raise ValueError(f"model must be one of {list(self._MODELS)}")
        self._model = int(value)

    @property
    def side(self):
        return {v: k for k, v in self._SIDES.items()}[self._side]

    @side.setter
    def side(self, value):
        if isinstance(value, str):
            if value not in self._SIDES:
                raise ValueError("side must be 'entry' or 'exit'")
            value = self._SIDES[value]
        if int(value) not in (0, 1):
            raise ValueError("side must be 'entry' or 'exit'")
        self._side = int(value)

    def _fill(self, rec):
        rec["cls"] = self._cls
        rec["model"] = self._model
        rec["side"] = self._side
        for f in ("k", "e1", "hgap", "fint", "r21", "r43"):
            rec[f] = getattr(self, f)

    def _repr_items(self):
        return [("k", self.k), ("e1", self.e1), ("e1_fd", self.e1_fd), ("hgap", self.hgap),
                ("fint", self.fint), ("model", self.model), ("side", self.side)]


class LimitPolygon(BeamElement):
    """Polygonal aperture (limit_polygon.py): a particle survives when the
    crossing-number test puts (x, y) inside the closed polygon of the
    vertices (limitpolygon.h:13-90)."""
    _cls = _abi.CLS_LIMIT_POLYGON

    def __init__(self, x_vertices=None, y_vertices=None, shift_x=0.0, shift_y=0.0, rot_s_rad=0.0,
                 rot_s_rad_no_frame=0.0):
        self.shift_x = float(shift_x)
        self.shift_y = float(shift_y)
        self.rot_s_rad = float(rot_s_rad)
        self.rot_s_rad_no_frame = float(rot_s_rad_no_frame)
        x = np.ascontiguousarray(x_vertices, dtype=np.float64)
        y = np.ascontiguousarray(y_vertices, dtype=np.float64)
        if x.shape != y.shape or x.ndim != 1 or len(x) < 3:
            raise ValueError("LimitPolygon needs matching x/y vertex arrays of length >= 3")
        xc, yc = np.append(x, x[0]), np.append(y, y[0])
        if not np.all(np.hypot(np.diff(xc), np.diff(yc)) > 0):
            raise ValueError("LimitPolygon has repeated consecutive vertices")
        self.x_vertices = x
        self.y_vertices = y

    @property
    def x_closed(self):
        return np.append(self.x_vertices, self.x_vertices[0])

    @property
    def y_closed(self):
        return np.append(self.y_vertices, self.y_vertices[0])

    def get_area(self, signed=False):
        """Shoelace formula."""
        x, y = self.x_closed, self.y_closed
        a = 0.5 * np.sum(x[:-1] * y[1:] - x[1:] * y[:-1])
        return a if signed else abs(a)

    @property
    def area(self):
        return self.get_area()

    def impact_point_and_normal(self, x_in, y_in, z_in, x_out, y_out, z_out):
        """First crossing of each segment (in -> out) with the polygon's
        boundary and the unit normal of the edge crossed, with the
        reference's orientation (limit_polygon.py: (-dy, dx) along the edge
        of a counter-clockwise polygon, i.e. pointing inwards): returns x, y,
        z of the crossings, Nx, Ny, and the index of the edge."""
        x_in, y_in, z_in = (np.atleast_1d(np.asarray(v, dtype=np.float64)) for v in (x_in, y_in, z_in))
        x_out, y_out, z_out = (np.atleast_1d(np.asarray(v, dtype=np.float64))
                               for v in (x_out, y_out, z_out))
        xc, yc = self.x_closed, self.y_closed
        ex, ey = np.diff(xc), np.diff(yc)
        nx, ny = -ey, ex
        if self.get_area(signed=True) < 0:
            nx, ny = -nx, -ny
        norm = np.hypot(nx, ny)
        nx, ny = nx / norm, ny / norm
        n = len(x_in)
        out = [np.zeros(n) for _ in range(5)]
        found = np.full(n, -1, dtype=np.int64)
        for k in range(n):
            dx, dy = x_out[k] - x_in[k], y_out[k] - y_in[k]
            best = np.inf
            for i in range(len(ex)):
                den = dx * ey[i] - dy * ex[i]
                if den == 0:
                    continue
                wx, wy = xc[i] - x_in[k], yc[i] - y_in[k]
                t = (wx * ey[i] - wy * ex[i]) / den      # along the segment
                u = (wx * dy - wy * dx) / den            # along the edge
                # rays through a vertex hit both neighbouring edges at
                # their ends: accept the end points within rounding
                if -1e-12 <= t <= 1 + 1e-12 and -1e-12 <= u <= 1 + 1e-12 and t < best:
                    best = t
                    found[k] = i
            if found[k] >= 0:
                t = best
                i = found[k]
                out[0][k] = x_in[k] + t * dx
                out[1][k] = y_in[k] + t * dy
                out[2][k] = z_in[k] + t * (z_out[k] - z_in[k])
                out[3][k] = nx[i]
                out[4][k] = ny[i]
        if np.any(found < 0):
            raise ValueError("a segment does not cross the polygon")
        return out[0], out[1], out[2], out[3], out[4], found

    def _fill(self, rec):
        import ctypes
        rec["cls"] = self._cls
        desc = _abi.XtgPolygon(len(self.x_vertices), self.x_vertices.ctypes.data,
                               self.y_vertices.ctypes.data)
        self.__dict__.setdefault("_descs", []).append(desc)
        rec["aux"] = ctypes.addressof(desc)

    def _repr_items(self):
        return [("n_vertices", len(self.x_vertices))]


# ---------------------------------------------------------------------------
# Slices (slice_elements_thick.py, slice_elements_thin.py,
# slice_elements_drift.py, slice_elements_edge.py): a slice refers to its
# parent and adds its own weight; the record carries the parent's
# parameters with the slice kind and weight.
# ---------------------------------------------------------------------------
class _Slice(BeamElement):
    _kind = _abi.SLICE_NONE

    def __init__(self, _parent, weight=1.0, parent_name=None):
        self._parent = _parent
        self.weight = float(weight)
        self.parent_name = parent_name

    @property
    def isthick(self):
        return self._kind in (_abi.SLICE_THICK, _abi.SLICE_DRIFT)

    def _fill(self, rec):
        self._parent._fill(rec)
        rec["slice"] = self._kind
        rec["weight"] = self.weight

    def _repr_items(self):
        return [("parent", self.parent_name), ("weight", self.weight)]


def _make_slice_classes():
    out = {}
    kinds = {"ThickSlice": _abi.SLICE_THICK, "ThinSlice": _abi.SLICE_THIN,
             "DriftSlice": _abi.SLICE_DRIFT}
    for parent in ("Bend", "Quadrupole", "Sextupole", "Octupole", "Multipole", "Cavity"):
        for prefix, kind in kinds.items():
            name = prefix + parent
            out[name] = type(name, (_Slice,), {"_kind": kind})
        if parent not in ("Multipole", "Cavity"):
            out[f"ThinSlice{parent}Entry"] = type(f"ThinSlice{parent}Entry", (_Slice,),
                                                  {"_kind": _abi.SLICE_ENTRY})
            out[f"ThinSlice{parent}Exit"] = type(f"ThinSlice{parent}Exit", (_Slice,),
                                                 {"_kind": _abi.SLICE_EXIT})
    return out


_SLICE_CLASSES = _make_slice_classes()
globals().update(_SLICE_CLASSES)


def slice_class(parent, prefix, suffix=""):
    """Slice class named <prefix><ParentClass><suffix> (e.g. ThickSliceBend)."""
    return _SLICE_CLASSES.get(prefix + type(parent).__name__ + suffix)


__all__ = ["Marker", "Drift", "Multipole", "Bend", "Quadrupole", "Sextupole", "Octupole",
           "Cavity", "LimitEllipse", "LimitRect", "LimitRectEllipse", "LimitPolygon", "DipoleEdge",
           "BeamElement",
           "slice_class"] + sorted(_SLICE_CLASSES)
