"""Line and element dictionaries in xtrack's format, and JSON files.

``element_to_dict`` writes, and ``element_from_dict`` reads, the
dictionaries xtrack's elements produce with ``to_dict`` (a ``__class__``
key plus the ``_xofields`` by their public names: beam_elements/
_common.py:405-418 for the multipolar classes, 720-735 for Bend, slice_base.py:
33-41 for slices), so a line saved by xtrack (``line.to_json``, a
``{"line": ..., "particle": ...}`` test fixture) loads here and a line saved
here loads in xtrack. Fields outside the push's scope must hold their
neutral value (misalignments zero, no radiation, no tapering); any other
value raises, naming the element and the field.

``load`` follows xtrack/load.py:49 for JSON: a file holding a line, or a
dict with a ``line`` entry.
"""
import json

import numpy as np

from . import elements as el

# fields that must keep their neutral value: name -> neutral value
_NEUTRAL = {
    "radiation_flag": 0, "delta_taper": 0.0, "hyl": 0.0, "lag_taper": 0.0, "phase_taper": 0.0,
    "shift_x": 0.0, "shift_y": 0.0, "shift_s": 0.0, "rot_x_rad": 0.0, "rot_y_rad": 0.0,
    "rot_s_rad": 0.0, "rot_s_rad_no_frame": 0.0, "rot_shift_anchor": 0.0, "resc_fac": 1.0,
}
# derived fields that are recomputed, not read
_DERIVED = {"inv_factorial_order", "h", "k0_from_h", "_isthick", "prototype", "x_normal",
            "y_normal", "svg", "name_associated_aperture", "r21", "r43", "extra"}

_MAGNET_KEYS = ("knl", "ksl", "order", "knl_rel", "ksl_rel", "model", "integrator",
                "num_multipole_kicks")
_EDGE_KEYS = ("edge_entry_active", "edge_exit_active", "edge_entry_model", "edge_exit_model",
              "edge_entry_angle", "edge_exit_angle", "edge_entry_angle_fdown",
              "edge_exit_angle_fdown", "edge_entry_fint", "edge_exit_fint", "edge_entry_hgap",
              "edge_exit_hgap")

_ACCEPT = {
    "Marker": (),
    "Drift": ("length", "model"),
    "Multipole": ("length", "hxl", "isthick", "main_order", "main_is_skew", "shift_x", "shift_y",
                  "rot_s_rad", "rot_s_rad_no_frame") + _MAGNET_KEYS,
    "Bend": ("length", "angle", "k0", "k1", "k2") + _MAGNET_KEYS + _EDGE_KEYS,
    "Quadrupole": ("length", "k1", "k1s", "main_is_skew", "edge_entry_active",
                   "edge_exit_active") + _MAGNET_KEYS,
    "Sextupole": ("length", "k2", "k2s", "main_is_skew", "edge_entry_active",
                  "edge_exit_active") + _MAGNET_KEYS,
    "Octupole": ("length", "k3", "k3s", "main_is_skew", "edge_entry_active",
                 "edge_exit_active") + _MAGNET_KEYS,
    "Cavity": ("voltage", "frequency", "lag", "phase", "harmonic", "length", "absolute_time",
               "num_kicks", "model", "integrator"),
    "LimitEllipse": ("a_squ", "b_squ", "a_b_squ", "a", "b", "shift_x", "shift_y", "rot_s_rad",
                     "rot_s_rad_no_frame"),
    "LimitRect": ("min_x", "max_x", "min_y", "max_y", "shift_x", "shift_y", "rot_s_rad",
                     "rot_s_rad_no_frame"),
    "LimitRectEllipse": ("max_x", "max_y", "a_squ", "b_squ", "a_b_squ", "a", "b", "shift_x",
                         "shift_y", "rot_s_rad", "rot_s_rad_no_frame"),
    "LimitPolygon": ("x_vertices", "y_vertices", "shift_x", "shift_y", "rot_s_rad",
                     "rot_s_rad_no_frame"),
    "DipoleEdge": ("k", "e1", "e1_fd", "hgap", "fint", "model", "side", "shift_x", "shift_y",
                   "rot_s_rad", "rot_s_rad_no_frame"),
}


def _is_neutral(v, neutral):
    if isinstance(v, (list, tuple, np.ndarray)):
        return all(float(x) == 0.0 for x in np.ravel(v))
    return v is None or float(v) == float(neutral)


def element_from_dict(dct, name="?"):
    """An element of this package from an xtrack element dict."""
    d = dict(dct)
    cname = d.pop("__class__")
    if cname in el._SLICE_CLASSES:
        raise ValueError("slices are built by Line.from_dict (they need their parent)")
    if cname not in _ACCEPT:
        raise ValueError(f"element {name!r}: class {cname} is outside the push's element set")
    kw = {}
    for k, v in d.items():
        if k in _DERIVED:
            continue
        if k in _NEUTRAL and k not in _ACCEPT[cname]:
            if not _is_neutral(v, _NEUTRAL[k]):
                raise ValueError(f"element {name!r} ({cname}): field {k}={v!r} is not supported "
                                 f"(only {_NEUTRAL[k]!r})")
            continue
        if k not in _ACCEPT[cname]:
            raise ValueError(f"element {name!r} ({cname}): unknown field {k!r}")
        kw[k] = v
    if cname == "Bend":
        # bend.py backward compatibility (_common.py:728-741): h -> angle
        if "angle" not in kw and "h" in d:
            kw["angle"] = float(d["h"]) * float(kw.get("length", 0.0))
        if d.get("k0_from_h"):
            kw["k0"] = "from_h"
    if cname == "DipoleEdge" and "k" not in kw and "h" in d:
        # dipole_edge.py backward compatibility: h -> k
        kw["k"] = d["h"]
    if cname == "Multipole" and "isthick" in kw:
        kw["isthick"] = bool(kw["isthick"])
    if cname in ("LimitEllipse", "LimitRectEllipse") and ("a" in kw or "b" in kw) and \
            "a_squ" in kw:
        kw.pop("a", None)
        kw.pop("b", None)
    klass = getattr(el, cname)
    return klass(**kw)


_TRANSFORM_KEYS = ("shift_x", "shift_y", "rot_s_rad", "rot_s_rad_no_frame")


def element_to_dict(e):
    """xtrack-format dict of an element of this package."""
    cname = type(e).__name__
    if isinstance(e, el._Slice):
        return {"__class__": cname, "weight": e.weight, "parent_name": e.parent_name}
    out = {"__class__": cname}
    if isinstance(e, el.Marker):
        return out
    if isinstance(e, el.Drift):
        out.update(length=e.length, model=e._model)
        return out
    if isinstance(e, el.Cavity):
        out.update(voltage=e.voltage, frequency=e.frequency, lag=e.lag, phase=e.phase,
                   harmonic=e.harmonic, length=e.length, absolute_time=e.absolute_time,
                   num_kicks=e.num_kicks, model=e._model, integrator=e._integrator)
        return out
    if isinstance(e, (el.LimitEllipse, el.LimitRect, el.LimitPolygon, el.LimitRectEllipse)):
        if isinstance(e, el.LimitRectEllipse):
            out.update(max_x=e.max_x, max_y=e.max_y, a_squ=e.a_squ, b_squ=e.b_squ,
                       a_b_squ=e.a_b_squ)
        elif isinstance(e, el.LimitEllipse):
            out.update(a_squ=e.a_squ, b_squ=e.b_squ, a_b_squ=e.a_b_squ)
        elif isinstance(e, el.LimitRect):
            out.update(min_x=e.min_x, max_x=e.max_x, min_y=e.min_y, max_y=e.max_y)
        else:
            out.update(x_vertices=e.x_vertices.tolist(), y_vertices=e.y_vertices.tolist())
        for f in ("shift_x", "shift_y", "rot_s_rad", "rot_s_rad_no_frame"):
            if getattr(e, f) != 0.0:
                out[f] = getattr(e, f)
        return out
    if isinstance(e, el.DipoleEdge):
        # dipole_edge.py to_dict: nonzero scalars, model and side when not default
        for f in ("k", "e1", "e1_fd", "hgap", "fint"):
            v = getattr(e, f)
            if not np.isclose(v, 0, atol=1e-16):
                out[f] = v
        if e._model != 0:
            out["model"] = e.model
        if e._side != 0:
            out["side"] = e.side
        out.update({f: getattr(e, f) for f in _TRANSFORM_KEYS if getattr(e, f) != 0.0})
        return out
    # magnets
    out.update(knl=e.knl.tolist(), ksl=e.ksl.tolist(), order=e.order,
               knl_rel=e.knl_rel.tolist(), ksl_rel=e.ksl_rel.tolist(), model=e._model,
               integrator=e._integrator, num_multipole_kicks=e.num_multipole_kicks)
    if isinstance(e, el.Multipole):
        out.update(length=e.length, hxl=e.hxl, isthick=int(e.isthick),
                   main_order=e.main_order, main_is_skew=int(e.main_is_skew))
        out.update({f: getattr(e, f) for f in _TRANSFORM_KEYS if getattr(e, f) != 0.0})
    elif isinstance(e, el.Bend):
        out.update(length=e.length, angle=e.angle, k1=e.k1, k2=e.k2)
        if e.k0 != "from_h":
            out["k0"] = e.k0
        else:
            out["k0_from_h"] = 1
        for k in _EDGE_KEYS:
            v = getattr(e, "_" + k) if k in ("edge_entry_model", "edge_exit_model") else \
                getattr(e, k)
            out[k] = v
    else:
        n, s = e._main
        out.update(length=e.length, main_is_skew=int(e.main_is_skew),
                   edge_entry_active=e.edge_entry_active, edge_exit_active=e.edge_exit_active)
        out[n] = getattr(e, n)
        out[s] = getattr(e, s)
    return out


def line_from_dict(dct):
    """A Line from an xtrack line dict ({'elements': {name: dict}, 'element_names': [...]}).
    Only the elements the sequence uses, and the parents of its slices, are
    built: a dict written by an environment also holds prototypes that no
    line references."""
    from .line import Line
    all_elements = dct["elements"]
    used = set(dct["element_names"])
    missing = used - set(all_elements)
    if missing:
        raise ValueError(f"element_names refer to unknown elements {sorted(missing)[:5]}")
    for n in list(used):
        d = all_elements[n]
        if d["__class__"] in el._SLICE_CLASSES:
            pname = d.get("parent_name", d.get("_parent_name"))
            if pname in all_elements:
                used.add(pname)
    elements = {}
    slices = {}
    for n, d in all_elements.items():
        if n not in used:
            continue
        if d["__class__"] in el._SLICE_CLASSES:
            slices[n] = d
        else:
            elements[n] = element_from_dict(d, n)
    for n, d in slices.items():
        pname = d.get("parent_name", d.get("_parent_name"))
        if pname not in elements:
            raise ValueError(f"slice {n!r}: parent {pname!r} not in the line's elements")
        unknown = set(d) - {"__class__", "weight", "parent_name", "_parent_name"}
        for k in unknown:
            if k in _NEUTRAL and _is_neutral(d[k], _NEUTRAL[k]):
                continue
            if k in _DERIVED:
                continue
            raise ValueError(f"slice {n!r}: unknown field {k!r}")
        klass = el._SLICE_CLASSES[d["__class__"]]
        elements[n] = klass(elements[pname], weight=float(d.get("weight", 1.0)),
                            parent_name=pname)
    line = Line(elements=elements, element_names=list(dct["element_names"]))
    line._extra_config.update(dct.get("extra_config", {}))
    cfg = dct.get("config", {})
    for k, v in cfg.items():
        try:
            setattr(line.config, k, v)
        except Exception:
            raise ValueError(f"line config {k!r} is not supported") from None
    return line


def line_to_dict(line):
    out = {"elements": {}, "element_names": list(line.element_names)}
    for n in line.element_names:
        if n not in out["elements"]:
            out["elements"][n] = element_to_dict(line.element_dict[n])
    # parents of slices that are not themselves in the sequence
    for n in line.element_names:
        e = line.element_dict[n]
        if isinstance(e, el._Slice) and e.parent_name not in out["elements"]:
            out["elements"][e.parent_name] = element_to_dict(e._parent)
    out["config"] = dict(line.config._v)
    out["extra_config"] = dict(line._extra_config)
    return out


def _json_default(o):
    if isinstance(o, np.ndarray):
        return o.tolist()
    if isinstance(o, (np.integer,)):
        return int(o)
    if isinstance(o, (np.floating,)):
        return float(o)
    raise TypeError(f"not serialisable: {type(o)}")


def save_json(line, path, particle=None):
    dct = line_to_dict(line)
    if particle is not None:
        dct = {"line": dct, "particle": particle.to_dict()}
    with open(path, "w") as f:
        json.dump(dct, f, default=_json_default)


def load(path, device=None):
    """xtrack/load.py:49 for JSON files: returns the Line (a file with
    ``line`` and ``particle`` entries gives the Line, with the particle
    set as ``line.particle_ref``)."""
    with open(path) as f:
        dct = json.load(f)
    if "line" in dct:
        line = line_from_dict(dct["line"])
        if "particle" in dct:
            from .particles import Particles
            line.particle_ref = particles_from_dict(dct["particle"], device=device or "cpu")
        return line
    return line_from_dict(dct)


def particles_from_dict(d, device=None):
    """Particles from an xtrack particles dict (reference ``to_dict``
    keys; the random-generator seeds and unused fields are ignored)."""
    from .particles import Particles
    kw = {}
    for k in ("q0", "mass0", "p0c", "x", "px", "y", "py", "zeta", "delta", "s", "chi",
              "charge_ratio", "weight", "particle_id", "at_element", "at_turn", "state",
              "parent_particle_id"):
        if k in d:
            kw[k] = d[k]
    if "p0c" not in kw:
        for k in ("gamma0", "beta0"):
            if k in d:
                kw[k] = d[k]
                break
    if "delta" not in kw and "ptau" in d:
        kw["ptau"] = d["ptau"]
    return Particles(device=device, **kw)
