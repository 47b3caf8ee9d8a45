"""Slicing of thick elements (xtrack/slicing.py).

``Uniform`` and ``Teapot`` weight schemes (slicing.py:81-114), ``Strategy``
matching (slicing.py:160-212, the last matching strategy wins, drifts are
only sliced when explicitly selected) and the slice sequence of
``Slicer._make_slices`` (slicing.py:342-473): entry map, alternating drift /
thin slices (thin mode) or thick slices (thick mode), exit map, wrapped in
``<name>_entry`` / ``<name>_exit`` markers (slicing.py:286-295).
"""
import re
from itertools import zip_longest

from . import elements as el


class ElementSlicingScheme:
    def __init__(self, slicing_order, mode="thin"):
        if mode not in ("thin", "thick"):
            raise ValueError(f"Unknown slicing mode: {mode}")
        self.mode = mode
        if mode == "thick":
            slicing_order -= 1
        self.slicing_order = slicing_order

    def iter_weights(self, element_length=None):
        for drift_weight, elem_weight in zip_longest(self.drift_weights(element_length),
                                                     self.element_weights(element_length),
                                                     fillvalue=None):
            yield drift_weight, True
            if elem_weight is None:
                break
            if self.mode == "thin":
                yield elem_weight, False

    def __repr__(self):
        return f"{type(self).__name__}({self.slicing_order})"


class Uniform(ElementSlicingScheme):
    def element_weights(self, element_length=None):
        if self.slicing_order == 0 and self.mode == "thick":
            return [1.0]
        return [1.0 / self.slicing_order] * self.slicing_order

    def drift_weights(self, element_length=None):
        if self.slicing_order == 0:
            return [1.0]
        slices = self.slicing_order + 1
        return [1.0 / slices] * slices


class Teapot(ElementSlicingScheme):
    def element_weights(self, element_length=None):
        if self.slicing_order == 0 and self.mode == "thick":
            return [1.0]
        return [1.0 / self.slicing_order] * self.slicing_order

    def drift_weights(self, element_length=None):
        if self.slicing_order == 0:
            return [1.0]
        if self.slicing_order == 1:
            return [0.5, 0.5]
        edge_weight = 1.0 / (2 * (1 + self.slicing_order))
        middle_weight = self.slicing_order / (self.slicing_order ** 2 - 1)
        return [edge_weight, *([middle_weight] * (self.slicing_order - 1)), edge_weight]


class Strategy:
    def __init__(self, slicing, name=None, element_type=None, exact=False):
        if name is None and element_type is None:
            exact = True
        self.regex = not exact
        if name is not None and isinstance(name, str) and self.regex:
            self.match_name = re.compile(name)
        else:
            self.match_name = name
        self.element_type = element_type
        self.slicing = slicing

    def _match_on_name(self, name):
        if self.regex:
            return self.match_name.match(name)
        return self.match_name == name

    def match_element(self, name, element):
        if isinstance(element, el.Drift):
            matched = False
            if self.match_name and not self.element_type:
                matched = bool(self._match_on_name(name))
            elif self.element_type and not self.match_name:
                matched = isinstance(element, self.element_type)
            elif self.match_name and self.element_type:
                matched = bool(self._match_on_name(name)) and isinstance(element, self.element_type)
        else:
            matched = True
            if self.match_name:
                matched = matched and bool(self._match_on_name(name))
            if self.element_type:
                matched = matched and isinstance(element, self.element_type)
        return matched


def _is_thick(element):
    return bool(element.isthick)


def slice_line(line, slicing_strategies, _edge_markers=True):
    """Slices ``line`` in place; returns {name: [slice names]}."""
    strategies = [Strategy(None, element_type=el.Drift)] + list(slicing_strategies)
    new_names = []
    slices = {}
    for name in list(line.element_names):
        element = line.element_dict[name]
        subsequence = [name]
        length = getattr(element, "length", None)
        if _is_thick(element) and not (length is not None and length == 0):
            chosen = None
            found = False
            for st in reversed(strategies):
                if st.match_element(name, element):
                    chosen = st.slicing
                    found = True
                    break
            if not found:
                raise ValueError(f"No slicing strategy found for the element {name}: {element}.")
            if chosen is not None:
                sub = _make_slices(line, element, chosen, name)
                if _edge_markers and not isinstance(element, el.Drift):
                    line.element_dict[f"{name}_entry"] = el.Marker()
                    line.element_dict[f"{name}_exit"] = el.Marker()
                    sub = [f"{name}_entry"] + sub + [f"{name}_exit"]
                subsequence = sub
        new_names += subsequence
        slices[name] = subsequence
    line.element_names = new_names
    return slices


def _unique(line, base):
    return base not in line.element_dict


def _make_slices(line, element, chosen, name):
    out = []
    d = line.element_dict
    entry_cls = el.slice_class(element, "ThinSlice", "Entry")
    if entry_cls is not None:
        nn = f"{name}..entry_map"
        d[nn] = entry_cls(element, parent_name=name)
        out.append(nn)
    elem_length = element.length
    if isinstance(element, el.Drift):
        # drifts are replaced by drifts of the slice lengths
        idx = 0
        for weight, is_drift in chosen.iter_weights(elem_length):
            if not is_drift:
                continue
            nn = f"{name}..{idx}"
            idx += 1
            d[nn] = el.Drift(length=elem_length * weight, model=element.model)
            out.append(nn)
        return out
    drift_idx = elem_idx = 0
    if chosen.mode == "thin":
        thin_cls = el.slice_class(element, "ThinSlice")
        drift_cls = el.slice_class(element, "DriftSlice")
        for weight, is_drift in chosen.iter_weights(elem_length):
            if is_drift:
                nn = f"drift_{name}..{drift_idx}"
                drift_idx += 1
                d[nn] = drift_cls(element, weight=weight, parent_name=name)
            else:
                nn = f"{name}..{elem_idx}"
                elem_idx += 1
                d[nn] = thin_cls(element, weight=weight, parent_name=name)
            out.append(nn)
    else:
        thick_cls = el.slice_class(element, "ThickSlice")
        for weight, _ in chosen.iter_weights(elem_length):
            nn = f"{name}..{elem_idx}"
            elem_idx += 1
            d[nn] = thick_cls(element, weight=weight, parent_name=name)
            out.append(nn)
    exit_cls = el.slice_class(element, "ThinSlice", "Exit")
    if exit_cls is not None:
        nn = f"{name}..exit_map"
        d[nn] = exit_cls(element, parent_name=name)
        out.append(nn)
    return out
