"""Loss-location refinement (xtrack/loss_location_refinement/
loss_location_refinement.py:29-212, 305-383, 385-417, 466-571).

A particle lost at an aperture is recorded at that aperture; it actually
left the pipe somewhere between the previous aperture and this one. The
refinement backtracks the lost particles from the aperture to the first
thick element after the previous aperture (global aperture ignored), then
tracks them forward through a short line in which copies of the aperture
are inserted every ``ds`` metres (thick elements cut at those points), so
that each particle stops at the first inserted aperture it fails. The lost
particles' coordinates and ``s`` are replaced by those at that point;
``state`` and ``at_element`` keep the original aperture.

Both steps run on the GPU push: the backtracking uses the line's own
tracker with the backtracking flag, the forward pass a tracker of the
short line.

Built here: the reference's "replicate" mode, used when the two apertures
are identical (same class and parameters; misalignments are not supported
by the push at all). Consecutive apertures that differ use polygon
interpolation in the reference (LimitPolygon, outside the push's element
set): ``refine_loss_location`` raises NotImplementedError for them.
"""
import numpy as np
import torch

from . import elements as el
from .particles import Particles

# classes through which backtracking is allowed (the reference's
# has_backtrack and allow_loss_refinement attributes: drift.py,
# _common.py:562-563, quadrupole.py, sextupole.py, octupole.py,
# cavity.py:60-61, marker.py:17-18, slice_elements_thick.py:20,
# slice_elements_drift.py:21; thin multipoles only when thick with a
# length, multipole.py:118-125; thin slices not, slice_elements_thin.py:21)
_REFINABLE = (el.Marker, el.Drift, el.Bend, el.Quadrupole, el.Sextupole, el.Octupole,
              el.Cavity)


def _is_aperture(e):
    return type(e).__name__.startswith("Limit")


def _is_thick(e):
    return bool(getattr(e, "isthick", False))


def _allow_refinement(e):
    if isinstance(e, el.Multipole):
        return e.isthick and e.length != 0
    if isinstance(e, el._Slice):
        return e._kind in (el._abi.SLICE_THICK, el._abi.SLICE_DRIFT)
    return isinstance(e, _REFINABLE)


def find_apertures(line):
    idx = [i for i, n in enumerate(line.element_names) if _is_aperture(line[n])]
    return idx, [line[line.element_names[i]] for i in idx]


def find_adjacent_thick(line, i_element, direction):
    """loss_location_refinement.py:533-550."""
    inc = -1 if direction == "upstream" else 1
    ii = i_element
    while not _is_thick(line[line.element_names[ii]]):
        ii += inc
    return ii


def apertures_are_identical(a, b):
    """loss_location_refinement.py:243-292 for the aperture classes of the push."""
    if type(a) is not type(b):
        return False
    fields = {"LimitRect": ("min_x", "max_x", "min_y", "max_y"),
              "LimitEllipse": ("a_squ", "b_squ", "a_b_squ")}[type(a).__name__]
    return all(abs(getattr(a, f) - getattr(b, f)) <= 1e-15 for f in fields)


def interp_aperture_locations(s_elements, i_aper_0, i_aper_1, ds):
    """loss_location_refinement.py:466-476."""
    s0 = s_elements[i_aper_0]
    s1 = s_elements[i_aper_1]
    assert s1 >= s0
    n_segments = int(np.ceil((s1 - s0) / ds))
    if n_segments <= 1:
        s_vect = np.array([])
    else:
        s_vect = np.linspace(s0, s1, n_segments + 1)[1:-1]
    return s0, s1, s_vect


def _cut(e, pieces):
    """Pieces of thick element ``e`` with the given lengths: drifts are cut
    into drifts, magnets into an entry edge, thick slices weighted by
    length and an exit edge (the thick slicing xtrack applies when an
    element is inserted inside a thick magnet)."""
    if isinstance(e, el.Drift):
        return [el.Drift(length=l, model=e.model) for l in pieces]
    if isinstance(e, (el.Bend, el.Quadrupole, el.Sextupole, el.Octupole)):
        out = []
        entry = el.slice_class(e, "ThinSlice", "Entry")
        exit_ = el.slice_class(e, "ThinSlice", "Exit")
        thick = el.slice_class(e, "ThickSlice")
        out.append(entry(e, weight=1.0))
        for l in pieces:
            out.append(thick(e, weight=l / e.length))
        out.append(exit_(e, weight=1.0))
        return out
    if isinstance(e, el._Slice) and e._kind in (el._abi.SLICE_THICK, el._abi.SLICE_DRIFT):
        total = e._parent.length * e.weight
        return [type(e)(e._parent, weight=e.weight * l / total, parent_name=e.parent_name)
                for l in pieces]
    raise NotImplementedError(f"cannot cut {type(e).__name__} for loss refinement")


def build_interp_line(line, i_end_thin_0, i_start_thin_1, s0, s_vect, aperture):
    """The short line: an aperture copy, the elements between the thick
    neighbours of the two apertures with aperture copies at ``s_vect``
    (cutting thick elements there), and a final aperture copy
    (loss_location_refinement.py:493-530)."""
    from .line import Line, _element_length
    elems = [aperture.copy()]
    s = s0
    cuts = list(s_vect)
    ci = 0
    for n in line.element_names[i_end_thin_0 + 1:i_start_thin_1]:
        e = line[n]
        L = _element_length(e)
        if L == 0:
            while ci < len(cuts) and cuts[ci] <= s:
                elems.append(aperture.copy())
                ci += 1
            elems.append(e)
            continue
        # cut points strictly inside, or at the entrance, of this element
        inside = []
        while ci < len(cuts) and cuts[ci] < s + L:
            inside.append(cuts[ci])
            ci += 1
        if not inside:
            elems.append(e)
        else:
            bounds = [s] + inside + [s + L]
            pieces = [b - a for a, b in zip(bounds[:-1], bounds[1:])]
            if pieces[0] == 0.0:
                # a cut exactly at the entrance: aperture before the element
                pieces = pieces[1:]
                elems.append(aperture.copy())
                n_inner = len(inside) - 1
            else:
                n_inner = len(inside)
            cut = _cut(e, pieces)
            has_edges = len(cut) == len(pieces) + 2
            body = cut[1:-1] if has_edges else cut
            if has_edges:
                elems.append(cut[0])
            for k, piece in enumerate(body):
                elems.append(piece)
                if k < n_inner:
                    elems.append(aperture.copy())
            if has_edges:
                elems.append(cut[-1])
        s += L
    while ci < len(cuts):
        elems.append(aperture.copy())
        ci += 1
    elems.append(aperture.copy())
    names = [f"_interp_{k}" for k in range(len(elems))]
    out = Line(elements=elems, element_names=names)
    out.config.XTRACK_GLOBAL_XY_LIMIT = line.config.XTRACK_GLOBAL_XY_LIMIT
    out.config.XTRACK_USE_EXACT_DRIFTS = line.config.XTRACK_USE_EXACT_DRIFTS
    out.reset_s_at_end_turn = False
    return out


class LossLocationRefinement:
    """Refines the loss location of particles lost at apertures of ``line``
    (loss_location_refinement.py:29-108). ``ds``: spacing of the inserted
    apertures [m]. ``n_theta``, ``r_max`` and ``dr`` belong to the polygon
    mode, which is not built; they are accepted and ignored."""

    def __init__(self, line, backtrack_line=None, n_theta=None, r_max=None, dr=None, ds=None,
                 save_refine_lines=False, allowed_backtrack_types=()):
        if backtrack_line is not None:
            raise ValueError("Backtracking line not supported anymore!")
        if ds is None:
            raise ValueError("ds is required")
        if getattr(line, "tracker", None) is None:
            raise RuntimeError("the line needs a tracker (line.build_tracker())")
        self.line = line
        self.ds = float(ds)
        self.n_theta, self.r_max, self.dr = n_theta, r_max, dr
        self.allowed_backtrack_types = tuple(allowed_backtrack_types)
        self.i_apertures, self.apertures = find_apertures(line)
        self.save_refine_lines = save_refine_lines
        if save_refine_lines:
            self.refine_lines = {}
        self._s = np.asarray(line.get_s_elements())

    def _check_backtrack(self, i_start, i_stop):
        for n in self.line.element_names[i_start:i_stop]:
            e = self.line[n]
            if _allow_refinement(e):
                continue
            if self.allowed_backtrack_types and isinstance(e, self.allowed_backtrack_types):
                continue
            raise TypeError(f"Cannot backtrack through element {n} of type {type(e).__name__}")

    def refine_loss_location(self, particles, i_apertures=None, with_progress=False):
        """loss_location_refinement.py:110-212 (replicate mode)."""
        if i_apertures is None:
            i_apertures = self.i_apertures
        state = particles.state.cpu().numpy()
        at_el = particles.at_element.cpu().numpy()
        for i_ap in i_apertures:
            mask = (at_el == i_ap) & (state == 0)
            if not np.any(mask):
                continue
            k = self.i_apertures.index(i_ap)
            if k == 0:
                continue            # the first aperture of the line cannot be handled
            i_aper_1 = i_ap
            i_aper_0 = self.i_apertures[k - 1]
            s0, s1, s_vect = interp_aperture_locations(self._s, i_aper_0, i_aper_1, self.ds)
            if s1 - s0 <= self.ds:
                continue
            a0 = self.line[self.line.element_names[i_aper_0]]
            a1 = self.line[self.line.element_names[i_aper_1]]
            if not apertures_are_identical(a0, a1):
                raise NotImplementedError(
                    f"apertures {i_aper_0} and {i_aper_1} differ: the polygon interpolation "
                    "mode is not built")
            i_start_thin_1 = find_adjacent_thick(self.line, i_aper_1, "upstream") + 1
            i_end_thin_0 = find_adjacent_thick(self.line, i_aper_0, "downstream") - 1
            interp = build_interp_line(self.line, i_end_thin_0, i_start_thin_1, s0, s_vect, a1)
            self._refine_single(particles, mask, i_aper_1, i_end_thin_0, interp)
            if self.save_refine_lines:
                interp.i_start_thin_0 = i_end_thin_0
                interp.i_start_thin_1 = i_start_thin_1
                interp.s0 = s0
                interp.s1 = s1
                self.refine_lines[i_ap] = interp

    def _refine_single(self, particles, mask, i_aper_1, i_end_thin_0, interp):
        """loss_location_refinement.py:305-383."""
        dev = particles.device
        sel = torch.from_numpy(np.nonzero(mask)[0]).to(dev)

        def take(f):
            return getattr(particles, f).index_select(0, sel).cpu().numpy()

        part = Particles(device=dev, p0c=take("p0c"), mass0=particles.mass0, q0=particles.q0,
                         x=take("x"), px=take("px"), y=take("y"), py=take("py"),
                         zeta=take("zeta"), delta=take("delta"), s=take("s"), chi=take("chi"),
                         charge_ratio=take("charge_ratio"))
        i_start = i_end_thin_0 + 1
        i_stop = i_aper_1
        self._check_backtrack(i_start, i_stop)
        tr = self.line.tracker
        flags = tr.track_flags
        old = flags.XS_FLAG_IGNORE_GLOBAL_APERTURE
        flags.XS_FLAG_IGNORE_GLOBAL_APERTURE = True
        try:
            tr._track(part, ele_start=i_start, ele_stop=i_stop, backtrack=True,
                      _force_no_end_turn_actions=True)
        finally:
            flags.XS_FLAG_IGNORE_GLOBAL_APERTURE = old
        itr = interp.build_tracker(device=dev, arith=tr.arith)
        itr.track_flags.XS_FLAG_IGNORE_GLOBAL_APERTURE = True
        itr._track(part)
        if np.any(part.state.cpu().numpy() < 0):
            raise RuntimeError("particles lost with error codes during the refinement")
        order = torch.argsort(part.particle_id)
        for f in ("x", "px", "y", "py", "zeta", "s", "delta", "ptau", "rvv", "rpp", "p0c",
                  "gamma0", "beta0"):
            getattr(particles, f).index_copy_(0, sel, getattr(part, f).index_select(0, order))
        return part
