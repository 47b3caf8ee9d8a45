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

Both of the reference's modes are built: "replicate" when the two
apertures are identical (misalignments are not supported by the push at
all), and polygon interpolation otherwise: each aperture is characterised
as a convex polygon by tracking test particles on rays through it, and the
apertures inserted along the gap are LimitPolygons whose vertices move
linearly in s from one polygon to the other.
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
    if isinstance(a, el.LimitPolygon):
        return (len(a.x_vertices) == len(b.x_vertices)
                and np.allclose(a.x_vertices, b.x_vertices, rtol=0, atol=1e-15)
                and np.allclose(a.y_vertices, b.y_vertices, rtol=0, atol=1e-15))
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


def build_interp_line(line, i_end_thin_0, i_start_thin_1, s0, s_vect, aperture,
                      aper_0=None, aper_1=None, aper_interp=None):
    """The short line: the first aperture, the elements between the thick
    neighbours of the two apertures with an aperture at each of ``s_vect``
    (cutting thick elements there), and the last aperture
    (loss_location_refinement.py:493-530). Copies of ``aperture`` serve
    where ``aper_0`` / ``aper_1`` / ``aper_interp`` are not given."""
    from .line import Line, _element_length
    if aper_interp is None:
        aper_interp = [aperture.copy() for _ in s_vect]
    aper_iter = iter(aper_interp)

    class _Next:
        def copy(self):
            return next(aper_iter)

    first = aper_0 if aper_0 is not None else aperture.copy()
    last = aper_1 if aper_1 is not None else aperture.copy()
    aperture = _Next()
    elems = [first]
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
    elems.append(last)
    names = [f"_interp_{k}" for k in range(len(elems))]
    out = Line(elements=elems, element_names=names)
    out.config.XTRACK_GLOBAL_XY_LIMIT = line.config.XTRACK_GLOBAL_XY_LIMIT
    out.config.XTRACK_USE_EXACT_DRIFTS = line.config.XTRACK_USE_EXACT_DRIFTS
    out.reset_s_at_end_turn = False
    return out


def _convex_hull_polygon(x, y):
    """LimitPolygon through the convex hull of the points, vertices in
    their original (angle) order (loss_location_refinement.py:449-455)."""
    from scipy.spatial import ConvexHull
    hull = ConvexHull(np.array([x, y]).T)
    i_hull = np.sort(hull.vertices)
    return el.LimitPolygon(x_vertices=x[i_hull], y_vertices=y[i_hull])


def characterize_aperture(line, i_aperture, n_theta, r_max, dr, coming_from="upstream"):
    """Polygon approximating the aperture seen from its thick neighbour
    (loss_location_refinement.py:573-658): test particles on n_theta rays
    are tracked from the thick neighbour through the aperture (two passes,
    coarse then at step ``dr``); the first lost point of each ray gives a
    vertex; the convex hull of these is resampled at every ray angle.
    Returns (polygon, index of the first thin element)."""
    assert coming_from in ("upstream", "downstream")
    if coming_from == "upstream":
        i_start = find_adjacent_thick(line, i_aperture, "upstream") + 1
        i_stop = i_aperture + 1
        backtrack = False
        index_start_thin = i_start
    else:
        i_stop = find_adjacent_thick(line, i_aperture, "downstream")
        i_start = i_aperture
        backtrack = True
        index_start_thin = i_stop - 1
    theta = np.linspace(0, 2 * np.pi, n_theta + 1)[:-1]
    rmin, rmax = 0.0, r_max
    step = (rmax - rmin) / 100.
    rmin_theta = 0 * theta
    tr = line.tracker
    for iteration in range(2):
        r_vect = np.arange(rmin, rmax, step)
        RR, TT = np.meshgrid(r_vect, theta)
        RR += np.atleast_2d(rmin_theta).T
        x_test = RR.flatten() * np.cos(TT.flatten())
        y_test = RR.flatten() * np.sin(TT.flatten())
        ptest = Particles(p0c=1, x=x_test.copy(), y=y_test.copy(), device=tr.device)
        flags = tr.track_flags
        old = flags.XS_FLAG_IGNORE_GLOBAL_APERTURE
        flags.XS_FLAG_IGNORE_GLOBAL_APERTURE = True
        try:
            tr._track(ptest, ele_start=i_start, ele_stop=i_stop, backtrack=backtrack,
                      _force_no_end_turn_actions=True)
        finally:
            flags.XS_FLAG_IGNORE_GLOBAL_APERTURE = old
        pid = ptest.particle_id.cpu().numpy()
        state = ptest.state.cpu().numpy()[np.argsort(pid)]
        state_mat = state.reshape(RR.shape)
        i_r_aper = np.argmin(state_mat > 0, axis=1)
        rmin_theta = r_vect[i_r_aper - 1]
        rmin, rmax = 0.0, 2 * step
        step = dr
    x_mat = x_test.reshape(RR.shape)
    y_mat = y_test.reshape(RR.shape)
    xv = np.array([x_mat[k, i_r_aper[k]] for k in range(n_theta)])
    yv = np.array([y_mat[k, i_r_aper[k]] for k in range(n_theta)])
    temp = _convex_hull_polygon(xv, yv)
    r_out = 1.0
    res = temp.impact_point_and_normal(x_in=0 * theta, y_in=0 * theta, z_in=0 * theta,
                                       x_out=r_out * np.cos(theta), y_out=r_out * np.sin(theta),
                                       z_out=0 * theta)
    return el.LimitPolygon(x_vertices=res[0], y_vertices=res[1]), index_start_thin


def interp_aperture_using_polygons(line, i_aper_0, i_aper_1, n_theta, r_max, dr, ds, s_elements):
    """loss_location_refinement.py:419-463."""
    polygon_1, i_start_thin_1 = characterize_aperture(line, i_aper_1, n_theta, r_max, dr,
                                                      coming_from="upstream")
    polygon_0, i_end_thin_0 = characterize_aperture(line, i_aper_0, n_theta, r_max, dr,
                                                    coming_from="downstream")
    s0, s1, s_vect = interp_aperture_locations(s_elements, i_aper_0, i_aper_1, ds)
    delta_s = s1 - s0
    interp = []
    for ss in s_vect:
        xn = polygon_1.x_vertices * (ss - s0) / delta_s + polygon_0.x_vertices * (s1 - ss) / delta_s
        yn = polygon_1.y_vertices * (ss - s0) / delta_s + polygon_0.y_vertices * (s1 - ss) / delta_s
        interp.append(_convex_hull_polygon(xn, yn))
    interp_line = build_interp_line(line, i_end_thin_0, i_start_thin_1, s0, s_vect, None,
                                    aper_0=polygon_0, aper_1=polygon_1, aper_interp=interp)
    return interp_line, i_end_thin_0, i_start_thin_1, s0, s1


class LossLocationRefinement:
    """Refines the loss location of particles lost at apertures of ``line``
    (loss_location_refinement.py:29-108). ``ds``: spacing of the inserted
    apertures [m]. ``n_theta`` (rays), ``r_max`` and ``dr`` [m] set the
    characterisation of differing apertures (polygon mode)."""

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
            if apertures_are_identical(a0, a1):
                i_start_thin_1 = find_adjacent_thick(self.line, i_aper_1, "upstream") + 1
                i_end_thin_0 = find_adjacent_thick(self.line, i_aper_0, "downstream") - 1
                interp = build_interp_line(self.line, i_end_thin_0, i_start_thin_1, s0, s_vect,
                                           a1)
            else:
                if self.n_theta is None or self.r_max is None or self.dr is None:
                    raise ValueError("apertures differ: n_theta, r_max and dr are needed for "
                                     "the polygon interpolation")
                interp, i_end_thin_0, i_start_thin_1, s0, s1 = interp_aperture_using_polygons(
                    self.line, i_aper_0, i_aper_1, self.n_theta, self.r_max, self.dr, self.ds,
                    self._s)
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
