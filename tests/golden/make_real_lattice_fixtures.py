"""Golden vectors on real lattices of the reference's test data, loaded
through xtrack_gb300.serialization (the reference's JSON format):

  sps      test_data/sps_w_spacecharge/line_no_spacecharge_and_particle.json:
           the thin SPS line, 8200 Drift, DipoleEdge, Multipole, LimitRect
           (one shifted in x), LimitEllipse, Cavity and Marker elements;
           128 particles spread wide enough that the apertures take some of
           them, 20 turns;
  psb      test_data/psb_injection/line_and_particle.json: the PS Booster
           injection line, 604 elements (DipoleEdges, thin multipoles, a
           cavity), protons; 128 particles, 20 turns;
  clic_dr  test_data/clic_dr/line.json: the CLIC damping ring, 36954
           elements (8824 DipoleEdges, 8596 thin multipoles), electrons;
           64 particles, 5 turns.

Elements with transformations outside the push (longitudinal shifts,
rotations of non-apertures) would be dropped and listed in the fixture's
metadata; these lines have none. Each fixture stores the packed raw element
records, the particles and their state after the turns of the
reference-compiled code (oracle/_ref), so state, at_turn and at_element
(aperture losses) are pinned with the coordinates.

Run from the repository root with the xtrack source tree named by
XTG_REFERENCE_SRC (default: a directory "reference" beside the
repository):  python tests/golden/make_real_lattice_fixtures.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

import numpy as np  # noqa: E402

import pyoracle  # noqa: E402
import xtrack_gb300 as xt  # noqa: E402
from xtrack_gb300 import serialization  # noqa: E402

REF = os.environ.get("XTG_REFERENCE_SRC") or os.path.join(os.path.dirname(ROOT), "reference")
DATA = os.path.join(REF, "test_data")
KEEP = ("x", "px", "y", "py", "zeta", "delta", "ptau", "rpp", "rvv", "s", "state",
        "at_turn", "at_element", "particle_id")
APERTURES = ("LimitRect", "LimitEllipse", "LimitPolygon", "LimitRectEllipse")
UNSUPPORTED = ("shift_s", "rot_x_rad", "rot_y_rad")

# name: (source, output, particles, turns, seed, beam sigmas)
LATTICES = {
    "sps": ("sps_w_spacecharge/line_no_spacecharge_and_particle.json",
            os.path.join("sps", "sps_thin_128p_20t.npz"), 128, 20, 15,
            {"x": 6e-3, "px": 1.5e-4, "y": 5e-3, "py": 1.5e-4, "zeta": 0.05, "delta": 5e-4}),
    "psb": ("psb_injection/line_and_particle.json",
            os.path.join("psb", "psb_injection_128p_20t.npz"), 128, 20, 21,
            {"x": 2e-3, "px": 2e-4, "y": 2e-3, "py": 2e-4, "zeta": 1.0, "delta": 1e-3}),
    "clic_dr": ("clic_dr/line.json", os.path.join("clic_dr", "clic_dr_64p_5t.npz"), 64, 5, 22,
                {"x": 5e-5, "px": 5e-6, "y": 1e-5, "py": 1e-6, "zeta": 1e-3, "delta": 1e-3}),
}


def _unsupported(e):
    if any(e.get(k, 0) != 0 for k in UNSUPPORTED):
        return True
    moved = any(e.get(k, 0) != 0 for k in ("shift_x", "shift_y", "rot_s_rad", "rot_s_rad_no_frame"))
    return moved and e["__class__"] not in APERTURES


def load_line(src):
    with open(os.path.join(DATA, src)) as f:
        d = json.load(f)
    ln = d["line"] if "line" in d else d
    els = ln["elements"]
    dropped = [n for n in ln["element_names"] if _unsupported(els[n])]
    names = [n for n in ln["element_names"] if n not in dropped]
    sub = {"elements": {n: els[n] for n in set(names)}, "element_names": names}
    line = serialization.line_from_dict(sub)
    pdict = d["particle"] if "particle" in d else ln["particle_ref"]
    part = serialization.particles_from_dict(pdict, device="cpu")
    return line, part, dropped


def make(name):
    src, out_path, n, turns, seed, sig = LATTICES[name]
    line, p0, dropped = load_line(src)
    recs = line._element_records()
    again = serialization.line_from_dict(serialization.line_to_dict(line))._element_records()
    assert np.ascontiguousarray(again).tobytes() == np.ascontiguousarray(recs).tobytes()
    rng = np.random.default_rng(seed)
    kw = {k: float(getattr(p0, k)[0]) + rng.normal(0.0, s, n) for k, s in sig.items()}
    p = xt.Particles(device="cpu", p0c=float(p0.p0c[0]), mass0=float(p0.mass0),
                     q0=float(p0.q0), **kw)
    arrs = pyoracle.host_arrays(p.to_numpy())
    out = {k: v.copy() for k, v in arrs.items()}
    L = line.get_length()
    pyoracle.track(recs, out, line_length=L, num_turns=turns, q0=float(p0.q0),
                   mass0=float(p0.mass0), which="ref")
    path = os.path.join(HERE, out_path)
    os.makedirs(os.path.dirname(path), exist_ok=True)
    payload = {"records": recs}
    for k in pyoracle.DOUBLE_FIELDS + pyoracle.INT_FIELDS:
        payload["in_" + k] = arrs[k]
    for k in KEEP:
        payload["out_" + k] = out[k]
    meta = dict(num_turns=turns, line_length=L, n_elements=len(recs), q0=float(p0.q0),
                mass0=float(p0.mass0), source="test_data/" + src, dropped=dropped)
    payload["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(path, **payload)
    lost = out["state"] <= 0
    print(path, len(recs), "elements,", int((~lost).sum()), "alive of", n,
          "; lost at turns", sorted(set(out["at_turn"][lost].tolist())))


def main():
    pyoracle.ensure_built(with_ref=True)
    if not pyoracle.ref_available():
        raise SystemExit("reference-compiled oracle not available: run `make -C oracle ref`")
    for name in (sys.argv[1:] or LATTICES):
        make(name)


if __name__ == "__main__":
    main()
