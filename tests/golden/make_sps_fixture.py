"""Golden vectors on a real lattice with apertures: the thin SPS line of
the reference's test data (test_data/sps_w_spacecharge/
line_no_spacecharge_and_particle.json), loaded through
xtrack_gb300.serialization (the reference's JSON format).

Every element of the line is inside the push's element set: 8200 Drift,
DipoleEdge, Multipole, LimitRect (one of them shifted in x), LimitEllipse,
Cavity and Marker elements. Elements with transformations outside the
push (longitudinal shifts, rotations, or shifts of non-apertures) would
be dropped and listed; this line has none. The fixture stores the packed raw element records, 128 particles spread
around the file's particle wide enough that the apertures take some of
them, and their state after 20 turns of the reference-compiled code
(oracle/_ref), so state, at_turn and at_element of real aperture losses
are pinned too.

Run from the repository root, in a checkout with the reference at
/root/reference:  python tests/golden/make_sps_fixture.py
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

SRC = "/root/reference/test_data/sps_w_spacecharge/line_no_spacecharge_and_particle.json"
OUT = os.path.join(HERE, "sps", "sps_thin_128p_20t.npz")
KEEP = ("x", "px", "y", "py", "zeta", "delta", "ptau", "rpp", "rvv", "s", "state",
        "at_turn", "at_element", "particle_id")
TURNS = 20


APERTURES = ("LimitRect", "LimitEllipse", "LimitPolygon")
UNSUPPORTED = ("shift_s", "rot_x_rad", "rot_y_rad", "rot_s_rad", "rot_s_rad_no_frame")


def _unsupported(e):
    if any(e.get(k, 0) != 0 for k in UNSUPPORTED):
        return True
    shifted = e.get("shift_x", 0) != 0 or e.get("shift_y", 0) != 0
    return shifted and e["__class__"] not in APERTURES


def load_line():
    with open(SRC) as f:
        d = json.load(f)
    ln = d["line"]
    els = ln["elements"]
    dropped = [n for n in ln["element_names"] if _unsupported(els[n])]
    names = [n for n in ln["element_names"] if n not in dropped]
    sub = {"elements": {n: els[n] for n in set(names)}, "element_names": names}
    line = serialization.line_from_dict(sub)
    part = serialization.particles_from_dict(d["particle"], device="cpu")
    return line, part, dropped


def main():
    pyoracle.ensure_built(with_ref=True)
    if not pyoracle.ref_available():
        raise SystemExit("reference-compiled oracle not available: run `make -C oracle ref`")
    line, p0, dropped = load_line()
    recs = line._element_records()
    again = serialization.line_from_dict(serialization.line_to_dict(line))._element_records()
    assert np.ascontiguousarray(again).tobytes() == np.ascontiguousarray(recs).tobytes()
    rng = np.random.default_rng(15)
    n = 128
    kw = {}
    for k, s in (("x", 6e-3), ("px", 1.5e-4), ("y", 5e-3), ("py", 1.5e-4), ("zeta", 0.05),
                 ("delta", 5e-4)):
        kw[k] = float(getattr(p0, k)[0]) + rng.normal(0.0, s, n)
    p = xt.Particles(device="cpu", p0c=float(p0.p0c[0]), mass0=float(p0.mass0),
                     q0=float(p0.q0), **kw)
    arrs = pyoracle.host_arrays(p.to_numpy())
    out = {k: v.copy() for k, v in arrs.items()}
    L = line.get_length()
    pyoracle.track(recs, out, line_length=L, num_turns=TURNS, which="ref")
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    payload = {"records": recs}
    for k in pyoracle.DOUBLE_FIELDS + pyoracle.INT_FIELDS:
        payload["in_" + k] = arrs[k]
    for k in KEEP:
        payload["out_" + k] = out[k]
    meta = dict(num_turns=TURNS, line_length=L, n_elements=len(recs), q0=float(p0.q0),
                mass0=float(p0.mass0),
                source="test_data/sps_w_spacecharge/line_no_spacecharge_and_particle.json",
                dropped=dropped)
    payload["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(OUT, **payload)
    lost = out["state"] <= 0
    print(OUT, len(recs), "elements,", int((~lost).sum()), "alive of", n,
          "; lost at turns", sorted(set(out["at_turn"][lost].tolist())))


if __name__ == "__main__":
    main()
