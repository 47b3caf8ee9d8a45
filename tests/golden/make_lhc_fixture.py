"""Golden vectors on a real lattice: the thin HL-LHC v1.4 line of the
reference's test data (test_data/hllhc_14/line_and_particle.json), loaded
through xtrack_gb300.serialization (the reference's JSON format).

The beam-beam elements (BeamBeamBiGaussian2D/3D) and RF multipoles are
outside the push's element set and are dropped; what remains is 11603
Drift / Multipole / Cavity elements. The fixture stores the packed raw
element records (the lattice cannot be rebuilt from a generator without
the reference's data file), 64 particles around the file's particle, and
their state after 10 turns of the reference-compiled code (oracle/_ref).

Run from the repository root with the xtrack source tree named by
XTG_REFERENCE_SRC (default: a directory "reference" beside the
repository):  python tests/golden/make_lhc_fixture.py
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
SRC = os.path.join(REF, "test_data", "hllhc_14", "line_and_particle.json")
OUT = os.path.join(HERE, "lhc", "hllhc14_thin_64p_10t.npz")
KEEP_CLASSES = {"Drift", "Multipole", "Cavity"}
KEEP = ("x", "px", "y", "py", "zeta", "delta", "ptau", "rpp", "rvv", "s", "state",
        "at_turn", "at_element", "particle_id")
TURNS = 10


def load_line():
    with open(SRC) as f:
        d = json.load(f)
    ln = d["line"]
    names = [n for n in ln["element_names"] if ln["elements"][n]["__class__"] in KEEP_CLASSES]
    sub = {"elements": {n: ln["elements"][n] for n in set(names)}, "element_names": names}
    line = serialization.line_from_dict(sub)
    part = serialization.particles_from_dict(d["particle"], device="cpu")
    return line, part


def main():
    pyoracle.ensure_built(with_ref=True)
    if not pyoracle.ref_available():
        raise SystemExit("reference-compiled oracle not available: run `make -C oracle ref`")
    line, p0 = load_line()
    recs = line._element_records()
    # the lattice written back to a dict and read again gives the same records
    again = serialization.line_from_dict(serialization.line_to_dict(line))._element_records()
    assert np.ascontiguousarray(again).tobytes() == np.ascontiguousarray(recs).tobytes()
    rng = np.random.default_rng(14)
    n = 64
    kw = {}
    for k, s in (("x", 2e-4), ("px", 5e-6), ("y", 2e-4), ("py", 5e-6), ("zeta", 5e-3),
                 ("delta", 1e-4)):
        kw[k] = float(getattr(p0, k)[0]) + rng.normal(0.0, s, n)
    p = xt.Particles(device="cpu", p0c=float(p0.p0c[0]), mass0=float(p0.mass0),
                     q0=float(p0.q0), **kw)
    arrs = pyoracle.host_arrays(p.to_numpy())
    out = {k: v.copy() for k, v in arrs.items()}
    L = line.get_length()
    pyoracle.track(recs, out, line_length=L, num_turns=TURNS, which="ref")
    payload = {"records": recs}
    for k in pyoracle.DOUBLE_FIELDS + pyoracle.INT_FIELDS:
        payload["in_" + k] = arrs[k]
    for k in KEEP:
        payload["out_" + k] = out[k]
    meta = dict(num_turns=TURNS, line_length=L, n_elements=len(recs), q0=float(p0.q0),
                mass0=float(p0.mass0), source="test_data/hllhc_14/line_and_particle.json",
                dropped=["BeamBeamBiGaussian2D", "BeamBeamBiGaussian3D", "RFMultipole"])
    payload["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(OUT, **payload)
    print(OUT, len(recs), "elements,", int((out["state"] > 0).sum()), "alive of", n)


if __name__ == "__main__":
    main()
