"""Generates the golden vectors of tests/golden/*.npz from the reference's
own element C code (oracle/_ref, built from the reference sources by
``make -C oracle ref``).

Each fixture stores the initial particle arrays, the arrays after the
reference-compiled push, the call arguments, and a SHA-256 of the raw
element records, so the lattice is rebuilt from the committed generator
(xtrack_gb300.workloads / tests/lattice_cases.py) and checked byte for
byte instead of being stored.

Run from the repository root:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]

import numpy as np  # noqa: E402

import pyoracle  # noqa: E402
import xtrack_gb300 as xt  # noqa: E402
from xtrack_gb300 import workloads  # noqa: E402
from lattice_cases import element_zoo, sliced_line, small_beam  # noqa: E402

KEEP = ("x", "px", "y", "py", "zeta", "delta", "ptau", "rpp", "rvv", "s", "state",
        "at_turn", "at_element", "particle_id", "ax", "ay")


def cases():
    """name -> (line factory, beam kwargs, track kwargs)."""
    return {
        "toy_ring_64p_10t": (workloads.toy_ring, small_beam(64, p0c=450e9, seed=31),
                             dict(num_turns=10)),
        "toy_ring_losses_64p_30t": (workloads.toy_ring, small_beam(64, p0c=450e9, seed=32, scale=12.0),
                                    dict(num_turns=30)),
        "thick_ring_16p_1t": (workloads.thick_ring, small_beam(16, seed=33), dict(num_turns=1)),
        "zoo_32p_1t": (element_zoo, small_beam(32, seed=34, scale=0.3), dict(num_turns=1)),
        "zoo_backtrack_32p_1t": (element_zoo, small_beam(32, seed=35, scale=0.3),
                                 dict(num_turns=1, track_flags=1)),
        "zoo_exact_drifts_32p_1t": (element_zoo, small_beam(32, seed=36, scale=0.3),
                                    dict(num_turns=1, use_exact_drifts=True)),
        "thin_sliced_32p_3t": (lambda: sliced_line(True), small_beam(32, seed=37), dict(num_turns=3)),
        "thick_sliced_32p_3t": (lambda: sliced_line(False), small_beam(32, seed=38), dict(num_turns=3)),
    }


def records_hash(recs):
    return hashlib.sha256(np.ascontiguousarray(recs).tobytes()).hexdigest()


def main():
    pyoracle.ensure_built(with_ref=True)
    if not pyoracle.ref_available():
        raise SystemExit("reference-compiled oracle not available: run `make -C oracle ref`")
    for name, (factory, beam_kw, kw) in cases().items():
        line = factory()
        recs = line._element_records()
        p = xt.Particles(device="cpu", **beam_kw)
        arrs = pyoracle.host_arrays(p.to_numpy())
        out = {k: v.copy() for k, v in arrs.items()}
        L = line.get_length()
        pyoracle.track(recs, out, line_length=L, which="ref", **kw)
        payload = {}
        for k in KEEP:
            payload["in_" + k] = arrs[k]
            payload["out_" + k] = out[k]
        for k in pyoracle.DOUBLE_FIELDS + pyoracle.INT_FIELDS:
            if k not in KEEP:
                payload["in_" + k] = arrs[k]
        meta = dict(kw, line_length=L, records_sha256=records_hash(recs), n_elements=len(recs))
        payload["meta"] = np.array(json.dumps(meta))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **payload)
        print(name, len(recs), "elements,", int((out["state"] > 0).sum()), "alive")


if __name__ == "__main__":
    main()
