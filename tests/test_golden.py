"""Golden vectors produced by the reference's own element C code
(tests/golden/make_golden.py, oracle/_ref). The CPU oracle must reproduce
them bit for bit; the GPU exact path within the tolerances of
test_gpu_parity.py. The lattices are rebuilt from the committed generators
and checked against the stored SHA-256 of their raw records."""
import glob
import hashlib
import json
import os

import numpy as np
import pytest

import pyoracle
from golden.make_golden import KEEP, cases

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
NAMES = [os.path.basename(f)[:-4] for f in FILES]


def _load(name):
    d = np.load(os.path.join(HERE, "golden", name + ".npz"))
    meta = json.loads(str(d["meta"]))
    factory, _, kw = cases()[name]
    line = factory()
    recs = line._element_records()
    assert hashlib.sha256(np.ascontiguousarray(recs).tobytes()).hexdigest() == meta["records_sha256"], \
        "lattice generator changed: regenerate the golden vectors"
    arrs = {k[3:]: d[k].copy() for k in d.files if k.startswith("in_")}
    arrs = pyoracle.host_arrays(arrs)
    out = {k[4:]: d[k] for k in d.files if k.startswith("out_")}
    return recs, arrs, out, meta, kw


def test_all_fixtures_present():
    assert set(NAMES) == set(cases())


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    recs, arrs, out, meta, kw = _load(name)
    pyoracle.track(recs, arrs, line_length=meta["line_length"], **kw)
    for k in KEEP:
        assert np.array_equal(arrs[k], out[k], equal_nan=True), k


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_exact_matches_golden(name):
    from xtg_testutil import gpu_track, rel_err
    recs, arrs, out, meta, kw = _load(name)
    got, _ = gpu_track(recs, arrs, arith="exact", line_length=meta["line_length"], **kw)
    for k in ("state", "at_turn", "at_element", "particle_id"):
        assert np.array_equal(got[k], out[k]), k
    tol = 1e-14 if name.startswith(("toy", "thick_ring")) else 5e-14
    ok = out["state"] > 0
    for k in ("x", "px", "y", "py", "zeta", "delta", "ptau", "rpp", "rvv", "s"):
        assert rel_err(got[k][ok], out[k][ok], k) <= tol, k
