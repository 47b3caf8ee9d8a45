"""xtrack-format dictionaries and JSON: round trips of every element class
and of sliced lines (same raw records), rejection of out-of-scope fields,
and a real lattice: the thin HL-LHC v1.4 line of the reference's test data,
loaded through the serializer, whose golden vectors come from the
reference-compiled code (tests/golden/make_lhc_fixture.py)."""
import json
import os

import numpy as np
import pytest

import pyoracle
import xtrack_gb300 as xt
from xtrack_gb300 import serialization as ser
from xtrack_gb300 import workloads
from lattice_cases import (element_zoo, fringe_zoo, shifted_apertures, shifted_thin_elements,
                           sliced_line)

HERE = os.path.dirname(os.path.abspath(__file__))
LHC = os.path.join(HERE, "golden", "lhc", "hllhc14_thin_64p_10t.npz")
SPS = os.path.join(HERE, "golden", "sps", "sps_thin_128p_20t.npz")
PSB = os.path.join(HERE, "golden", "psb", "psb_injection_128p_20t.npz")
CLIC_DR = os.path.join(HERE, "golden", "clic_dr", "clic_dr_64p_5t.npz")


def _same_records(a, b):
    """Raw records equal, except `aux` (the address of a descriptor built
    per call)."""
    a = np.array(a, copy=True)
    b = np.array(b, copy=True)
    a["aux"] = 0
    b["aux"] = 0
    return np.ascontiguousarray(a).tobytes() == np.ascontiguousarray(b).tobytes()


def _with_polygon():
    th = np.linspace(0, 2 * np.pi, 7)[:-1]
    return xt.Line(elements=[xt.Drift(length=1.0),
                             xt.LimitPolygon(x_vertices=0.01 * np.cos(th),
                                             y_vertices=0.008 * np.sin(th))],
                   element_names=["d", "poly"])


@pytest.mark.parametrize("factory", [workloads.toy_ring, element_zoo, lambda: sliced_line(True),
                                     _with_polygon, fringe_zoo, shifted_apertures,
                                     shifted_thin_elements, lambda: sliced_line(False),
                                     lambda: workloads.thick_ring(n_arcs=1, n_cells=2)])
def test_dict_and_json_round_trip(factory, tmp_path):
    line = factory()
    d = line.to_dict()
    json.dumps(d)                                   # plain JSON types only
    back = xt.Line.from_dict(d)
    assert back.element_names == line.element_names
    assert _same_records(back._element_records(), line._element_records())
    path = str(tmp_path / "line.json")
    line.to_json(path)
    again = xt.load(path)
    assert _same_records(again._element_records(), line._element_records())
    for n in line.element_names:
        if isinstance(line[n], xt.LimitPolygon):
            assert np.array_equal(again[n].x_vertices, line[n].x_vertices)
            assert np.array_equal(back[n].y_vertices, line[n].y_vertices)


def test_reference_style_dicts():
    # as xtrack writes them: ints for models, 'h' instead of 'angle', k0_from_h
    d = {"elements": {
        "d": {"__class__": "Drift", "length": 1.5},
        "m": {"__class__": "Multipole", "order": 1, "inv_factorial_order": 1.0, "length": 0.0,
              "hxl": 0.0, "hyl": 0.0, "radiation_flag": 0, "knl": [0.0, 1e-3], "ksl": [0.0, 0.0]},
        "b": {"__class__": "Bend", "length": 2.0, "h": 0.01, "k0_from_h": 1, "k1": 0.0,
              "model": 6, "integrator": 3, "num_multipole_kicks": 4, "edge_entry_model": 0,
              "shift_x": 0.0, "rot_s_rad": 0.0},
        "c": {"__class__": "Cavity", "voltage": 2e6, "frequency": 400e6, "phase": 3.14},
        "a": {"__class__": "LimitEllipse", "a_squ": 4e-4, "b_squ": 4e-4, "a_b_squ": 1.6e-7}},
        "element_names": ["d", "m", "b", "c", "a"]}
    line = xt.Line.from_dict(d)
    b = line["b"]
    assert b.k0 == "from_h" and abs(b.angle - 0.02) < 1e-15
    assert b.model == "drift-kick-drift-expanded" and b.integrator == "uniform"
    assert line["m"].knl.tolist() == [0.0, 1e-3]
    assert line["c"].phase == 3.14


@pytest.mark.parametrize("bad", [
    {"__class__": "Drift", "length": 1.0, "shift_x": 1e-3},
    {"__class__": "Multipole", "knl": [0.0], "radiation_flag": 1},
    {"__class__": "Multipole", "knl": [0.0], "hyl": 1e-3},
    {"__class__": "Cavity", "voltage": 1.0, "lag_taper": 5.0},
    {"__class__": "Drift", "length": 1.0, "mystery": 2},
    {"__class__": "BeamBeamBiGaussian2D"},
])
def test_out_of_scope_fields_are_rejected(bad):
    with pytest.raises(ValueError):
        ser.element_from_dict(bad, "e")


def test_dipole_edge_dicts():
    """DipoleEdge as the reference writes it (nonzero scalars, model and
    side by name) and in its older form (h for k, stored r21/r43, which are
    recomputed): the same element and record."""
    new = ser.element_from_dict({"__class__": "DipoleEdge", "k": 0.0013490601351007177,
                                 "e1": 0.004222570771, "hgap": 0.02, "fint": 0.5,
                                 "model": "full", "side": "exit"})
    old = ser.element_from_dict({"__class__": "DipoleEdge", "h": 0.0013490601351007177,
                                 "e1": 0.004222570771, "hgap": 0.02, "fint": 0.5,
                                 "r21": 1.0, "r43": 2.0, "model": "full", "side": "exit"})
    assert new.model == old.model == "full" and new.side == old.side == "exit"
    assert new.r21 == old.r21 and new.r43 == old.r43 and new.r21 != 1.0
    rec = new.to_record()
    assert rec["model"] == 1 and rec["side"] == 1 and rec["r21"] == new.r21
    assert ser.element_to_dict(new) == {"__class__": "DipoleEdge", "k": new.k, "e1": new.e1,
                                        "hgap": 0.02, "fint": 0.5, "model": "full",
                                        "side": "exit"}
    # changing a parameter recomputes the linear coefficients
    r43 = new.r43
    new.fint = 0.7
    assert new.r43 != r43


def _fixture(path):
    d = np.load(path)
    meta = json.loads(str(d["meta"]))
    recs = d["records"]
    arrs = pyoracle.host_arrays({k[3:]: d[k].copy() for k in d.files if k.startswith("in_")})
    out = {k[4:]: d[k] for k in d.files if k.startswith("out_")}
    return recs, arrs, out, meta


def test_lhc_fixture_oracle_reproduces_reference():
    recs, arrs, out, meta = _fixture(LHC)
    assert meta["n_elements"] == len(recs) == 11603
    pyoracle.track(recs, arrs, line_length=meta["line_length"], num_turns=meta["num_turns"],
                   q0=meta["q0"], mass0=meta["mass0"])
    for k, v in out.items():
        assert np.array_equal(arrs[k], v), k


@pytest.mark.gpu
@pytest.mark.parametrize("arith", ["exact", "fast"])
def test_lhc_fixture_gpu(arith):
    """The real 11603-element thin LHC line on the GPU against the
    reference-compiled result after 10 turns: exact within 1e-14, fast
    within 3x the reference's own FMA spread."""
    from xtg_testutil import compare, compare_within_spread, fma_spread, gpu_track
    recs, arrs, out, meta = _fixture(LHC)
    kw = dict(line_length=meta["line_length"], num_turns=meta["num_turns"], q0=meta["q0"],
              mass0=meta["mass0"])
    got, _ = gpu_track(recs, {k: v.copy() for k, v in arrs.items()}, arith=arith, **kw)
    if arith == "exact":
        compare(got, out, 1e-14)
    else:
        for f in ("state", "at_turn", "at_element"):
            assert np.array_equal(got[f], out[f]), f
        spread, ok = fma_spread(recs, arrs, **kw)
        compare_within_spread(got, out, spread, ok)


REAL = {"sps": (SPS, 8200), "psb": (PSB, 604), "clic_dr": (CLIC_DR, 36954)}


@pytest.mark.parametrize("name", list(REAL))
def test_real_lattice_fixture_oracle_reproduces_reference(name):
    """Real lattices of the reference's test data after their turns of the
    reference-compiled code: the thin SPS line (8200 elements, 1698
    apertures, real losses), the PS Booster injection line (604 elements)
    and the CLIC damping ring (36954 elements, electrons)."""
    path, n_el = REAL[name]
    recs, arrs, out, meta = _fixture(path)
    assert meta["n_elements"] == len(recs) == n_el and not meta["dropped"]
    if name == "sps":
        assert np.sum(out["state"] <= 0) > 5
    pyoracle.track(recs, arrs, line_length=meta["line_length"], num_turns=meta["num_turns"],
                   q0=meta["q0"], mass0=meta["mass0"])
    for k, v in out.items():
        assert np.array_equal(arrs[k], v), k


@pytest.mark.gpu
@pytest.mark.parametrize("arith", ["exact", "fast"])
@pytest.mark.parametrize("name", list(REAL))
def test_real_lattice_fixture_gpu(name, arith):
    """The real lattices on the GPU against the reference-compiled result:
    state, at_turn and at_element bit-exact. Exact mode: one turn within
    1e-14; all turns within 1e-10. The cavities' sin comes from CUDA's libm:
    on the SPS beam all 128 particles stay bit-identical for 16 turns, then
    one cavity pass of one particle gets a sin one ulp away from glibc's,
    rvv moves by an ulp, and the drifts of the following turns carry that
    to ~8e-12 relative in zeta. Fast mode: within 3x the reference's FMA
    spread."""
    from xtg_testutil import (compare, compare_within_spread, fma_spread, gpu_track,
                              near_edge_mask)
    recs, arrs, out, meta = _fixture(REAL[name][0])
    kw = dict(line_length=meta["line_length"], num_turns=meta["num_turns"], q0=meta["q0"],
              mass0=meta["mass0"])
    got, _ = gpu_track(recs, {k: v.copy() for k, v in arrs.items()}, arith=arith, **kw)
    near = near_edge_mask(recs, arrs, **kw)
    if arith == "exact":
        compare(got, out, 1e-10, near_edge=near, label=f"{name}, exact, {meta['num_turns']} turns:")
        kw1 = dict(kw, num_turns=1)
        one = {k: v.copy() for k, v in arrs.items()}
        pyoracle.track(recs, one, **kw1)
        g1, _ = gpu_track(recs, {k: v.copy() for k, v in arrs.items()}, arith=arith, **kw1)
        compare(g1, one, 1e-14)
    else:
        # integer fields against the reference, near-edge particles exempt
        # only where they differ
        compare(got, out, np.inf, near_edge=near, label=f"{name}, fast, {meta['num_turns']} turns:")
        spread, ok = fma_spread(recs, arrs, **kw)
        compare_within_spread(got, out, spread, ok)
