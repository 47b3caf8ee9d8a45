"""Host-side logic, checked without a GPU: the C-ABI library loads and
exports every entry point of include/xtrack_gb300.h, the ctypes mirror has
the C layout, unsupported elements are rejected before any device call,
Particles reproduces the reference's initialisation formulas, slicing
produces the reference's element sequence, the turn split follows
tracker.py:1270-1436, and the particle sharding of multi-GPU runs covers
the beam exactly once (gloo, two ranks)."""
import ctypes
import os
import re
import sys

import numpy as np
import pytest
import torch

import pyoracle
import xtrack_gb300 as xt
from xtrack_gb300 import _abi
from xtrack_gb300.particles import PROTON_MASS_EV

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "xtrack_gb300.h")


def _declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(xtg_\w+)\s*\(", text)))


def test_library_exports_every_declared_entry_point():
    lib = _abi.load_library()
    names = _declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), f"{n} declared in the header but not exported"
    assert lib.xtg_abi_version() == 3
    assert set(names) == set(_abi.EXPORTED_SYMBOLS)


def test_ctypes_layout_matches_c():
    pyoracle.ensure_built(with_ref=False)
    lib = pyoracle._load(pyoracle.ORACLE_LIB, "oracle")
    out = (ctypes.c_int64 * 12)()
    lib.xto_abi_sizes(out)
    assert out[0] == ctypes.sizeof(_abi.XtgElement) == _abi.ELEMENT_DTYPE.itemsize
    assert out[1] == ctypes.sizeof(_abi.XtgParticles)
    assert out[2] == ctypes.sizeof(_abi.XtgMonitor)
    assert out[3] == ctypes.sizeof(_abi.XtgConfig)
    assert out[4] == _abi.XtgElement.knl.offset
    assert out[5] == _abi.XtgElement.shift_x.offset
    assert out[6] == _abi.XtgMonitor.data.offset
    assert out[7] == ctypes.sizeof(_abi.XtgElementMonitor)
    assert out[8] == _abi.XtgElementMonitor.particles.offset
    assert out[9] == _abi.XtgElement.aux.offset
    assert out[10] == _abi.XtgElement.r21.offset
    assert out[11] == _abi.XtgElement.side.offset


@pytest.mark.parametrize("element,msg", [
    (xt.Bend(length=1.0, angle=0.01, model=42), "model"),
    (xt.Bend(length=1.0, angle=0.01, edge_entry_model=7), "edge model"),
])
def test_unsupported_elements_rejected_before_device(element, msg):
    line = xt.Line(elements=[xt.Drift(length=1.0), element])
    recs = line._element_records()
    lib = _abi.load_library()
    cfg = _abi.XtgConfig()
    cfg.has_global_xy_limit = 1
    cfg.global_xy_limit = 1.0
    h = ctypes.c_void_p()
    st = lib.xtg_lattice_create(recs.ctypes.data_as(ctypes.c_void_p), len(recs),
                                ctypes.byref(cfg), ctypes.byref(h))
    assert st == _abi.XTG_E_UNSUPPORTED
    assert msg in _abi.last_error(lib)
    assert "element 1" in _abi.last_error(lib)
    st, m = pyoracle.validate(recs)
    assert st == _abi.XTG_E_UNSUPPORTED and msg in m


def test_order_limits():
    with pytest.raises(ValueError):
        xt.Multipole(knl=[0.0] * 22).to_record()
    recs = xt.Line(elements=[xt.Multipole(knl=[1e-3])])._element_records()
    recs[0]["order"] = 25
    lib = _abi.load_library()
    cfg = _abi.XtgConfig()
    h = ctypes.c_void_p()
    st = lib.xtg_lattice_create(recs.ctypes.data_as(ctypes.c_void_p), 1, ctypes.byref(cfg),
                                ctypes.byref(h))
    assert st == _abi.XTG_E_UNSUPPORTED and "order" in _abi.last_error(lib)


def test_misaligned_record_rejected():
    recs = xt.Line(elements=[xt.Drift(length=1.0)])._element_records()
    recs[0]["shift_x"] = 1e-3
    lib = _abi.load_library()
    cfg = _abi.XtgConfig()
    h = ctypes.c_void_p()
    st = lib.xtg_lattice_create(recs.ctypes.data_as(ctypes.c_void_p), 1, ctypes.byref(cfg),
                                ctypes.byref(h))
    assert st == _abi.XTG_E_UNSUPPORTED and "misalignment" in _abi.last_error(lib)


@pytest.mark.parametrize("field,value,msg", [("model", 5, "DipoleEdge model"),
                                             ("side", 2, "DipoleEdge side")])
def test_invalid_dipole_edge_rejected(field, value, msg):
    recs = xt.Line(elements=[xt.DipoleEdge(k=1e-3, e1=0.01)])._element_records()
    recs[0][field] = value
    lib = _abi.load_library()
    h = ctypes.c_void_p()
    st = lib.xtg_lattice_create(recs.ctypes.data_as(ctypes.c_void_p), 1,
                                ctypes.byref(_abi.XtgConfig()), ctypes.byref(h))
    assert st == _abi.XTG_E_UNSUPPORTED and msg in _abi.last_error(lib)


def test_aperture_shifts_validated():
    """Transverse shifts and tilts pass for apertures; other rotations and
    longitudinal shifts do not, nor shifts or tilts of other classes."""
    line = xt.Line(elements=[xt.LimitRect(min_x=-0.01, max_x=0.01, shift_x=1e-3, rot_s_rad=0.1),
                             xt.LimitRectEllipse(max_x=0.01, max_y=0.01, a=0.02, b=0.02,
                                                 shift_y=-1e-3),
                             xt.Drift(length=1.0)])
    recs = line._element_records()
    lib = _abi.load_library()
    cfg = _abi.XtgConfig()
    assert pyoracle.validate(recs)[0] == _abi.XTG_OK
    for i, field in ((0, "rot_x_rad"), (0, "shift_s"), (2, "rot_s_rad"), (2, "shift_x")):
        bad = recs.copy()
        bad[i][field] = 1e-3
        st, msg = pyoracle.validate(bad)
        assert st == _abi.XTG_E_UNSUPPORTED and "misalignment" in msg
        h = ctypes.c_void_p()
        st = lib.xtg_lattice_create(bad.ctypes.data_as(ctypes.c_void_p), 3, ctypes.byref(cfg),
                                    ctypes.byref(h))
        assert st == _abi.XTG_E_UNSUPPORTED and "misalignment" in _abi.last_error(lib)


def test_thin_element_shifts_validated():
    """Transverse shifts and tilts pass for thin multipoles and dipole edges
    (oracle and library alike); a thick multipole or a quadrupole with one,
    or a thin multipole with a longitudinal shift, is rejected."""
    line = xt.Line(elements=[xt.Multipole(knl=[0.0, 0.1], shift_x=1e-3, rot_s_rad=0.2),
                             xt.DipoleEdge(k=1e-3, e1=0.01, shift_y=1e-3),
                             xt.Multipole(knl=[0.0, 0.1], length=1.0, isthick=True),
                             xt.Quadrupole(length=1.0, k1=0.01)])
    recs = line._element_records()
    lib = _abi.load_library()
    cfg = _abi.XtgConfig()
    h = ctypes.c_void_p()
    assert pyoracle.validate(recs)[0] == _abi.XTG_OK
    st = lib.xtg_lattice_create(recs.ctypes.data_as(ctypes.c_void_p), 4, ctypes.byref(cfg),
                                ctypes.byref(h))
    assert st != _abi.XTG_E_UNSUPPORTED       # without a GPU: validated, then no device
    if st == _abi.XTG_OK:
        lib.xtg_lattice_destroy(h)
    for i, field in ((2, "shift_x"), (3, "rot_s_rad"), (0, "shift_s"), (1, "rot_y_rad")):
        bad = recs.copy()
        bad[i][field] = 1e-3
        st, msg = pyoracle.validate(bad)
        assert st == _abi.XTG_E_UNSUPPORTED and "misalignment" in msg
        st = lib.xtg_lattice_create(bad.ctypes.data_as(ctypes.c_void_p), 4, ctypes.byref(cfg),
                                    ctypes.byref(h))
        assert st == _abi.XTG_E_UNSUPPORTED and "misalignment" in _abi.last_error(lib)


def test_null_arguments_return_errors():
    lib = _abi.load_library()
    assert lib.xtg_lattice_create(None, 0, None, None) == _abi.XTG_E_NULL
    assert lib.xtg_track(None, None, 1, 0, 0, 0, 0, 0, 0, 0.0, None, 0, None) == _abi.XTG_E_NULL
    assert lib.xtg_lattice_destroy(None) == _abi.XTG_OK
    # the wait check validates its bound before touching the device
    assert lib.xtg_check_bounded_wait(0) == _abi.XTG_E_VALUE
    assert lib.xtg_check_bounded_wait(5_000_000_000) == _abi.XTG_E_VALUE


def test_particles_initialisation_formulas():
    delta = np.array([0.0, 1e-3, -2e-4])
    p = xt.Particles(p0c=7e12, delta=delta, zeta=[0.1, 0.0, -0.1], device="cpu")
    p0c, m = 7e12, PROTON_MASS_EV
    e0 = np.sqrt(p0c ** 2 + m ** 2)
    beta0 = p0c / e0
    np.testing.assert_array_equal(p.beta0.numpy(), beta0)
    np.testing.assert_array_equal(p.gamma0.numpy(), e0 / m)
    ptau = np.sqrt(delta ** 2 + 2 * delta + 1 / beta0 ** 2) - 1 / beta0
    np.testing.assert_array_equal(p.ptau.numpy(), ptau)
    db = delta * beta0
    ptb = np.sqrt(db ** 2 + 2 * db * beta0 + 1) - 1
    np.testing.assert_array_equal(p.rvv.numpy(), (1 + delta) / (1 + ptb))
    np.testing.assert_array_equal(p.rpp.numpy(), 1 / (1 + delta))
    assert p.state.tolist() == [1, 1, 1]
    assert p.particle_id.tolist() == [0, 1, 2]
    q = xt.Particles(p0c=1e9, ptau=[1e-3], device="cpu")
    b0 = q.beta0.numpy()
    np.testing.assert_array_equal(q.delta.numpy(), np.sqrt(1e-3 ** 2 + 2 * 1e-3 / b0 + 1) - 1)
    r = xt.Particles(p0c=1e9, x=[1.0], _capacity=4, device="cpu")
    assert r.state.tolist() == [1, -999999999, -999999999, -999999999]
    with pytest.raises(ValueError):
        xt.Particles(x=[1, 2], y=[1, 2, 3], device="cpu")


def test_bend_parameters_and_records():
    b = xt.Bend(length=2.0, angle=0.02)
    assert b.h == 0.01 and b.k0 == "from_h"
    r = b.to_record()
    assert r["k0"] == 0.01 and r["h"] == 0.01 and r["order"] == 5
    assert r["edge_entry_active"] == 1 and r["edge_entry_model"] == 0
    b.k0 = 0.02
    assert b.to_record()["k0"] == 0.02
    q = xt.Quadrupole(length=1.0, k1=0.1, knl_rel=[1e-3, 2e-3], ksl_rel=[1e-4])
    r = q.to_record()
    assert r["order_rel"] == 1 and r["ksl_rel"][1] == 0.0
    m = xt.Multipole(knl=[0, 1e-3, 0.1])
    assert m.order == 2 and m.to_record()["inv_factorial_order"] == 0.5
    e = xt.LimitEllipse(a=0.02, b=0.01)
    assert e.a_b_squ == (0.02 * 0.02) * (0.01 * 0.01)   # a_squ * b_squ (limit_ellipse.py:54)


def test_thin_slicing_sequence():
    line = xt.Line(elements=[xt.Drift(length=1.0), xt.Bend(length=2.0, angle=0.01),
                             xt.Quadrupole(length=1.0, k1=0.1)], element_names=["d", "b", "q"])
    line.slice_thick_elements([xt.Strategy(slicing=xt.Teapot(2)),
                               xt.Strategy(slicing=xt.Uniform(1, mode="thick"), name="q")])
    assert line.element_names == [
        "d", "b_entry", "b..entry_map", "drift_b..0", "b..0", "drift_b..1", "b..1",
        "drift_b..2", "b..exit_map", "b_exit", "q_entry", "q..entry_map", "q..0",
        "q..exit_map", "q_exit"]
    w = [line[n].weight for n in ("drift_b..0", "drift_b..1", "drift_b..2")]
    np.testing.assert_allclose(w, [1 / 6, 2 / 3, 1 / 6])
    assert isinstance(line["b..0"], xt.ThinSliceBend) and line["b..0"].weight == 0.5
    assert isinstance(line["q..0"], xt.ThickSliceQuadrupole) and line["q..0"].weight == 1.0
    np.testing.assert_allclose(line.get_length(), 4.0)


def test_line_dict_roundtrip():
    from lattice_cases import sliced_line
    line = sliced_line(thin=True)
    again = xt.Line.from_dict(line.to_dict())
    assert again.element_names == line.element_names
    assert np.array_equal(again._element_records(), line._element_records())


def test_turn_split(monkeypatch):
    """tracker.py:1270-1336: first partial turn, middle turns, last turn.
    A first turn that is a whole turn with the middle turns' end-of-turn
    actions joins them in one call (the same arguments but the turn count,
    so the same result)."""
    calls = []

    class FakeTracker(xt.Tracker):
        def __init__(self, line):
            self.line = line
            self.num_elements = len(line.element_names)
            self.track_flags = xt.TrackFlags()
            self.frozen_longitudinal = False
            self.line_length = line.get_length()
            self.record_last_track = None
            self.time_last_track = None

        def _launch(self, pstruct, num_turns, ele_start, num_ele_track, flag_end,
                    flag_monitor, mstruct, flags, stream):
            calls.append((num_turns, ele_start, num_ele_track, bool(flag_end)))

    line = xt.Line(elements=[xt.Drift(length=1.0) for _ in range(10)])

    class P:
        start_tracking_at_element = -1

        class device:
            type = "cuda"

        def _xtg_struct(self):
            return None

    tr = FakeTracker(line)
    monkeypatch.setattr(torch.cuda, "current_stream", lambda d: type("S", (), {"cuda_stream": 0})())
    monkeypatch.setattr(torch.cuda, "device", lambda d: __import__("contextlib").nullcontext())
    cases = [
        (dict(num_turns=3), [(3, 0, 10, True)]),
        (dict(num_turns=1), [(1, 0, 10, True)]),
        (dict(ele_start=4, num_turns=2), [(1, 4, 6, True), (1, 0, 10, True)]),
        (dict(ele_start=3, ele_stop=7), [(1, 3, 4, False)]),
        (dict(ele_start=7, ele_stop=3), [(1, 7, 3, True), (1, 0, 3, False)]),
        (dict(ele_start=2, ele_stop=5, num_turns=3), [(1, 2, 8, True), (1, 0, 10, True),
                                                      (1, 0, 5, False)]),
        (dict(num_elements=25), [(2, 0, 10, True), (1, 0, 5, False)]),
        (dict(ele_start=5, num_elements=3), [(1, 5, 3, False)]),
    ]
    for kw, expected in cases:
        calls.clear()
        tr._track(P(), **kw)
        got = [c for c in calls if c[0] > 0 or c[2] > 0]
        assert got == expected, (kw, calls)
    # without end-of-turn actions the calls' arguments agree as well
    line.skip_end_turn_actions = True
    calls.clear()
    tr._track(P(), num_turns=3)
    assert calls == [(3, 0, 10, False)], calls
    calls.clear()
    tr._track(P(), ele_start=4, num_turns=2)
    assert calls == [(1, 4, 6, False), (1, 0, 10, False)], calls


def _shard_worker(rank, world, port, n, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from xtrack_gb300.parallel import shard_range
    lo, hi = shard_range(n, rank, world)
    t = torch.tensor([lo, hi], dtype=torch.int64)
    g = [torch.zeros(2, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(g, t)
    if rank == 0:
        out.put([x.tolist() for x in g])
    dist.destroy_process_group()


def _free_port():
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _run_ranks(target, world, *args):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, world, port) + args + (q,)) for r in range(world)]
    for p in procs:
        p.start()
    res = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    return res


def test_particle_sharding_gloo_two_ranks():
    ranges = _run_ranks(_shard_worker, 2, 1_000_001)
    assert ranges[0][0] == 0 and ranges[0][1] == ranges[1][0] and ranges[1][1] == 1_000_001


def _oracle_track(line, shard, num_turns=1):
    # the per-shard push of this CPU test: the oracle on the shard's arrays
    import pyoracle
    from xtrack_gb300.parallel import TRACKED_FIELDS
    arrs = pyoracle.host_arrays(shard.to_numpy())
    pyoracle.track(line._element_records(), arrs, num_turns=num_turns,
                   line_length=line.get_length())
    for f in TRACKED_FIELDS:
        setattr(shard, f, torch.from_numpy(arrs[f]))


def _sharded_track_worker(rank, world, port, n, turns, out):
    import sys
    import torch.distributed as dist
    sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from lattice_cases import small_beam
    from xtrack_gb300 import workloads
    from xtrack_gb300.parallel import track_sharded
    line = workloads.toy_ring()
    p = xt.Particles(device="cpu", **small_beam(n, p0c=450e9, seed=41, scale=7.0))
    # ids out of slot order: sharding goes by particle_id, not by slot
    perm = np.random.default_rng(3).permutation(n)
    p.particle_id = torch.from_numpy(perm)
    track_sharded(line, p, device="cpu", track=_oracle_track, num_turns=turns)
    if rank == 0:
        out.put(p.to_numpy())
    dist.destroy_process_group()


def test_sharded_track_gloo_two_ranks_equals_one_run():
    """One beam split by particle_id over two gloo ranks, each tracking its
    shard (through the oracle in this CPU test) and gathering the results:
    bit-identical to one unsharded run, losses included."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from lattice_cases import small_beam
    from xtrack_gb300 import workloads
    n, turns = 301, 12
    got = _run_ranks(_sharded_track_worker, 2, n, turns)
    line = workloads.toy_ring()
    p = xt.Particles(device="cpu", **small_beam(n, p0c=450e9, seed=41, scale=7.0))
    p.particle_id = torch.from_numpy(np.random.default_rng(3).permutation(n))
    ref = pyoracle.host_arrays(p.to_numpy())
    pyoracle.track(line._element_records(), ref, num_turns=turns, line_length=line.get_length())
    assert 10 < int(np.sum(ref["state"] <= 0)) < n - 10
    for f in ("x", "px", "y", "py", "zeta", "delta", "ptau", "rpp", "rvv", "s", "state",
              "at_turn", "at_element", "particle_id"):
        assert np.array_equal(np.asarray(got[f]).view(np.int64), np.asarray(ref[f]).view(np.int64)), f
