"""xtg_track_noalloc: the allocation-free variant of xtg_track (scratch in a
static device array) against xtg_track on the same inputs, two calls in a
row, with a turn-by-turn monitor, its capacity limit and its rejection of
backtracking before the reversed table exists. Named to be collected last;
it also passes on its own."""
import ctypes

import numpy as np
import pytest

import pyoracle
import xtrack_gb300 as xt
from xtrack_gb300 import _abi, workloads
from lattice_cases import small_beam

pytestmark = pytest.mark.gpu


def _lattice(lib, recs, arith):
    cfg = _abi.XtgConfig()
    cfg.has_global_xy_limit = 1
    cfg.global_xy_limit = 1.0
    cfg.arith = _abi.ARITH_EXACT if arith == "exact" else _abi.ARITH_FAST
    h = ctypes.c_void_p()
    recs = np.ascontiguousarray(recs)
    _abi.check(lib.xtg_lattice_create(recs.ctypes.data_as(ctypes.c_void_p), len(recs),
                                      ctypes.byref(cfg), ctypes.byref(h)), lib)
    return h


def _device_arrays(arrs):
    import torch
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in arrs.items()}
    ps = _abi.particles_struct_from_ptrs(len(arrs["x"]), 1.0, 938272088.16, 0.0,
                                         {k: v.data_ptr() for k, v in t.items()})
    return t, ps


def _call(lib, fn, h, ps, n, L, turns):
    _abi.check(fn(h, ctypes.byref(ps), turns, 0, n, 1, 1, 0, n, L, None, 0, None), lib)
    _abi.check(lib.xtg_sync(None), lib)


@pytest.mark.parametrize("arith", ["exact", "fast"])
def test_noalloc_equals_track_on_two_calls_in_a_row(arith):
    import torch
    lib = _abi.load_library()
    line = workloads.toy_ring()
    recs = line._element_records()
    L = line.get_length()
    p = xt.Particles(device="cpu", **small_beam(5000, p0c=450e9, seed=77, scale=8.0))
    arrs = pyoracle.host_arrays(p.to_numpy())
    h_ref = _lattice(lib, recs, arith)
    h_na = _lattice(lib, recs, arith)
    try:
        t = _abi.XtgTuning(block_size=128, compact_every=3, chunk_bytes=0, use_graph=0)
        _abi.check(lib.xtg_set_tuning(h_na, ctypes.byref(t)), lib)
        ref, ps_ref = _device_arrays(arrs)
        got, ps_got = _device_arrays(arrs)
        for _ in range(2):
            _call(lib, lib.xtg_track, h_ref, ps_ref, len(recs), L, 7)
            _call(lib, lib.xtg_track_noalloc, h_na, ps_got, len(recs), L, 7)
            lost = int((ref["state"] <= 0).sum())
            for f in ref:
                a, b = got[f], ref[f]
                if a.dtype == torch.float64:
                    a, b = a.view(torch.int64), b.view(torch.int64)
                assert torch.equal(a, b), f
        assert lost > 100
        # the device-side status of both paths reads clean
        _abi.check(lib.xtg_device_status(h_na), lib)
        # and the calls allocated nothing on the device
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        big = pyoracle.host_arrays(xt.Particles(
            device="cpu", **small_beam(300000, p0c=450e9, seed=78)).to_numpy())
        tb, psb = _device_arrays(big)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        _call(lib, lib.xtg_track_noalloc, h_na, psb, len(recs), L, 2)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free1
        assert free1 <= free0
    finally:
        lib.xtg_lattice_destroy(h_ref)
        lib.xtg_lattice_destroy(h_na)


def test_noalloc_rejects_capacity_above_limit():
    import torch
    lib = _abi.load_library()
    line = workloads.toy_ring()
    recs = line._element_records()
    h = _lattice(lib, recs, "exact")
    try:
        arrs = pyoracle.host_arrays(xt.Particles(device="cpu", **small_beam(16)).to_numpy())
        t, ps = _device_arrays(arrs)
        before = {k: v.clone() for k, v in t.items()}
        ps.capacity = _abi.XTG_NOALLOC_MAX_PARTICLES + 1   # checked before any access
        st = lib.xtg_track_noalloc(h, ctypes.byref(ps), 1, 0, len(recs), 1, 1, 0, len(recs),
                                   line.get_length(), None, 0, None)
        assert st == _abi.XTG_E_CAPACITY
        assert "static scratch limit" in _abi.last_error(lib)
        torch.cuda.synchronize()
        for k in t:
            assert torch.equal(t[k], before[k])
    finally:
        lib.xtg_lattice_destroy(h)


def test_noalloc_rejects_backtracking_before_the_reversed_table_exists():
    lib = _abi.load_library()
    line = workloads.toy_ring()
    recs = line._element_records()
    h = _lattice(lib, recs, "exact")
    try:
        arrs = pyoracle.host_arrays(xt.Particles(device="cpu", **small_beam(64)).to_numpy())
        t, ps = _device_arrays(arrs)
        st = lib.xtg_track_noalloc(h, ctypes.byref(ps), 1, 0, len(recs), 0, 0, 0, len(recs),
                                   line.get_length(), None, 1 << _abi.FLAG_BACKTRACK, None)
        assert st == _abi.XTG_E_VALUE
        assert "backtracking table" in _abi.last_error(lib)
    finally:
        lib.xtg_lattice_destroy(h)


@pytest.mark.parametrize("arith", ["exact", "fast"])
def test_noalloc_with_monitor_equals_track(arith):
    import torch
    from xtg_testutil import make_monitor
    lib = _abi.load_library()
    line = workloads.toy_ring()
    recs = line._element_records()
    L = line.get_length()
    n = len(recs)
    arrs = pyoracle.host_arrays(xt.Particles(device="cpu", **small_beam(300, p0c=450e9, seed=5,
                                                                          scale=6.0)).to_numpy())
    h_ref = _lattice(lib, recs, arith)
    h_na = _lattice(lib, recs, arith)
    try:
        out = []
        for h, fn in ((h_ref, lib.xtg_track), (h_na, lib.xtg_track_noalloc)):
            mon = make_monitor(0, 6, (0, 300))
            t, ps = _device_arrays(arrs)
            md = {k: torch.from_numpy(v).cuda() for k, v in mon["data"].items()}
            mst = _abi.XtgMonitor()
            for k in ("start_at_turn", "stop_at_turn", "part_id_start", "part_id_end",
                      "ebe_mode", "n_repetitions", "repetition_period", "n_records"):
                setattr(mst, k, int(mon[k]))
            mst.data = _abi.particles_struct_from_ptrs(mon["n_records"], 0., 0., 0.,
                                                       {k: v.data_ptr() for k, v in md.items()})
            _abi.check(fn(h, ctypes.byref(ps), 6, 0, n, 1, 1, 1, n, L, ctypes.byref(mst), 0, None),
                       lib)
            _abi.check(lib.xtg_sync(None), lib)
            out.append(({k: v.cpu().numpy() for k, v in t.items()},
                        {k: v.cpu().numpy() for k, v in md.items()}))
        (pa, ma), (pb, mb) = out
        for f in pa:
            assert np.array_equal(pa[f].view(np.int64), pb[f].view(np.int64)), f
        for f in ma:
            assert np.array_equal(ma[f].view(np.int64), mb[f].view(np.int64)), f
        assert np.count_nonzero(ma["at_turn"]) > 0
        _abi.check(lib.xtg_device_status(h_na), lib)
    finally:
        lib.xtg_lattice_destroy(h_ref)
        lib.xtg_lattice_destroy(h_na)
