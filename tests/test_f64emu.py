"""The integer-pipe binary64 multiply (xtg_f64emu.cuh) that the exact push
uses for its products: bit for bit equal to the hardware multiply.

The host form (xtg_f64_mul_host) is compared with numpy's multiply on the
CPU; the device form (xtg_f64_mul_device) with the GPU's own FP64 multiply
and with numpy. Operands cover random bit patterns (NaN, infinities,
subnormals, zeros included), every pair of exponents near the edges of the
normal range (underflow, overflow, the integer path's bounds), short
significands (exact products and ties) and the magnitudes of tracking."""
import ctypes

import numpy as np
import pytest

from xtrack_gb300 import _abi


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def _operands(n, seed):
    rng = np.random.default_rng(seed)
    parts = []
    # any bit pattern
    parts.append((rng.integers(0, 2**64, n, dtype=np.uint64, endpoint=False),
                  rng.integers(0, 2**64, n, dtype=np.uint64, endpoint=False)))
    # normal operands of moderate exponents, full and short significands
    for mask in (0x000FFFFFFFFFFFFF, 0x000FFFFFFF000000, 0x000FFF0000000000):
        ea = rng.integers(1023 - 100, 1023 + 100, n).astype(np.uint64)
        eb = rng.integers(1023 - 100, 1023 + 100, n).astype(np.uint64)
        fa = rng.integers(0, 2**52, n, dtype=np.uint64) & np.uint64(mask)
        fb = rng.integers(0, 2**52, n, dtype=np.uint64) & np.uint64(mask)
        sa = rng.integers(0, 2, n).astype(np.uint64) << np.uint64(63)
        sb = rng.integers(0, 2, n).astype(np.uint64) << np.uint64(63)
        parts.append((sa | (ea << np.uint64(52)) | fa, sb | (eb << np.uint64(52)) | fb))
    # exponent pairs at the edges of the range, zeros and all-ones fractions
    ex = np.r_[np.arange(0, 40), np.arange(1000, 1050), np.arange(2008, 2048)].astype(np.uint64)
    ea, eb = np.meshgrid(ex, ex)
    ea, eb = ea.ravel(), eb.ravel()
    m = len(ea)
    for fa_kind in range(3):
        fa = rng.integers(0, 2**52, m, dtype=np.uint64)
        if fa_kind == 1:
            fa[:] = 0
        elif fa_kind == 2:
            fa[:] = 0x000FFFFFFFFFFFFF
        fb = rng.integers(0, 2**52, m, dtype=np.uint64)
        fb[::7] = 0
        sa = rng.integers(0, 2, m).astype(np.uint64) << np.uint64(63)
        parts.append((sa | (ea << np.uint64(52)) | fa, (eb << np.uint64(52)) | fb))
    a = np.concatenate([p[0] for p in parts]).view(np.float64)
    b = np.concatenate([p[1] for p in parts]).view(np.float64)
    # tracking magnitudes: coordinates times coefficients
    a2 = rng.normal(0, 1e-3, n) * np.exp(rng.normal(0, 3, n))
    b2 = rng.normal(0, 1e-4, n) * np.exp(rng.normal(0, 3, n))
    return np.r_[a, a2], np.r_[b, b2]


def _same(got, ref):
    gb, rb = _bits(got), _bits(ref)
    nan = np.isnan(got) & np.isnan(ref)
    return (gb == rb) | nan


def test_host_multiply_matches_numpy():
    lib = _abi.load_library()
    a, b = _operands(400_000, seed=1)
    out = np.empty_like(a)
    _abi.check(lib.xtg_f64_mul_host(a.ctypes.data, b.ctypes.data, out.ctypes.data, len(a)))
    with np.errstate(all="ignore"):
        ref = a * b
    ok = _same(out, ref)
    assert ok.all(), f"{(~ok).sum()} mismatches, first: {a[~ok][:3]} * {b[~ok][:3]}"


def test_host_multiply_rejects_bad_arguments():
    lib = _abi.load_library()
    assert lib.xtg_f64_mul_host(None, None, None, -1) == _abi.XTG_E_VALUE
    assert lib.xtg_f64_mul_host(None, None, None, 4) == _abi.XTG_E_NULL
    assert lib.xtg_f64_mul_host(None, None, None, 0) == _abi.XTG_OK


@pytest.mark.gpu
def test_device_multiply_matches_hardware():
    import torch
    lib = _abi.load_library()
    a, b = _operands(1_000_000, seed=2)
    ta = torch.from_numpy(a).cuda()
    tb = torch.from_numpy(b).cuda()
    out = torch.empty_like(ta)
    _abi.check(lib.xtg_f64_mul_device(ctypes.c_void_p(ta.data_ptr()), ctypes.c_void_p(tb.data_ptr()),
                                      ctypes.c_void_p(out.data_ptr()), len(a), None))
    _abi.check(lib.xtg_sync(None))
    hw = (ta * tb).cpu().numpy()
    got = out.cpu().numpy()
    ok = _same(got, hw)
    assert ok.all(), f"{(~ok).sum()} mismatches vs the GPU multiply, first: {a[~ok][:3]} * {b[~ok][:3]}"
    with np.errstate(all="ignore"):
        ok = _same(got, a * b)
    assert ok.all(), f"{(~ok).sum()} mismatches vs numpy"


@pytest.mark.gpu
def test_emulated_multiply_rate_is_measured():
    lib = _abi.load_library()
    v = ctypes.c_double()
    _abi.check(lib.xtg_measure_emul_rate(ctypes.byref(v)))
    assert v.value > 1e10
