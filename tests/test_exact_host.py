"""CPU tests of the product's exact f32 helpers (retrofire_gb300/csrc/rf_exact.cuh).

rfx::seq_add_n(s, d, k) must equal k sequential IEEE additions bit for bit:
the tile rasteriser relies on it to enter scanlines and spans mid-way and
still reproduce the running sums of Iter::next (core/src/math/vary.rs:142-155).
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("shim") / "libseqsum.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                           os.path.join(HERE, "csrc", "seqsum_shim.cpp"), "-o", out])
    L = C.CDLL(out)
    L.shim_seq_add_n.argtypes = [C.c_float, C.c_float, C.c_uint32]
    L.shim_seq_add_n.restype = C.c_float
    L.shim_check.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64,
                             C.POINTER(C.c_uint64)]
    L.shim_check.restype = C.c_uint64
    L.shim_check_fast.argtypes = L.shim_check.argtypes
    L.shim_check_fast.restype = C.c_uint64
    return L


def _check(L, s, d, k):
    s = np.ascontiguousarray(s, np.float32)
    d = np.ascontiguousarray(d, np.float32)
    k = np.ascontiguousarray(k, np.uint32)
    for fn in (L.shim_check, L.shim_check_fast):
        fb = C.c_uint64(0)
        bad = fn(s.ctypes.data, d.ctypes.data, k.ctypes.data, s.size, C.byref(fb))
        if bad:
            i = fb.value
            pytest.fail("%s: %d mismatches; first s=%r d=%r k=%d"
                        % (fn.__name__, bad, s[i], d[i], k[i]))


def test_vary_kats(shim):
    """vary.rs:163-191 and the doc examples (vary.rs:36-46, 56-64)."""
    f = shim.shim_seq_add_n
    assert [f(0.0, 0.2, i) for i in range(5)] == [np.float32(x) for x in
                                                  (0.0, 0.2, 0.4, np.float32(0.4) + np.float32(0.2),
                                                   np.float32(np.float32(0.4) + np.float32(0.2)) + np.float32(0.2))]
    assert [f(2.0, 3.0, i) for i in range(3)] == [2.0, 5.0, 8.0]


def test_random_bits(shim):
    rng = np.random.default_rng(1)
    n = 300_000
    s = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
    d = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
    k = rng.integers(0, 64, n).astype(np.uint32)
    _check(shim, s, d, k)


def test_screen_like(shim):
    """Values and steps of the kind scanlines produce, long runs."""
    rng = np.random.default_rng(2)
    n = 200_000
    s = rng.uniform(-3000, 3000, n).astype(np.float32)
    d = (rng.uniform(-4, 4, n) * np.exp2(-rng.integers(0, 24, n))).astype(np.float32)
    k = rng.integers(0, 4096, n).astype(np.uint32)
    _check(shim, s, d, k)


def test_zero_crossing_and_ties(shim):
    rng = np.random.default_rng(3)
    n = 200_000
    s = (rng.integers(-4000, 4000, n) * 0.5).astype(np.float32)
    d = (rng.integers(-64, 64, n) * np.exp2(-rng.integers(0, 30, n).astype(np.float64))).astype(np.float32)
    k = rng.integers(0, 3000, n).astype(np.uint32)
    _check(shim, s, d, k)
    # crossing zero from both sides with steps of every binade
    s2 = rng.uniform(-1, 1, n).astype(np.float32)
    d2 = (-np.sign(s2) * rng.uniform(0, 1, n) * np.exp2(-rng.integers(0, 20, n))).astype(np.float32)
    k2 = rng.integers(0, 2000, n).astype(np.uint32)
    _check(shim, s2, d2, k2)


def test_subnormal_and_specials(shim):
    rng = np.random.default_rng(4)
    n = 100_000
    s = (rng.integers(0, 1 << 23, n).astype(np.uint32) |
         (rng.integers(0, 2, n).astype(np.uint32) << 31)).view(np.float32)
    d = (rng.integers(0, 1 << 24, n).astype(np.uint32) |
         (rng.integers(0, 2, n).astype(np.uint32) << 31)).view(np.float32)
    k = rng.integers(0, 500, n).astype(np.uint32)
    _check(shim, s, d, k)
    sp = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 3.4e38, -3.4e38], np.float32)
    S, D = np.meshgrid(sp, sp)
    for kk in (0, 1, 2, 7, 1000):
        _check(shim, S.ravel(), D.ravel(), np.full(S.size, kk, np.uint32))
