"""The device solve's FP64 bookkeeping on the integer pipe (mac_fp.cuh)
against the hardware conversions, bit for bit: double -> float rounding to
nearest even (ties, carries into the exponent, the float range edges,
denormals, inf, NaN, signed zeros) and the exact float -> double widening."""
import numpy as np
import pytest

import sayakaamr_gb300 as sg

pytestmark = pytest.mark.gpu


def edge_doubles():
    f32 = np.finfo(np.float32)
    vals = [0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, float(f32.max), -float(f32.max), float(f32.tiny),
            float(f32.tiny) / 2, float(f32.tiny) * (1 - 2 ** -30), float(f32.max) * (1 + 2 ** -25),
            float(f32.max) * (1 + 2 ** -24), float(f32.max) * (1 + 2 ** -23), 1e-45, 1.4e-45, 7e-46, 1e-300,
            1e300, 3.0e38, 3.5e38, 5e-324]
    out = np.array(vals, dtype=np.float64)
    # exact ties and near-ties of the 29 dropped mantissa bits, even and odd
    rng = np.random.default_rng(5)
    base = rng.uniform(-1e3, 1e3, 400).astype(np.float32).astype(np.float64).view(np.uint64)
    half = np.uint64(1 << 28)
    ties = np.concatenate([base + half, base + half - np.uint64(1), base + half + np.uint64(1),
                           base + np.uint64((1 << 29) - 1), (base | np.uint64((1 << 29) - 1)) + np.uint64(1) - half,
                           base + (np.uint64(1) << np.uint64(29)) + half])
    return np.concatenate([out, ties.view(np.float64)])


def random_doubles(rng, n):
    # exponents spread over the whole double range, weighted toward floats'
    e = np.concatenate([rng.integers(0, 2047, n // 4), rng.integers(850, 1200, 3 * n // 4)])
    m = rng.integers(0, 1 << 52, len(e), dtype=np.uint64)
    s = rng.integers(0, 2, len(e)).astype(np.uint64) << np.uint64(63)
    return (s | (e.astype(np.uint64) << np.uint64(52)) | m).view(np.float64)


def random_floats(rng, n):
    u = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    return np.concatenate([u.view(np.float32), np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45,
                                                        1.17549435e-38, 3.4028235e38], dtype=np.float32)])


def same_bits(a, b):
    """bitwise equal, except that any NaN matches any NaN"""
    na, nb = np.isnan(a), np.isnan(b)
    assert np.array_equal(na, nb)
    ia = a.view(np.uint32 if a.dtype == np.float32 else np.uint64)[~na]
    ib = b.view(np.uint32 if b.dtype == np.float32 else np.uint64)[~nb]
    bad = np.nonzero(ia != ib)[0]
    assert len(bad) == 0, (a[~na][bad[:5]], b[~nb][bad[:5]])


def test_integer_pipe_conversions_match_hardware():
    rng = np.random.default_rng(17)
    d = np.concatenate([edge_doubles(), random_doubles(rng, 200000)])
    f = random_floats(rng, len(d) - 9)
    assert len(f) == len(d)
    nar, nar_hw, wid, wid_hw, wid0, wid0_hw = sg.fp_selftest(d, f)
    same_bits(nar, nar_hw)
    same_bits(wid, wid_hw)
    same_bits(wid0, wid0_hw)
    # and against numpy's IEEE conversions where no NaN is involved
    ok = ~np.isnan(d)
    with np.errstate(over="ignore"):
        same_bits(nar[ok], d[ok].astype(np.float32))
