"""Reader for the golden fixtures in tests/golden/ (written by oracle/ref_dump.cpp
from the reference implementation itself) and the seeded input generator that
reproduces the fixture inputs bit-for-bit.

Record format: b"SYKG", then repeated
  u32 name_len | name | u8 dtype (0=i32, 1=f64) | u64 count | payload.
"""
import gzip
import os
import struct

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# tags used by oracle/ref_dump.cpp for its seeded inputs
TAG = dict(op_x=1, op_rhs=2, sm_corr0=3, sm_resid=4, rs_in=5, pr_in=6, fx_phi=7,
           vc_p=8, bc_phi=9, bc_rhs0=10, sv_rand=11)

# per-fixture seeds (must match make_case() in oracle/ref_dump.cpp)
SEEDS = dict(c1=20251, t2s=777, t2b=4242, t3s=99, t3n=31337)


def load(name):
    path = os.path.join(GOLDEN_DIR, name + ".bin.gz")
    with gzip.open(path, "rb") as f:
        buf = f.read()
    assert buf[:4] == b"SYKG", path
    out = {}
    p = 4
    while p < len(buf):
        (nl,) = struct.unpack_from("<I", buf, p)
        p += 4
        key = buf[p:p + nl].decode()
        p += nl
        dt = buf[p]
        p += 1
        (n,) = struct.unpack_from("<Q", buf, p)
        p += 8
        if dt == 0:
            arr = np.frombuffer(buf, dtype="<i4", count=n, offset=p).copy()
            p += 4 * n
        else:
            arr = np.frombuffer(buf, dtype="<f8", count=n, offset=p).copy()
            p += 8 * n
        out[key] = arr
    return out


def _splitmix64(x):
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def seeded(seed, tag, n):
    """value[i] = 2 * (splitmix64(seed*2^32 + tag*2^20 + i) >> 11) * 2^-53 - 1"""
    base = (np.uint64(seed) << np.uint64(32)) + (np.uint64(tag) << np.uint64(20))
    z = _splitmix64(base + np.arange(n, dtype=np.uint64))
    return 2.0 * ((z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)) - 1.0


def seeded_input(fixture, key, n):
    return seeded(SEEDS[fixture], TAG[key], n)
