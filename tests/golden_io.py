"""Reader for the golden fixtures in tests/golden/ (written by oracle/ref_dump.cpp
from the reference implementation itself) and the seeded input generator that
reproduces the fixture inputs bit-for-bit.

Record format: b"SYKG", then repeated
  u32 name_len | name | u8 dtype (0=i32, 1=f64, 2=digest) | u64 count | payload.
A digest record (fixtures of the 16^d-cell cases, tests/golden/digest_fixture.py)
stands for an FP64 array of `count` values by the SHA-256 of its canonical
bytes; load() returns it as a Digest, and the inputs the tests need whole
(face B, the solve's right-hand side) are regenerated here and checked
against their digests.
"""
import gzip
import hashlib
import math
import os
import struct

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# tags used by oracle/ref_dump.cpp for its seeded inputs
TAG = dict(op_x=1, op_rhs=2, sm_corr0=3, sm_resid=4, rs_in=5, pr_in=6, fx_phi=7,
           vc_p=8, bc_phi=9, bc_rhs0=10, sv_rand=11)

# iterations of the mg_solve / relax_solve dumps (kMgIters, kRelaxIters of
# oracle/ref_dump.cpp), run with a relative tolerance of 1e-30
MG_ITERS, RELAX_ITERS = 6, 25

# per-fixture seeds (must match make_case() in oracle/ref_dump.cpp)
SEEDS = dict(c1=20251, t2s=777, t2b=4242, t3s=99, t3n=31337, n2=1616, n3=4096)


def digest(a):
    """SHA-256 over FP64 values with both zeros and every NaN made canonical"""
    a = np.asarray(a, dtype="<f8").copy()
    a[a == 0] = 0.0
    a[np.isnan(a)] = np.nan
    return hashlib.sha256(a.tobytes()).digest()


class Digest:
    """an FP64 fixture array held as its digest"""

    def __init__(self, raw, n):
        self.raw, self.size = raw, int(n)

    def matches(self, a):
        a = np.asarray(a, dtype=np.float64).reshape(-1)
        return a.size == self.size and digest(a) == self.raw

    def __repr__(self):
        return "Digest(%s..., n=%d)" % (self.raw.hex()[:12], self.size)


def matches(a, ref):
    """bit-for-bit equality of an FP64 result with a fixture array or digest
    (-0.0 and +0.0 are the same value)"""
    if isinstance(ref, Digest):
        return ref.matches(a)
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(ref, dtype=np.float64)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


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
        elif dt == 2:
            arr = Digest(bytes(buf[p:p + 32]), n)
            p += 32
        else:
            arr = np.frombuffer(buf, dtype="<f8", count=n, offset=p).copy()
            p += 8 * n
        out[key] = arr
    _regenerate(name, out)
    return out


def _leaf(g):
    return g["tower_%d_blocks" % int(g["finest_level"][0])]


def face_b(g, bamp):
    """leaf face B of ref_dump.cpp's run_case: 1 + bamp sin(2 pi x) cos(2 pi y)
    at the face centre, floored to a multiple of 1/1024; other blocks -777
    (libm sin/cos, correctly rounded, as the reference's)"""
    nd, nb, n = int(g["ndim"][0]), int(g["nb"][0]), int(g["num_blocks"][0])
    lo = g["block_lo"].reshape(n, 3)
    dx = g["block_len"].reshape(n, 3) / nb
    out = []
    two_pi = 2 * math.pi
    for fd in range(nd):
        ext = [nb + (d == fd) for d in range(nd)]
        per = int(np.prod(ext))
        a = np.full((n, per), -777.0)
        idx = np.stack(np.meshgrid(*[np.arange(e) for e in ext[::-1]], indexing="ij")[::-1], axis=-1).reshape(-1, nd)
        for b in _leaf(g):
            pts = [lo[b, d] + (idx[:, d] + 0.5) * dx[b, d] for d in range(nd)]
            pts[fd] = pts[fd] - 0.5 * dx[b, fd]
            v = np.array([1.0 + bamp * math.sin(two_pi * x0) * math.cos(two_pi * x1)
                          for x0, x1 in zip(pts[0], pts[1])])
            a[b] = np.floor(v * 1024.0) / 1024.0
        out.append(a.reshape(-1))
    return out


def solve_rhs(g, seed):
    """the random right-hand side of a solve case (not all-Neumann): the
    seeded values on the finest tower's blocks, 0 elsewhere, negated"""
    nd, nb, n = int(g["ndim"][0]), int(g["nb"][0]), int(g["num_blocks"][0])
    nc = nb ** nd
    r = seeded(seed, TAG["sv_rand"], n * nc).reshape(n, nc)
    f = np.zeros((n, nc))
    leaf = _leaf(g)
    f[leaf] = r[leaf]
    return (-f).reshape(-1)


# leaf B amplitude of the digest-only fixtures (make_case in oracle/ref_dump.cpp)
BAMP = dict(n2=0.5, n3=0.5)


def _regenerate(name, g):
    if isinstance(g.get("in_b0"), Digest):
        for d, a in enumerate(face_b(g, BAMP[name])):
            assert g["in_b%d" % d].matches(a), "regenerated face B %d of %s differs from the fixture" % (d, name)
            g["in_b%d" % d] = a
    if isinstance(g.get("sv_rhs"), Digest):
        a = solve_rhs(g, SEEDS[name])
        assert g["sv_rhs"].matches(a), "regenerated right-hand side of %s differs from the fixture" % name
        g["sv_rhs"] = a


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
