"""Shrinks a golden fixture written by oracle/ref_dump.cpp for a large case
(16^d-cell blocks): every FP64 array beyond a few values is replaced by its
digest, a SHA-256 over the values with both zeros and every NaN made
canonical (digest record: dtype 2, count = the array's length, 32-byte
payload).  Integer tables, scalars and block geometry stay whole.  The tests
compare their own results through the same digest (golden_io.digest), so a
digest match is a bit-for-bit match of the array.

    python digest_fixture.py IN.bin OUT.bin
"""
import struct
import sys

import numpy as np

KEEP_WHOLE = ("block_lo", "block_hi", "block_len", "block_center")
SMALL = 64


def canonical_digest(a):
    import hashlib
    a = np.asarray(a, dtype="<f8").copy()
    a[a == 0] = 0.0
    a[np.isnan(a)] = np.nan
    return hashlib.sha256(a.tobytes()).digest()


def shrink(src, dst):
    buf = open(src, "rb").read()
    assert buf[:4] == b"SYKG", src
    out = [b"SYKG"]
    p = 4
    while p < len(buf):
        (nl,) = struct.unpack_from("<I", buf, p)
        name = buf[p + 4:p + 4 + nl]
        p += 4 + nl
        dt = buf[p]
        (n,) = struct.unpack_from("<Q", buf, p + 1)
        p += 9
        esz = 4 if dt == 0 else 8
        payload = buf[p:p + esz * n]
        p += esz * n
        head = struct.pack("<I", nl) + name
        if dt == 1 and n > SMALL and name.decode() not in KEEP_WHOLE:
            arr = np.frombuffer(payload, dtype="<f8")
            out.append(head + struct.pack("<BQ", 2, n) + canonical_digest(arr))
        else:
            out.append(head + struct.pack("<BQ", dt, n) + payload)
    open(dst, "wb").write(b"".join(out))


if __name__ == "__main__":
    shrink(sys.argv[1], sys.argv[2])
