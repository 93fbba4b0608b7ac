#!/bin/bash
# Regenerates the golden fixtures in this directory from the reference
# implementation itself (haloless/SayakaAmr compiled from its unmodified
# sources by oracle/Makefile).  Needs the reference checkout at
# /root/reference (or REF=<path to its src/>); not run on the GPU host.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(cd "$HERE/../.." && pwd)"
make -C "$ROOT/oracle" -j8 ${REF:+REF=$REF} >/dev/null
TMP="$(mktemp -d)"
"$ROOT/oracle/_ref/ref_dump2" "$TMP" t2s t2b c1 rg2 n2 tf2 > "$TMP/log2.txt" 2>&1
"$ROOT/oracle/_ref/ref_dump3" "$TMP" t3s t3n rg3 n3 tf3 > "$TMP/log3.txt" 2>&1
# 16^d-cell cases: FP64 arrays kept as digests
for c in n2 n3; do
  python3 "$HERE/digest_fixture.py" "$TMP/$c.bin" "$TMP/$c.d.bin"
  mv "$TMP/$c.d.bin" "$TMP/$c.bin"
done
for f in "$TMP"/*.bin; do
  gzip -9 -n -c "$f" > "$HERE/$(basename "$f").gz"
done
grep -h '^\[' "$TMP"/log*.txt
rm -rf "$TMP"
