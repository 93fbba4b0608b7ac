"""Build recipe for the native library (CUDA kernels + C ABI + host tree) and
for the CPU oracle used by the tests.

    python -m sayakaamr_gb300.build            # library + oracle
Outputs (git-ignored):
    sayakaamr_gb300/_lib/libsayaka_gb300.so
    oracle/build/libsayaka_oracle.so
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(PKG, "_lib", "obj")
LIB = os.path.join(LIBDIR, "libsayaka_gb300.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "build", "libsayaka_oracle.so")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
# -fmad=false: FP64 stencils must round exactly like the reference's
# (no fused multiply-add), so parity against it can be bit-exact.
NVCC_FLAGS = ["-O3", "-std=c++17", ARCH, "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O2", "--expt-relaxed-constexpr"]
SOURCES = ["tree.cpp", "tower.cpp", "abi.cpp", "mac_solver.cu", "mac_kernels.cu", "mac_fast.cu", "mac_vcycle.cu",
           "mac_noalloc.cu", "mac_projection.cu", "mac_coef.cu",
           "mac_learned.cu", "mac_transfer.cu"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force=False, verbose=False):
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "sayaka_gb300.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        obj = os.path.join(OBJDIR, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [sp] + headers):
            cmd = [nvcc] + NVCC_FLAGS + ["-I" + CSRC, "-I" + os.path.join(ROOT, "include"), "-c", sp, "-o", obj]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                sys.stdout.write(o)
    if force or _stale(LIB, objs):
        _run([nvcc, ARCH, "-shared", "-cudart", "static", "-o", LIB] + objs + ["-lpthread", "-ldl", "-lrt"])
    return LIB


def build_oracle(force=False):
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    src = os.path.join(ORACLE_DIR, "mac_oracle.c")
    if not os.path.exists(src):
        return None
    if force or _stale(ORACLE_LIB, [src]):
        cc = os.environ.get("CC", "gcc")
        # -ffp-contract=off: no FMA contraction on either host architecture
        _run([cc, "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", "-o", ORACLE_LIB, src, "-lm"])
    return ORACLE_LIB


def reference_src():
    """the reference's src/ directory: $REF when set (the variable
    oracle/Makefile takes), else the Makefile's own default"""
    ref = os.environ.get("REF")
    if ref:
        return ref
    with open(os.path.join(ORACLE_DIR, "Makefile")) as f:
        for line in f:
            if line.startswith("REF") and "?=" in line:
                return line.split("?=", 1)[1].strip()
    return None


def build_reference_oracle():
    """oracle/_ref from the reference sources (only where they are present)."""
    ref = reference_src()
    if not ref or not os.path.isdir(ref):
        return None
    _run(["make", "-C", ORACLE_DIR, "-j8", "-s", "REF=" + ref])
    return os.path.join(ORACLE_DIR, "_ref")


def main():
    force = "--force" in sys.argv
    print(build_library(force=force, verbose=True))
    print(build_oracle(force=force))


if __name__ == "__main__":
    main()
