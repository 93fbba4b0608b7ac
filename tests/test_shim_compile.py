"""The C++ drop-in class include/SayakaMacSolverGpu.h compiles against the
reference's own headers, in 2D and 3D, driving the whole MacSolver call
sequence of the reference's drivers (src/Test6.h:255-298).  Needs the
reference's sources (the REF variable of oracle/Makefile); skipped where they
are absent, e.g. on the GPU host."""
import os
import shutil
import subprocess

import pytest

from sayakaamr_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r'''
#include "SayakaMacSolverGpu.h"
using namespace sayaka;
int drive(const AmrTree &tree, TreeData &phi, TreeData &rhs, std::vector<TreeData *> &b, const BCRegister &reg,
          const TreeData &ls, TreeData &flux) {
  MacSolverGpu S(tree);
  S.prepareSolver();
  S.setIBFracByLS(ls, 0);
  S.setCoefB(b, 0);
  S.setBC(reg);
  S.fixBC(phi, rhs, 0, 0);
  S.setRhs(rhs, 0);
  S.setZeroSol();
  S.setTolerance(1e-8, 0.0);
  S.setMaxIteration(200);
  S.setPostSmoothNum(2);
  S.setCGUseMGPrecond(1);
  int st = S.cg_solve();
  S.getSol(phi, 0);
  S.mg_flux_level(tree.currentFinestLevel(), 0, flux, phi, 0, 0);
  S.setReferencePath(true);
  st += S.mg_solve() + S.relax_solve();
  return st + S.lastSolve().iterations;
}
'''


def ref_src():
    r = build.reference_src()
    return r if r and os.path.isdir(r) else None


@pytest.mark.parametrize("ndim", [2, 3])
def test_drop_in_class_compiles_against_reference_headers(ndim, tmp_path):
    ref = ref_src()
    if not ref:
        pytest.skip("reference sources not present")
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if not cxx:
        pytest.skip("no C++ compiler")
    src = tmp_path / "drive.cpp"
    src.write_text(DRIVER)
    # the reference's portability shims of oracle/Makefile (command line only)
    cmd = [cxx, "-std=c++14", "-c", "-o", str(tmp_path / "drive.o"), "-DNDEBUG", "-D_USE_MATH_DEFINES",
           "-D__declspec(x)=", "-include", "cstring", "-include", "tuple", "-include", "memory", "-include", "cmath",
           "-include", "functional", "-Dstricmp=strcasecmp", "-DSAYAKA_SPACEDIM=%d" % ndim, "-I" + ref,
           "-I" + os.path.join(ROOT, "include"), "-w", str(src)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-4000:]
