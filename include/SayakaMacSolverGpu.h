/*
 * SayakaMacSolverGpu.h -- drop-in for sayaka::MacSolver (src/SayakaMacSolver.h)
 * on a GB300, header-only C++ over the C ABI of sayaka_gb300.h.
 *
 * A reference driver replaces `MacSolver` by `MacSolverGpu` and keeps its
 * call sequence (src/Test6.h:255-298, src/Test7.h:612-637):
 *   MacSolverGpu S(tree); S.prepareSolver(); S.setIBFracByLS(ls, c);
 *   S.setCoefB(b, c); S.setBC(reg); S.fixBC(phi, rhs, pc, rc);
 *   S.setRhs(rhs, c); S.setZeroSol(); S.setTolerance(rel, abs);
 *   S.setCGUseMGPrecond(1); S.cg_solve(); S.getSol(phi, c);
 *   S.mg_flux_level(finest, dir, flux, phi, fc, pc);
 * Field buffers are the reference's own TreeData objects, passed through by
 * their base address (TreeData allocates every block in one chunk,
 * src/SayakaTreeData.cpp:105-121).  The tree stays host-owned: after a
 * regrid, make a new solver (as the reference's drivers do).
 *
 * prepareSolver() selects the device-resident solve (dense bottom solve,
 * FP32 V-cycle inside the FP64 outer BiCGSTAB, the whole iteration in a CUDA
 * graph) for the MG-preconditioned cg_solve.  setReferencePath(true) selects
 * the reference's own arithmetic and control flow instead (host-driven,
 * bottom BiCGSTAB to the bottom tolerances), e.g. to reproduce its iterates.
 *
 * Errors: a failing call throws std::runtime_error with the library's
 * message (the reference asserts or exits); the solvers return the
 * reference's int status (0 ok, 1 breakdown).
 *
 * Needs the reference's headers (SayakaTree.h, SayakaTreeData.h,
 * SayakaBoundaryPatch.h) on the include path, SAYAKA_SPACEDIM defined as for
 * the reference, and libsayaka_gb300.so at link time.
 */
#ifndef SAYAKA_MAC_SOLVER_GPU_H
#define SAYAKA_MAC_SOLVER_GPU_H

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "SayakaBoundaryPatch.h"
#include "SayakaTree.h"
#include "SayakaTreeData.h"
#include "sayaka_gb300.h"

namespace sayaka {

class MacSolverGpu {
 public:
  /* MacSolver(tree) + define (src/SayakaMacSolver.h:56-87) */
  explicit MacSolverGpu(const AmrTree &tree) : m_tree(&tree) {
    sayaka_params_default(&m_prm);
    upload();
  }
  ~MacSolverGpu() { sayaka_mac_destroy(m_h); }
  MacSolverGpu(const MacSolverGpu &) = delete;
  MacSolverGpu &operator=(const MacSolverGpu &) = delete;

  /* prepareSolver (src/SayakaMacSolver.cpp:12-26): the device-resident solve */
  void prepareSolver() {
    m_prm.bottom = m_reference ? 0 : 1;
    m_prm.precision = m_reference ? 0 : 1;
    m_prepared = true;
  }
  /* host-driven reference arithmetic (true) or the device-resident solve */
  void setReferencePath(bool on) {
    m_reference = on;
    if (m_prepared) prepareSolver();
  }

  /* setBC (src/SayakaMacOperator.cpp:1462-1469): the register resolved per
   * physical block face, as BlockBCRecord does (src/SayakaBoundaryPatch.h:126-175) */
  void setBC(const BCRegister &reg) {
    const int n = m_tree->numBlocks;
    std::vector<int32_t> bc((size_t)n * 6, -1);
    for (int b = 0; b < n; b++)
      for (int f = 0; f < 2 * NDIM; f++) {
        const int code = (*m_tree)[b].neighbor[f];
        if (code > NeighborType::PhysBndry) continue;
        const SurroundingIndex s = SurroundingIndex::FaceSurrounding(FaceIndex(f));
        bc[(size_t)b * 6 + f] = reg.getBCMap(s.ipos(), s.jpos(), s.kpos(), code);
      }
    check(sayaka_mac_set_bc(m_h, bc.data()));
  }
  /* setCoefB (src/SayakaMacCoef.cpp:36-76) */
  void setCoefB(const std::vector<TreeData *> &b, int comp) {
    for (int d = 0; d < NDIM; d++)
      check(sayaka_mac_set_coef_b(m_h, d, base(*b[d]), b[d]->numComp(), b[d]->numGrow(), comp));
  }
  /* setIBFracByLS (src/SayakaMacIB.cpp:34-154) */
  void setIBFracByLS(const TreeData &ls, int comp) {
    check(sayaka_mac_set_ib_frac_by_ls(m_h, base(ls), ls.numComp(), ls.numGrow(), comp));
  }
  /* fixBC (src/SayakaMacOperator.cpp:1470-1594) */
  void fixBC(const TreeData &phi, TreeData &rhs, int phicomp, int rhscomp) {
    check(sayaka_mac_fix_bc(m_h, base(phi), phi.numComp(), phi.numGrow(), phicomp, base(rhs), rhs.numComp(),
                            rhs.numGrow(), rhscomp));
  }
  /* setRhs / setInitSol / setZeroSol / getSol (src/SayakaMacSolver.h:117-132) */
  void setRhs(const TreeData &d, int c) { check(sayaka_mac_set_rhs(m_h, base(d), d.numComp(), d.numGrow(), c)); }
  void setInitSol(const TreeData &d, int c) {
    check(sayaka_mac_set_init_sol(m_h, base(d), d.numComp(), d.numGrow(), c));
  }
  void setZeroSol() { check(sayaka_mac_set_zero_sol(m_h)); }
  void getSol(TreeData &d, int c) { check(sayaka_mac_get_sol(m_h, base(d), d.numComp(), d.numGrow(), c)); }
  /* after AmrTree::regrid: the solution of the solver of the old tree as the
   * initial solution, carried as AmrTree::initNewBlockDataAfterRegrid carries
   * a cell state with centered-linear prolongation after an average-down
   * (src/SayakaRegrid.cpp:987-1105); bc_val[face position] are the BC values
   * of the pressure's register (null: 0).  Call setBC first. */
  void setInitSolFromRegrid(const MacSolverGpu &old, const double *bc_val = nullptr) {
    check(sayaka_mac_init_new_block_data(m_h, old.m_h, bc_val));
  }

  /* solver parameters (src/SayakaMacSolver.h:346-358) */
  void setTolerance(double rel, double abs) {
    m_prm.tol_rel = rel;
    m_prm.tol_abs = abs;
  }
  void setMaxIteration(int n) { m_prm.max_iter = n; }
  void setPostSmoothNum(int n) { m_prm.n_post_smooth = n; }
  void setCGUseMGPrecond(int on) { m_prm.use_mg_precond = on; }
  void setVerbose(int v) { m_prm.verbose = v; }
  /* the library's own parameters (precision, smoother, ...), see sayaka_params */
  sayaka_params &params() { return m_prm; }

  /* cg_solve (src/SayakaMacSolver.cpp:455-680) */
  int cg_solve() { return solve(sayaka_mac_cg_solve); }
  /* mg_solve (src/SayakaMacSolver.cpp:43-162), relax_solve (:377-452) */
  int mg_solve() { return solve(sayaka_mac_mg_solve); }
  int relax_solve() { return solve(sayaka_mac_relax_solve); }
  /* outcome of the last solve (iterations, residual norms, wall time) */
  const sayaka_solve_info &lastSolve() const { return m_info; }

  /* mg_flux_level (src/SayakaMacOperator.cpp:161-239) on the finest level */
  void mg_flux_level(int mg_level, int dir, TreeData &flux, const TreeData &phi, int fluxcomp, int phicomp) {
    if (mg_level != m_tree->currentFinestLevel()) throw std::runtime_error("mg_flux_level: finest level only");
    check(sayaka_mac_flux(m_h, dir, base(phi), phi.numComp(), phi.numGrow(), phicomp, base(flux), flux.numComp(),
                          flux.numGrow(), fluxcomp));
  }

  sayaka_mac *handle() { return m_h; }

 private:
  static double *base(const TreeData &d) {  // the start of the one-chunk buffer of every block
    const IndexBox &g = d.indexBox();
    return const_cast<double *>(&d[0](g.ilo(), g.jlo(), g.klo(), 0));
  }
  int solve(int (*fn)(sayaka_mac *, sayaka_solve_info *)) {
    if (!m_prepared) prepareSolver();
    check(sayaka_mac_set_params(m_h, &m_prm));
    const int st = fn(m_h, &m_info);
    if (st != SAYAKA_OK && st != SAYAKA_BREAKDOWN && st != SAYAKA_NOT_CONVERGED) check(st);
    return st == SAYAKA_BREAKDOWN ? 1 : 0;  // the reference's int status
  }
  void upload() {
    const AmrTree &t = *m_tree;
    const int n = t.numBlocks;
    m_lev.resize(n);
    m_nbr.resize((size_t)6 * n);
    m_chd.resize((size_t)8 * n);
    m_par.resize(n);
    m_wc.resize(n);
    m_nt.resize(n);
    m_len.resize((size_t)3 * n);
    for (int b = 0; b < n; b++) {
      const AmrTreeNode &x = t[b];
      m_lev[b] = x.refineLevel;
      m_par[b] = x.parent;
      m_wc[b] = x.whichChild;
      m_nt[b] = x.nodeType;
      for (int f = 0; f < 6; f++) m_nbr[(size_t)6 * b + f] = x.neighbor[f];
      for (int c = 0; c < 8; c++) m_chd[(size_t)8 * b + c] = x.child[c];
      for (int d = 0; d < 3; d++) m_len[(size_t)3 * b + d] = x.blockLength(d);
    }
    const sayaka_tree_tables tb{NDIM,        t.validBlockCellBox().size(0),
                                n,           t.minAmrLevel,
                                t.maxAmrLevel, m_lev.data(),
                                m_nbr.data(), m_chd.data(),
                                m_par.data(), m_wc.data(),
                                m_nt.data(),  m_len.data()};
    const int st = sayaka_mac_create(&tb, &m_h);
    if (st != SAYAKA_OK) throw std::runtime_error("sayaka_mac_create failed (status " + std::to_string(st) + ")");
  }
  void check(int st) {
    if (st != SAYAKA_OK) throw std::runtime_error(sayaka_mac_last_error(m_h));
  }

  const AmrTree *m_tree;
  sayaka_mac *m_h = nullptr;
  sayaka_params m_prm;
  sayaka_solve_info m_info{};
  bool m_reference = false, m_prepared = false;
  std::vector<int32_t> m_lev, m_nbr, m_chd, m_par, m_wc, m_nt;
  std::vector<double> m_len;
};

}  // namespace sayaka

#endif /* SAYAKA_MAC_SOLVER_GPU_H */
