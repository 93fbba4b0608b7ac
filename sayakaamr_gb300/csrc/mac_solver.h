// GPU MAC solver: owns the device block pools and runs the reference's
// MG-preconditioned BiCGSTAB (src/SayakaMacSolver.cpp:683-949) with the
// kernels of mac_kernels.cu.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "mac_device.h"
#include "mac_learned.h"

namespace sayaka_gb300 {

// the tree as plain tables (what the C ABI receives)
struct TreeTables {
  int ndim = 2, nb = 8, num_blocks = 0, min_level = 1, max_level = 1;
  std::vector<int> level, neighbor, child, parent, which_child, node_type;  // 1, 6, 8, 1, 1, 1 per block
  std::vector<double> block_len;                                            // 3 per block
};

struct SolverParams {
  int max_iter = 2000;      // outer BiCGSTAB (src/SayakaMacSolver.h:72)
  double tol_rel = 1e-6;    // (src/SayakaMacSolver.h:73)
  double tol_abs = 0.0;     // (src/SayakaMacSolver.h:74)
  int n_post = 2;           // post-smoothing sweeps (src/SayakaMacSolver.h:77)
  double bot_tol_rel = 1e-6, bot_tol_abs = 1e-6;  // (src/SayakaMacSolver.h:78-79)
  int bot_max_iter = 2000;                        // (src/SayakaMacSolver.h:80)
  int use_mg_precond = 0;   // setCGUseMGPrecond (src/SayakaMacSolver.h:358)
  int precision = 0;        // 0: FP64 V-cycle, 1: FP32 V-cycle (FP64 outer + bottom)
  int bottom = 0;           // 0: BiCGSTAB (reference), 1: dense direct solve
  int verbose = 0;
  int graph = 1;            // device path: 1 graph + WHILE node, 0 host loop of direct launches
  int vcycle_kernel = 0;    // device path: 0 one launch per phase, 1 one cooperative launch, 2 cluster phases
  int pdl = 0;              // device path: programmatic dependent launch between the iteration's kernels
  int cluster_cells = 16384;  // vcycle_kernel 2: phases touching at most this many cells run in the cluster
  int smooth_variant = -1;    // device smoother launch bounds: -1 autotune at prepare, else variant index
  int learned = 0;            // device path, FP32 V-cycle: apply the trained block correction
  int fuse_prolong = 1;       // device path: prolongation fused with the first red sweep of its level
  int vcycle_out = 0;         // FP32 V-cycle output to the BiCGSTAB kernels: 0 = read in place in 2D and on 3D
                              // towers up to 2M cells, else widened once into FP64 vectors; 1 = in place with the
                              // operator in double-float; 2 = always widened; 3 = always in place
  int prolong_form = 1;       // that fused launch: 1 = one warp per block (2D FP32 16x16 blocks), 0 = one CTA
                              // per block with a shared-memory tile (same values)
  int bottom_half = 0;        // device path, FP32 V-cycle: 1 = FP16 copy of the bottom inverse with row scales,
                              // 0 = FP32 copy
  int bottom_level = 0;       // device path: level of the dense bottom solve; 0 = the coarsest level whose
                              // tower is one uniform level of at most kBottomMaxCells cells per component
  int sublevel_order = 1;     // device V-cycle smoothing order over a tower's sublevels: 0 = finest to
                              // coarsest, red then black per sublevel (the reference's); 1 = one launch per
                              // colour and level parity (sublevels two levels apart never touch)
  int smoother = 0;           // device V-cycle smoother: 0 = red-black sweeps (n_post per tower, one launch
                              // per colour); 1 = block-hybrid passes (n_post per tower, each one launch of
                              // inner_sweeps red-black sweeps per block, Jacobi between blocks)
  int inner_sweeps = 2;       // smoother 1: red-black sweeps per block in one pass
  int learned_loss = 0;       // training loss of the learned correction: 0 = the block-local residual it
                              // leaves, 1 = its distance to the error the V-cycle left (block-local part)
  int learned_tc05 = 1;       // learned correction of 16x16 blocks: 1 = hidden layer on tcgen05 (tensor memory
                              // accumulator), 0 = on mma.sync (the same network; products summed in another order)
  int bottom_refresh = 1;     // device path: 1 = the dense bottom inverse is rebuilt after every coefficient
                              // change; 0 = kept from the last build until the tree or the bottom level changes
                              // (a fixed, slightly stale coarsest-level solve inside the preconditioner)
  int uniform = 1;            // device path: constant-coefficient blocks read their face coefficients from a
                              // per-block record (same results; 0 = every block reads the face arrays)
  int per_problem = 1;        // device path, a tree of several independent problems (connected components):
                              // 1 = one BiCGSTAB state per problem, each stopping at its own tolerance;
                              // 0 = one state shared by all
  double relax_omega = 1.0;   // device V-cycle smoothers: relaxation weight of every red-black update of a fluid
                              // cell, u = u_old + omega * (u_gs - u_old); 1 = plain Gauss-Seidel (default)
};

struct SolveInfo {
  int status = 0;        // 0 ok, 1 breakdown, 2 not converged
  int iterations = 0;
  double rnorm0 = 0, rnorm = 0;
  double seconds = 0;
};

class MacGpu {
 public:
  explicit MacGpu(const TreeTables &tt);
  ~MacGpu();
  MacGpu(const MacGpu &) = delete;
  MacGpu &operator=(const MacGpu &) = delete;

  const std::string &error() const { return err_; }
  int ndim() const { return tt_.ndim; }
  int nb() const { return tt_.nb; }
  int ncell() const { return ncell_; }
  int nfb() const { return nfb_; }
  int num_blocks() const { return tt_.num_blocks; }
  int finest() const { return finest_; }
  const std::vector<int> &tower_blocks(int L) const { return towers_[L].blocks; }

  // coefficients and fractions (all blocks, compact layouts).  Setters taking
  // leaf values perform the reference's c/f AVG sync and AVG restriction.
  void set_scalars(double alpha, double beta);
  void set_coef_b_leaf(int dir, const double *face_all);       // src/SayakaMacCoef.cpp:36-76
  void set_ib_frac_leaf(const double *vol_all, const double *const area_all[3]);  // src/SayakaMacIB.cpp:34-97
  void set_ib_frac_by_ls(const double *ls_grown, int ngrow, bool dev = false);  // binary fractions from a level set
  void set_bc_types(const int *bc6);                            // math BC per block face (-1 interior)
  void get_coef(int which, int dir, double *out_all);           // 0 B, 1 area frac, 2 vol frac

  // user vectors (compact, all blocks)
  void set_rhs(const double *all, bool on_device = false);
  void set_sol(const double *all, bool on_device = false);
  void zero_sol();
  void get_sol(double *all, bool on_device = false);
  // the same between the device and a TreeData-layout field (ncomp
  // components of ngrow ghost layers per block) that the GPU can address:
  // pinned host memory read and written by the kernel over the CPU-GPU link,
  // no staging copy (0 ok, else a CUDA error was recorded)
  int set_field_td(const double *td, int ncomp, int ngrow, int comp, bool rhs);
  int get_sol_td(double *td, int ncomp, int ngrow, int comp);
  double *rhs_dev() { return vec_[kRHS]; }
  double *sol_dev() { return vec_[kSOL]; }

  void set_params(const SolverParams &p) { prm_ = p; }
  const SolverParams &params() const { return prm_; }

  int cg_solve(SolveInfo *info);
  // mg_solve / relax_solve: stand-alone V-cycles / Gauss-Seidel sweeps on the
  // finest tower, reference arithmetic (0 ok, -1 CUDA error; info->status)
  int mg_solve(SolveInfo *info);
  int relax_solve(SolveInfo *info);
  // graph-captured device-resident solve (dense bottom); enqueue variant for
  // timing: no host synchronisation, the result stays on the device
  int cg_solve_device(SolveInfo *info);
  int cg_solve_enqueue();
  int prepare_device();
  int solve_state(SolveInfo *info);
  int enqueue_kernel(int which, int L);
  // the device solve's FP64 operator (which 0) or smoothing pass of tower L
  // (which 1) on given compact host arrays (0 ok, 1 bad input, 2 CUDA error)
  int device_kernel_compact(int which, int L, int variant, const double *in, const double *in2, double *out);
  int tower_size(int L, int sublevel) const;
  int tuned_smoother(int precision, float *us, int n) const;
  int bottom_level() const { return bottom_ready_ ? bot_level_ : -1; }
  // number of independent problems (connected components) of the tree
  int problems() const { return ncomp_; }
  // per-problem outcome of the last device solve (one state per problem):
  // iterations and final relative residual |r|/|r0|; returns the problem
  // count, or -1 when the last solve shared one state
  int problem_states(int *iterations, double *rel_resid, int n);
  int uniform_blocks();  // constant-coefficient blocks (after preparing the device solve)
  int device() const { return device_; }

  // building blocks, exposed for parity tests (compact arrays, all blocks)
  void apply(int L, const double *x_all, double *y_all);
  void residual(int L, const double *x_all, const double *rhs_all, double *r_all);
  void smooth(int L, const double *phi_all, const double *rhs_all, double *out_all);
  void restrict_sweep(const double *in_all, double *out_all);
  void prolong_sweep(const double *in_all, double *out_all);
  void vcycle(const double *p_all, double *phat_all);
  void flux(int dir, const double *phi_all, double *flux_all);
  void fix_bc(const double *phi_grown, int ngrow, double *rhs_all);

  // learned block correction (mac_learned.cu)
  bool learned_supported() const;
  int learned_collect(int max_iters, int max_samples = 0);  // max_samples 0: every block of every iterate
  float learned_train(int epochs, float lr, int batch, unsigned seed);
  float learned_eval();  // mean loss of the collected pairs under the current weights
  float learned_loss_grad(const float *feat, const float *aux, int n, float *grad);
  int aux_len() const { return 3 * tt_.nb * tt_.nb + 2 * (tt_.nb + 1) * tt_.nb; }
  int learned_forward(const float *feat, int n, float *y);
  int learned_set_weights(const float *w, int n);
  int learned_get_weights(float *w, int n);
  int learned_samples() const { return ls_.nsamp; }
  bool learned_ready() const { return ls_.trained; }

  // projection step around the solve (compact all-block face arrays, host)
  void rhs_from_div(const double *const *u_all, const double *const *w_all, double scale);
  void correct_vel(int dir, double dt, double *u_all);
  void get_rhs(double *all);
  // the solution of a solver on the tree before a regrid, carried onto this
  // tree (0 ok, 1 bad input: why says which, 2 CUDA error)
  int init_solution_from(const MacGpu &old, std::string *why);
  // the same as AmrTree::initNewBlockDataAfterRegrid with centered-linear
  // prolongation after an average-down of the old solution; bc_val: the BC
  // value of each face position (null = 0)
  int init_new_block_data(const MacGpu &old, const double *bc_val, std::string *why);

  // r = rhs - A x on tower L and out = {|r|_inf, r.r}; device pointers to
  // compact all-block arrays, enqueued on s, no device allocation (scratch in
  // a static device array).  0 ok, 1 bad input or size (why says which),
  // 2 CUDA error
  int residual_norm_noalloc(int L, const double *x, const double *rhs, double *r, double *out, cudaStream_t s,
                            std::string *why);

  cudaStream_t stream() const { return stream_; }

 private:
  enum Vec {
    kRHS, kSOL, kRESID, kCORR, kTMP,
    kX0, kX, kR, kRHAT, kP, kPHAT, kS, kSHAT, kV, kT,
    kBX0, kBX, kBR, kBRHAT, kBP, kBS, kBV, kBT,
    kNumVec
  };
  struct DevList {
    int *blocks = nullptr;
    uint16_t *ftypes = nullptr;
    int *hx = nullptr;     // halo descriptors (tower lists)
    int *links = nullptr;  // parents (level lists) or children (non-leaf lists)
    int n = 0;
  };
  struct DevTower {
    DevList all;
    std::vector<int> begin, end;
    std::vector<int> blocks;
    // the smoothed sublevels regrouped by level parity: [L, L-2, ... | L-1,
    // L-3, ...]; group 0 is [0, par_split), its first par_top entries are
    // the blocks of level L
    DevList par;
    int par_split = 0, par_top = 0;
  };

  BlockList tower_list(int L) const;
  BlockList sublevel_list(int L, int l) const;
  // parity group g of tower L (sublevel_order 1); skip_top leaves out the
  // level-L blocks of group 0
  BlockList parity_list(int L, int g, bool skip_top) const;
  BlockList level_list(int l) const;
  BlockList nonleaf_list(int l) const;

  void init_coefs();  // B = 1 and fractions 1 on every block, on the device
  void recompute_face_coef();
  // coefficient averaging on the device (mac_coef.cu)
  void build_coef_lists();
  void free_coef_lists();
  void coef_average(int dmask, double *const F[3], double *V);
  void coef_changed();
  void pull_coefs();
  // B, area and volume fractions of the listed blocks, compact in list order
  void pull_block_coefs(const std::vector<int> &blocks, std::vector<double> &vf, std::vector<double> (&bc)[3],
                        std::vector<double> (&af)[3]);
  std::vector<int *> d_sync_up_, d_sync_copy_;
  std::vector<int> n_sync_up_, n_sync_copy_;
  bool coef_lists_ = false;
  bool coef_uploaded_ = false;    // the initial coefficients are on the device
  // the bottom solve's arrays were allocated for this level, size and form
  int bot_built_level_ = -1, bot_built_half_ = -1;
  long long bot_built_tot_ = -1;
  bool host_coef_stale_ = false;  // bcoef_/afrac_/vf_ behind the device arrays
  double *d_ls_ = nullptr;        // level set staged for set_ib_frac_by_ls
  size_t ls_cap_ = 0;

  // vector ops over a block list (FP64)
  void vcopy(const BlockList &L, double *dst, const double *src);
  void vzero(const BlockList &L, double *dst);
  void vaxpby(const BlockList &L, double *out, double a, const double *x, double b, const double *y);
  double vdot(const BlockList &L, const double *a, const double *b);
  double vnorm(const BlockList &L, const double *a);

  void mg_apply(int L, double *out, const double *in, const double *rhs_for_residual);
  void mg_smooth(int L, double *phi, const double *rhs);
  void mg_restrict(int lc, double *phi);
  void mg_prolong(int lf, double *phi);
  void precond(int L, double *sol, const double *rhs);
  int bottom_solve();
  int bicgstab(int L, double *sol, const double *rhs, double tol_rel, double tol_abs, int max_iter, bool use_precond,
               bool bottom, SolveInfo *info);

  void fail(const std::string &m);

  // device-resident path (mac_fast.cu)
  void ensure_fast_buffers();
  void refresh_fp32();
  void build_op_factors();
  void build_smooth_factors();
  void ensure_smooth_factors();
  long sfac_version_ = -1;  // coefficient version of the FP64 smoother factors
  void tune_smoother(int precision);
  template <typename T>
  int rbgs_var() const {
    const int v = rbgs_variant_[sizeof(T) == 4 ? 1 : 0];
    return v < 0 ? 2 : v;
  }
  void build_bottom();
  template <typename T>
  void vcycle_device(int L, T *resid, T *corr, const Coef<T> &c, double *out);
  template <typename T>
  void iteration_device(T *resid, T *corr, const Coef<T> &c);
  template <typename T, typename TO>
  void iteration_body(T *resid, T *corr, const Coef<T> &c, const TO *PH, const TO *SH, double *out_p, double *out_s);
  void capture_loop(int precision);
  int enqueue_solve();
  void build_vcycle_program();
  template <typename T>
  void vcycle_coop(T *resid, T *corr, const Coef<T> &c, double *out);
  template <typename T>
  void vcycle_cluster(T *resid, T *corr, const Coef<T> &c, double *out);
  template <typename T>
  void bottom_launch(T *resid, T *corr);
  template <typename T>
  void precondition(int L, T *resid, T *corr, const Coef<T> &c, double *out);
  bool learned_active() const { return prm_.learned && prm_.precision == 1 && ls_.trained && learned_supported(); }
  template <typename T>
  void vc_out_launch(const BlockList &TL, T *corr, double *out);

  TreeTables tt_;
  SolverParams prm_;
  std::string err_;
  int ncell_ = 0, nfb_ = 0, finest_ = 0;
  cudaStream_t stream_ = nullptr;

  // host mirrors
  std::vector<double> geom_;           // [nblocks*8]
  std::vector<double> bcoef_[3], afrac_[3], vf_;
  std::vector<int> bc_type_;           // [nblocks*6]
  std::vector<int> fc_neigh_;          // [nblocks*6]
  double alpha_ = 0.0, beta_ = 1.0;

  // device tables
  int *d_neighbor_ = nullptr, *d_child_ = nullptr, *d_parent_ = nullptr, *d_wc_ = nullptr;
  int *d_fc_neigh_ = nullptr, *d_bc_type_ = nullptr;
  int *d_err_ = nullptr;  // error word of the bounded waits (Topo::err)
  double *d_geom_ = nullptr;
  double *d_bcoef_[3] = {nullptr, nullptr, nullptr}, *d_afrac_[3] = {nullptr, nullptr, nullptr};
  double *d_tff_[3] = {nullptr, nullptr, nullptr}, *d_vf_ = nullptr;
  double *vec_[kNumVec] = {};
  double *d_red_ = nullptr;        // reduction partials
  unsigned *d_counter_ = nullptr;  // last-block counter
  double *h_red_ = nullptr;        // pinned scalar readback

  std::vector<DevTower> towers_;
  std::vector<DevList> levels_, nonleaf_;
  std::vector<std::vector<int>> level_blocks_, nonleaf_blocks_;

  Topo topo_{};
  Coef<double> c64_{};

  // device-resident path
  bool fast_ready_ = false, bottom_ready_ = false;
  long coef_version_ = 1, fast_coef_version_ = 0;
  float *d_tff32_[3] = {}, *d_bcoef32_[3] = {}, *d_afrac32_[3] = {}, *d_vf32_ = nullptr, *d_geom32_ = nullptr;
  float *d_resid32_ = nullptr, *d_corr32_ = nullptr;
  // second correction vector of the block-hybrid smoother's passes (they
  // read one and write the other)
  float *d_corr32b_ = nullptr;
  double *d_corr64b_ = nullptr;
  template <typename T>
  T *corr_alt() {
    if constexpr (sizeof(T) == 4)
      return d_corr32b_;
    else
      return d_corr64b_;
  }
  // tower L with its FP64 smoother factors, every sublevel (block-hybrid passes)
  BlockList smooth_list(int L) const;
  // independent problems of a forest (connected components of the tree)
  // with one BiCGSTAB state each (prm_.per_problem): the finest tower listed
  // problem by problem, its chunks, the states and the reduction scratch
  int ncomp_ = 1;
  std::vector<int> comp_of_block_;
  int *d_comp_ = nullptr;
  DevList tlc_;
  int *d_chunk_ = nullptr;  // [comp | beg | end] per chunk, then [first chunk | chunks] per problem
  int nchunks_ = 0;
  FState *d_stc_ = nullptr, *h_stc_ = nullptr;
  double *d_cpart_ = nullptr;
  unsigned *d_ccnt_ = nullptr;
  bool solve_lists_ = false;  // block lists carry the states (set while a solve is recorded)
  bool multi() const { return ncomp_ > 1 && prm_.per_problem != 0 && d_stc_ != nullptr; }
  BlockList attach(BlockList r) const;
  Coef<float> c32_{};
  FState *d_st_ = nullptr, *h_st_ = nullptr;
  double *d_part_ = nullptr;
  double *d_opP_ = nullptr, *d_opS_ = nullptr;  // factors of the device solve's operator
  // their nearest double-float pairs, and those of the block records
  float2 *d_opP2_ = nullptr, *d_opS2_ = nullptr, *d_uni2_ = nullptr;
  // constant-coefficient block records (Coef::ut) and the FP64 coefficients
  // the device solve's kernels read (c64_ with the records when enabled)
  double *d_uni64_ = nullptr;
  float *d_uni32_ = nullptr;
  Coef<double> cd64_{};
  void build_uniform();
  void bind_uniform();
  std::vector<double *> d_sfac_;                // FP64 smoother factors per tower: sa then ia
  std::vector<double *> d_pfac_;                // the same for the parity-grouped tower lists
  std::vector<double *> d_face_;                // face fields of the projection step (u, w, flux)
  LearnedState ls_;
  std::vector<double *> *record_ = nullptr;     // iterates recorded by a collection solve
  void learned_init(unsigned seed);
  void learned_sync_bf16();
  void learned_reserve(int more);
  void learned_free();
  void learned_vcycle(float *r, float *z);
  void learned_apply(float *resid, float *corr);
  void learned_prepare();
  float learned_grad(const int *d_idx, int nblk, float inv_norm, float *h1, float *h2, float *dy);
  double *face_scratch(int k);
  unsigned *d_cnt_ = nullptr;
  double *d_binv_ = nullptr;
  int *d_bot_blocks_ = nullptr, *d_comp_row0_ = nullptr, *d_comp_n_ = nullptr, *d_tile_comp_ = nullptr,
      *d_tile_row0_ = nullptr;
  long long *d_comp_off_ = nullptr;
  BottomDev bot_{};
  float *d_binv32_ = nullptr, *d_rscale_ = nullptr;
  unsigned short *d_binv16_ = nullptr;
  int bot_level_ = 1, bot_param_ = -1, bot_half_ = -1, program_bot_ = -1;
  int device_ = 0;
  int choose_bottom_level(std::string *why) const;
  int n_bot_ = 0, n_pins_ = 0, n_bot_comp_ = 0;
  void bottom_free();
  void drop_graph();
  cudaGraph_t graph_ = nullptr;
  cudaGraphExec_t graph_exec_ = nullptr;
  int graph_prec_ = -1, graph_npost_ = -1;
  int kernels_per_iter_ = 0;
  int graph_coop_ = -1, graph_pdl_ = -1, graph_cc_ = -1, graph_var_ = -1, graph_nn_ = -1, graph_order_ = -1;
  int graph_smoother_ = -1, graph_inner_ = -1, graph_multi_ = -1, graph_uniform_ = -1, graph_pform_ = -1,
      graph_vout_ = -1;
  double graph_omega_ = -1.0;
  bool last_multi_ = false;  // the last device solve kept one state per problem
  Chunks chunks() const;
  bool graph_stale() const;
  int rbgs_variant_[2] = {-1, -1};  // tuned smoother variant per precision (0 FP64, 1 FP32)
  float rbgs_us_[2][16] = {};       // measured microseconds per variant (kRbgsVariants <= 16)
  // cooperative V-cycle
  VPhase *d_phases_ = nullptr;
  std::vector<VPhase> h_phases_;
  int n_phases_ = 0, program_npost_ = -1, program_order_ = -1, coop_grid_ = 0;
  unsigned *d_bar_ = nullptr;  // [0] count, [1] generation, [2] error word
  // cluster V-cycle: restriction program, bottom, prolongation/smoothing program
  int n_down_ = 0, cluster_size_ = 0;

 public:
  // kernel launches of one captured BiCGSTAB iteration; a device solve
  // launches kPrologueKernels + iterations * this + kEpilogueKernels
  int kernels_per_iteration() const { return kernels_per_iter_; }
  static constexpr int kPrologueKernels = 3, kEpilogueKernels = 1;
};

// integer-pipe precision conversions of the vector kernels against the
// hardware conversions, on the current device (0 ok, 2 CUDA error)
int fp_selftest(const double *d, const float *f, int n, float *nar, float *nar_hw, double *wid, double *wid_hw,
                double *wid0, double *wid0_hw);

}  // namespace sayaka_gb300
