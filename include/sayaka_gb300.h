/*
 * sayaka_gb300 -- C ABI of the GB300 MAC pressure-Poisson solver.
 *
 * Drop-in boundary for the MAC solver path of the SayakaAmr library
 * (haloless/SayakaAmr): the class sayaka::MacSolver (src/SayakaMacSolver.h)
 * operating on an AmrTree (src/SayakaTree.h) and TreeData fields
 * (src/SayakaTreeData.h).  Plain pointers and sizes only.
 *
 * Host field buffers use the reference's TreeData layout: block b, component
 * c, cell (i,j,k) of the grown box at
 *     b*cap*ncomp + c*cap + (i+g) + (j+g)*Gx + (k+g)*Gx*Gy
 * with g = ngrow, Gx = nb+2g (+1 for x-face data), Gy likewise, cap = the
 * grown box size (in 2D the third extent is 1 and carries no ghost layer).
 * "compact" entry points take [block][k][j][i] valid cells (face data:
 * [block][...][face index], the staggered valid box) for every tree block.
 *
 * Every entry point returns a sayaka_status; a non-OK status leaves a message
 * for sayaka_mac_last_error().  Nothing here exits the process.
 */
#ifndef SAYAKA_GB300_H
#define SAYAKA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum sayaka_status {
  SAYAKA_OK = 0,
  SAYAKA_BREAKDOWN = 1,      /* BiCGSTAB breakdown: rho, r^.v or t.t == 0 (src/SayakaMacSolver.cpp:773-900) */
  SAYAKA_NOT_CONVERGED = 2,  /* max_iter reached (the reference prints "failure", :915-917) */
  SAYAKA_STALL_FALLBACK = 3, /* learned preconditioner stalled; finished with plain MG */
  SAYAKA_BAD_INPUT = 4,
  SAYAKA_CUDA_ERROR = 5
} sayaka_status;

/* ------------------------------------------------------------------------
 * Tree tables: the AmrTree block arrays the solver reads
 * (AmrTreeNode, src/SayakaTree.h:52-152).  Neighbour codes: >= 0 block id at
 * the same level, -1 coarser neighbour, <= -20 physical boundary code.
 * ---------------------------------------------------------------------- */
typedef struct sayaka_tree_tables {
  int32_t ndim;       /* 2 or 3 (SAYAKA_SPACEDIM, src/SayakaCommons.h:4-12) */
  int32_t nb;         /* cells per block edge, even (blockValidIndex) */
  int32_t num_blocks; /* AmrTree::numBlocks */
  int32_t min_level;  /* AmrTree::minAmrLevel */
  int32_t max_level;  /* AmrTree::maxAmrLevel */
  const int32_t *level;       /* [num_blocks]   refineLevel */
  const int32_t *neighbor;    /* [num_blocks*6] neighbor[MAX_FACE] */
  const int32_t *child;       /* [num_blocks*8] child[MAX_CHILD] */
  const int32_t *parent;      /* [num_blocks] */
  const int32_t *which_child; /* [num_blocks] */
  const int32_t *node_type;   /* [num_blocks]   TreeNodeType (src/SayakaTree.h:27-32) */
  const double *block_len;    /* [num_blocks*3] blockLength */
} sayaka_tree_tables;

/* ------------------------------------------------------------------------
 * Host tree mirror: AmrTree / regrid (src/SayakaTree.cpp, src/SayakaRegrid.cpp)
 * ---------------------------------------------------------------------- */
typedef struct sayaka_tree sayaka_tree;

/* AmrTree::init with an explicit block capacity (src/SayakaTree.cpp:34-91) */
int sayaka_tree_create(int32_t ndim, int32_t nb, int32_t min_level, int32_t max_level, int32_t capacity,
                       sayaka_tree **out);
void sayaka_tree_destroy(sayaka_tree *t);
/* AmrTree::initUniformRootLevel (src/SayakaTree.cpp:93-201) */
int sayaka_tree_init_uniform_root(sayaka_tree *t, const int32_t ndiv[3], const double lo[3], const double hi[3],
                                  const int32_t bc_type[6], const int32_t periodic[6]);
/* AmrTree::initRefineToMinLevel (src/SayakaTree.cpp:204-233) */
int sayaka_tree_init_refine_to_min_level(sayaka_tree *t);
/* AmrTree::refineFlag / coarsenFlag (src/SayakaTree.h:221-222), n <= capacity */
int sayaka_tree_set_refine_flags(sayaka_tree *t, const int32_t *flags, int32_t n);
int sayaka_tree_set_coarsen_flags(sayaka_tree *t, const int32_t *flags, int32_t n);
/* AmrTree::regrid (src/SayakaRegrid.cpp:26-125) */
int sayaka_tree_regrid(sayaka_tree *t);
int32_t sayaka_tree_num_blocks(const sayaka_tree *t);
/* tables of the current tree; pointers stay valid until the next regrid */
int sayaka_tree_get_tables(sayaka_tree *t, sayaka_tree_tables *out);
/* boundBox lo/hi, blockCenter [num_blocks*3] each; nodeType2 [num_blocks*6] */
int sayaka_tree_get_geometry(const sayaka_tree *t, double *lo, double *hi, double *center);
int sayaka_tree_get_node_type2(const sayaka_tree *t, int32_t *out);
/* SurroundingBlocks blocks/types/bcrefs [num_blocks*27], position
 * (ii,jj,kk) in {-1,0,1}^3 at (ii+1) + 3(jj+1) + 9(kk+1) (src/SayakaTree.h:336-526) */
int sayaka_tree_get_surrounding(const sayaka_tree *t, int32_t *blocks, int32_t *types, int32_t *bcrefs);
/* MGLevelTower block list and [begin,end) per sublevel 1..L
 * (src/SayakaTower.cpp:28-187); sizes: blocks >= num_blocks, begin_end >= 2L */
int sayaka_tree_get_tower(const sayaka_tree *t, int32_t L, int32_t *blocks, int32_t *n, int32_t *begin_end);
/* BlockFaceRegister of every tower block, per face:
 * type, neigh, fine_crse_offset[3], crse_fine_neigh[4]  (9 ints) */
int sayaka_tree_get_face_regs(const sayaka_tree *t, int32_t L, int32_t *regs);

/* ------------------------------------------------------------------------
 * MAC solver (sayaka::MacSolver, src/SayakaMacSolver.h:25-425)
 * ---------------------------------------------------------------------- */
typedef struct sayaka_mac sayaka_mac;

typedef struct sayaka_params {
  int32_t max_iter;       /* setMaxIteration (src/SayakaMacSolver.h:349), default 2000 */
  double tol_rel;         /* setTolerance (:350), default 1e-6 */
  double tol_abs;         /* default 0 */
  int32_t n_post_smooth;  /* setPostSmoothNum (:353), default 2 */
  int32_t use_mg_precond; /* setCGUseMGPrecond (:358), default 0 */
  double bot_tol_rel;     /* bottom BiCGSTAB, default 1e-6 (:78-80) */
  double bot_tol_abs;     /* default 1e-6 */
  int32_t bot_max_iter;   /* default 2000 */
  int32_t precision;      /* 0: FP64 V-cycle; 1: FP32 V-cycle inside the FP64 outer solve */
  int32_t bottom;         /* 0: BiCGSTAB bottom (reference); 1: dense direct bottom solve */
  int32_t verbose;
  int32_t graph;          /* device path: 1 = CUDA graph with a WHILE node (default), 0 = the same
                             kernels launched from a host loop (for per-kernel profilers) */
  int32_t vcycle_kernel;  /* device path: 0 = one launch per restriction / smoother / prolongation phase,
                             1 = the whole V-cycle as one cooperative launch,
                             2 = restriction and smoothing phases inside one thread-block cluster */
  int32_t pdl;            /* device path: 1 = programmatic dependent launch between kernels (default 0) */
  int32_t cluster_cells;  /* vcycle_kernel 2: runs of consecutive phases that each touch at most this many
                             cells share one cluster launch; larger phases get their own launch (16384) */
  int32_t smooth_variant; /* device smoother launch bounds (register cap): -1 = autotuned at prepare by
                             timing every variant on the finest level (default), 0..9 = fixed */
  int32_t learned;        /* device path with the FP32 V-cycle: 1 = add the trained learned block
                             correction after every V-cycle (default 0); see sayaka_mac_learned_* */
  int32_t bottom_level;   /* device path: level of the dense bottom solve; 0 = auto (the finest level below the
                             finest whose tower is one uniform level with at most 1024 (2D) / 4096 (3D) cells
                             per connected component; level 1 otherwise), n >= 1 = level n if its tower is
                             one uniform level of at most 4096 cells per component */
  int32_t bottom_half;    /* device path, FP32 V-cycle: 1 = apply an FP16 copy of the dense bottom inverse
                             with one FP32 scale per row (half the bytes), 0 = an FP32 copy */
  int32_t sublevel_order; /* device V-cycle smoothing over a tower's sublevels: 0 = finest to coarsest,
                             red then black per sublevel (the reference's order, mg_smooth_level);
                             1 = one launch per colour and level parity (default) */
  int32_t smoother;       /* device V-cycle smoother (per-phase V-cycle): 0 = red-black sweeps, one launch per
                             colour (default); 1 = block-hybrid passes: n_post_smooth passes per tower, each
                             one launch of inner_sweeps red-black sweeps of every block from shared memory with
                             the values outside the block frozen (Gauss-Seidel inside a block, Jacobi between
                             blocks; a fixed linear map, another preconditioner with the same solution) */
  int32_t inner_sweeps;   /* smoother 1: red-black sweeps per block and pass (default 2) */
  int32_t per_problem;    /* device path, a tree made of several independent problems (connected components,
                             e.g. a forest of trees given as one table): 1 = one BiCGSTAB state per problem,
                             each stopping at its own tolerance, as if solved alone (default); 0 = one shared
                             state (scalars over all problems) */
  int32_t uniform;        /* device path: 1 = blocks whose face coefficients are constant per direction and
                             whose cells are all fluid (vf = 1) read the coefficients from a per-block record
                             instead of the face arrays and vf (same arithmetic, same results; default);
                             0 = every block reads the arrays */
  int32_t bottom_refresh; /* device path: 1 = the dense bottom inverse is rebuilt after every coefficient change
                             (default); 0 = the inverse of the last build is kept while only coefficients change
                             (a fixed coarsest-level solve of the preconditioner, slightly stale; the outer
                             BiCGSTAB still converges to the new operator's solution) */
  int32_t learned_tc05;   /* learned correction of 16x16-cell blocks: 1 = its 32 -> 32 layer as an implicit GEMM
                             on tcgen05 with the accumulator in tensor memory (default); 0 = on mma.sync warp
                             MMAs (the same network, products summed in another order) */
  int32_t vcycle_out;     /* how the BiCGSTAB kernels read the FP32 V-cycle's output: 0 = in place (widened
                             exactly on the integer pipe where they read it) in 2D and on 3D towers of at most
                             2,097,152 cells, widened once into FP64 vectors on larger 3D towers (default); 1 =
                             in place, the operator evaluated in double-float on the FP32 pipe; 2 = always
                             widened; 3 = always in place */
  int32_t prolong_form;   /* device V-cycle, the prolongation fused with the first red sweep of its level:
                             1 = one warp per block with the block in registers (2D FP32 16x16 blocks,
                             default; elsewhere form 0), 0 = one CTA per block with a shared-memory tile; the
                             same values */
  int32_t learned_loss;   /* training loss of the learned correction u: 0 = the residual u leaves under the
                             block-local operator (default); 1 = the distance of u to the block-local part of the
                             error the V-cycle left, known from the solver's own converged solution */
  double relax_omega;     /* device V-cycle: relaxation weight of every red-black update of a fluid cell,
                             u = u_old + omega * (u_gs - u_old), in (0, 2); 1 = Gauss-Seidel, the reference's
                             smoother (default).  Over-relaxation (about 1.1) is another fixed linear
                             preconditioner with the same solution; the reference-order host path
                             (bottom 0) ignores it */
} sayaka_params;

typedef struct sayaka_solve_info {
  int32_t status;     /* sayaka_status of the solve */
  int32_t iterations; /* outer BiCGSTAB iterations */
  double rnorm0;      /* |r0|_inf */
  double rnorm;       /* final |r|_inf (reference criterion, src/SayakaMacSolver.cpp:891) */
  double seconds;     /* wall time of the solve */
} sayaka_solve_info;

void sayaka_params_default(sayaka_params *p);

/* MacSolver(tree) + define + prepareSolver (src/SayakaMacSolver.h:56-87,
 * src/SayakaMacOperator.cpp:13-60, src/SayakaMacSolver.cpp:12-26):
 * alpha=0, beta=1, B=1, unit IB fractions */
int sayaka_mac_create(const sayaka_tree_tables *tables, sayaka_mac **out);
/* ~MacSolver (src/SayakaMacSolver.h:89-112) */
void sayaka_mac_destroy(sayaka_mac *h);
const char *sayaka_mac_last_error(const sayaka_mac *h);

/* setScalars (src/SayakaMacSolver.h:346) */
int sayaka_mac_set_scalars(sayaka_mac *h, double alpha, double beta);
/* setCoefB(dir, TreeData, comp): leaf copy, c/f AVG sync, AVG restriction
 * (src/SayakaMacCoef.cpp:36-76); face data of direction dir */
int sayaka_mac_set_coef_b(sayaka_mac *h, int32_t dir, const double *face, int32_t ncomp, int32_t ngrow,
                          int32_t comp);
/* setIBFracByLS (src/SayakaMacIB.cpp:34-154): binary fractions, ls <= 0
 * solid; ls cell data with ngrow >= 1 */
int sayaka_mac_set_ib_frac_by_ls(sayaka_mac *h, const double *ls, int32_t ncomp, int32_t ngrow, int32_t comp);
/* the same from one component given as the grown boxes of every block back
 * to back ((nb + 2 ngrow)^ndim values per block, i fastest); `on_device` != 0:
 * the pointer is device memory (a level set computed on the GPU is used
 * where it lies, no host round trip) */
int sayaka_mac_set_ib_frac_by_ls_compact(sayaka_mac *h, const double *ls, int32_t ngrow, int32_t on_device);
/* fractional IB fractions on leaf blocks (the protected m_ib_volfrac /
 * m_ib_areafrac of src/SayakaMacSolver.h:383-384), then the same c/f AVG sync
 * and AVG restriction; compact arrays, area[d] for d < ndim */
int sayaka_mac_set_ib_frac_compact(sayaka_mac *h, const double *vol, const double *area0, const double *area1,
                                   const double *area2);
/* setBC(BCRegister) resolved to BlockBCRecord (src/SayakaMacOperator.cpp:1462-1469,
 * src/SayakaBoundaryPatch.h:126-175): math BC per block face,
 * [num_blocks*6], 0 Neumann, 1 Dirichlet, 2 SimpleFill (physical faces) */
int sayaka_mac_set_bc(sayaka_mac *h, const int32_t *bc_type);
/* fixBC (src/SayakaMacOperator.cpp:1470-1594): BC values in phi's ghost
 * layer (ngrow >= 1) lifted into rhs on leaf blocks */
int sayaka_mac_fix_bc(sayaka_mac *h, const double *phi, int32_t phi_ncomp, int32_t phi_ngrow, int32_t phi_comp,
                      double *rhs, int32_t rhs_ncomp, int32_t rhs_ngrow, int32_t rhs_comp);

/* setRhs / setInitSol / setZeroSol / getSol (src/SayakaMacSolver.h:117-132) */
int sayaka_mac_set_rhs(sayaka_mac *h, const double *data, int32_t ncomp, int32_t ngrow, int32_t comp);
int sayaka_mac_set_init_sol(sayaka_mac *h, const double *data, int32_t ncomp, int32_t ngrow, int32_t comp);
int sayaka_mac_set_zero_sol(sayaka_mac *h);
int sayaka_mac_get_sol(sayaka_mac *h, double *data, int32_t ncomp, int32_t ngrow, int32_t comp);
/* compact variants; `on_device` != 0: the pointer is device memory */
int sayaka_mac_set_rhs_compact(sayaka_mac *h, const double *cells, int32_t on_device);
int sayaka_mac_get_sol_compact(sayaka_mac *h, double *cells, int32_t on_device);

/* setTolerance / setMaxIteration / setPostSmoothNum / setCGUseMGPrecond */
int sayaka_mac_set_params(sayaka_mac *h, const sayaka_params *p);
/* cg_solve (src/SayakaMacSolver.cpp:455-680): BiCGSTAB on the finest tower */
int sayaka_mac_cg_solve(sayaka_mac *h, sayaka_solve_info *info);
/* mg_solve (src/SayakaMacSolver.cpp:43-162): stand-alone V-cycles on the
 * finest tower (reference arithmetic, bottom BiCGSTAB with bot_tol_*), SOL
 * updated in place from its current value, until |r|_inf < |r0|_inf tol_rel +
 * tol_abs or max_iter; SAYAKA_NOT_CONVERGED when the tolerance is not met,
 * SAYAKA_BREAKDOWN when the bottom solve breaks down (the reference exits).
 * The reference runs its preconditioner's fixed V-cycle count instead of
 * max_iter after a preconditioned cg_solve; this one always follows max_iter. */
int sayaka_mac_mg_solve(sayaka_mac *h, sayaka_solve_info *info);
/* relax_solve (src/SayakaMacSolver.cpp:377-452): red-black Gauss-Seidel
 * sweeps of the finest tower (mg_smooth_level) on SOL, same stopping test */
int sayaka_mac_relax_solve(sayaka_mac *h, sayaka_solve_info *info);

/* Device-resident solve path (params.bottom = 1, use_mg_precond = 1):
 * build the FP32 coefficient copies, the dense level-1 inverse and the CUDA
 * graph of one BiCGSTAB iteration ahead of time ... */
int sayaka_mac_prepare(sayaka_mac *h);
/* ... enqueue a whole cg_solve on the solver's stream without waiting ... */
int sayaka_mac_cg_solve_async(sayaka_mac *h);
/* ... and read its outcome (waits for the stream) */
int sayaka_mac_solve_info(sayaka_mac *h, sayaka_solve_info *info);
/* the CUDA stream (cudaStream_t) every launch of this handle goes to */
void *sayaka_mac_stream(sayaka_mac *h);
/* enqueue one launch of a hot kernel on the solver's current data, for
 * per-kernel timing: which = 0 FP64 operator on tower L (x = solution),
 * 1 FP32 red-black sweep (colour 0) of the finest level of tower L,
 * 2 FP64 red-black sweep (colour 0) of the finest level of tower L,
 * 3 the device solve's FP64 operator with its dot product (L = finest) */
int sayaka_mac_enqueue_kernel(sayaka_mac *h, int32_t which, int32_t L);
/* kernel launches of a device-resident solve: prologue + per iteration +
 * epilogue (out pointers may be NULL) */
int sayaka_mac_launch_counts(sayaka_mac *h, int32_t *prologue, int32_t *per_iteration, int32_t *epilogue);
/* the launch-bounds variant of the device smoother that the autotuner chose
 * for precision (0 FP64, 1 FP32 V-cycle) at sayaka_mac_prepare, -1 if not
 * tuned yet; us (may be NULL) receives the measured microseconds per variant
 * (n entries, 13 variants: 0-4 one thread per cell with register caps
 * 128/80/64/40/32, 5-7 the block staged in shared memory, caps 128/64/40,
 * 8 the block's tile and face coefficients staged by TMA bulk copies,
 * 9 persistent CTAs streaming blocks through double-buffered bulk copies,
 * 10 two cells per thread (the same cell of two blocks, operands of both
 * gathered before either is updated), cap 64, 11-12 one warp per 16x16
 * block of a 2D FP32 sweep with the block in registers: 16-byte loads and
 * stores, neighbours by shuffles, caps 64/48, 13 the same with every load of
 * a block issued before its first branch, cap 64 (elsewhere 11-13 are the
 * same as 3)) */
int32_t sayaka_mac_tuned_smoother(sayaka_mac *h, int32_t precision, float *us, int32_t n);
/* number of smoother launch variants the autotuner times */
int32_t sayaka_smoother_variants(void);
/* level of the device solve's dense bottom solve once prepared (-1 before) */
int32_t sayaka_mac_bottom_level(const sayaka_mac *h);
/* number of independent problems (connected components) of the handle's
 * tree; with per_problem = 1 the last device solve's per-problem outcome:
 * iterations[k] and the final relative residual rel_resid[k] = |r|/|r0| of
 * problem k (problems numbered by their lowest block id; arrays of n >= the
 * count, either may be NULL).  Returns the count, or -1 after a solve with
 * one shared state.  No counterpart in the reference (it solves one tree). */
int32_t sayaka_mac_problem_count(const sayaka_mac *h);
int32_t sayaka_mac_problem_states(sayaka_mac *h, int32_t *iterations, double *rel_resid, int32_t n);
/* number of constant-coefficient blocks of the tree (face coefficients
 * constant per direction, every cell fluid), whose records the device solve
 * reads with params.uniform = 1; prepares the device solve first.  -1 on
 * error.  No counterpart in the reference (a property of this layout). */
int32_t sayaka_mac_uniform_blocks(sayaka_mac *h);
/* number of blocks in tower L, or at one level of it (sublevel >= 1) */
int32_t sayaka_mac_tower_size(sayaka_mac *h, int32_t L, int32_t sublevel);

/* mg_flux_level (src/SayakaMacOperator.cpp:161-239): face flux -d(phi)/dh of
 * direction dir on the leaf blocks; phi in TreeData layout (ngrow any) */
int sayaka_mac_flux(sayaka_mac *h, int32_t dir, const double *phi, int32_t phi_ncomp, int32_t phi_ngrow,
                    int32_t phi_comp, double *flux, int32_t flux_ncomp, int32_t flux_ngrow, int32_t flux_comp);

/* ---- learned block correction (no counterpart in the reference) ----
 * A per-block convolutional network (3x3 convolutions 3 -> 32 -> 32 -> 1,
 * ReLU; inputs: the block's residual after the V-cycle scaled by its max,
 * log10 of the face-averaged B, the volume fraction) predicts the V-cycle's
 * remaining error as a multiple of the Jacobi correction; the device solve
 * with the FP32 V-cycle adds it after every V-cycle when params.learned = 1,
 * and switches it off (status SAYAKA_STALL_FALLBACK on convergence) when the
 * residual stops improving.  Training minimises the residual the correction
 * leaves under the block's own operator.  2D trees with 8x8 or 16x16 blocks. */
int32_t sayaka_mac_learned_nparam(void);
/* training pairs from one plain device solve of the current right-hand side
 * (zero initial guess, tolerance 1e-12, at most max_iter iterations): one
 * pair per iterate and finest-tower block; the solution is reset to zero */
int sayaka_mac_learned_collect(sayaka_mac *h, int32_t max_iter, int32_t *iterates);
/* the same with at most max_samples pairs (every k-th block of each iterate,
 * the offset moving between iterates; 0 = no limit), for large forests */
int sayaka_mac_learned_collect_sampled(sayaka_mac *h, int32_t max_iter, int32_t max_samples, int32_t *iterates);
/* Adam on the collected pairs, FP32 forward/backward kernels on the GPU;
 * loss = mean over blocks of the weighted squared error (last epoch) */
int sayaka_mac_learned_train(sayaka_mac *h, int32_t epochs, float lr, int32_t batch, uint32_t seed, float *loss);
/* the same loss, mean over blocks, of the collected pairs under the current
 * weights, without training (held-out evaluation: collect the pairs of
 * another right-hand side first) */
int sayaka_mac_learned_eval(sayaka_mac *h, float *loss);
int sayaka_mac_learned_get_weights(sayaka_mac *h, float *w, int32_t n);
int sayaka_mac_learned_set_weights(sayaka_mac *h, const float *w, int32_t n);
/* test hooks: loss and weight gradient of explicit blocks (feat [n][3][nb*nb];
 * aux [n][3*nb*nb + 2*(nb+1)*nb] = Jacobi factor, dv*vf, x-face and y-face
 * coefficients of the block-local operator, error target), and the
 * tensor-core (BF16)
 * forward of explicit feature blocks (y [n][nb*nb]) */
int sayaka_mac_learned_loss_grad(sayaka_mac *h, const float *feat, const float *aux, int32_t n, float *grad,
                                 float *loss);
int sayaka_mac_learned_forward(sayaka_mac *h, const float *feat, int32_t n, float *y);

/* ---- projection step around the solve ---- */
/* The solve's right-hand side from a face velocity, on the device, then
 * setRhs: rhs = sum_d (scale/dh_d) * (u_d(i+1) - u_d(i)) on every block,
 * accumulated from d = 0 (calc_pres_rhs_block, src/Test7.h:587-609, with
 * scale = -1/dt; calc_block_rhs_value, src/Test6.h:798-830, with scale = 1
 * and, when wcomp >= 0, both face values weighted by component wcomp of the
 * same buffer).  u[d] (d < ndim): face TreeData of direction d. */
int sayaka_mac_set_rhs_div(sayaka_mac *h, const double *const *u, int32_t ncomp, int32_t ngrow, int32_t ucomp,
                           int32_t wcomp, double scale);
/* corr_vel (src/Test7.h:634-645): u_dir += dt * mg_flux_level(finest, dir,
 * solution) on the finest tower's blocks (TreeData::AddEqual,
 * src/SayakaTreeData.cpp:311-334); the solution never leaves the device.
 * u: face TreeData of direction dir, updated in place. */
int sayaka_mac_correct_vel(sayaka_mac *h, int32_t dir, double dt, double *u, int32_t ncomp, int32_t ngrow,
                           int32_t comp);

/* After AmrTree::regrid: the solution of the solver `old` (on the tree
 * before the regrid, same device) becomes the initial solution of `h` (on the
 * new tree), as the cell data part of initNewBlockDataAfterRegrid
 * (src/SayakaRegrid.cpp:987-1105): blocks matched by root and child path are
 * copied, refined blocks injected from their old leaf ancestor (prolongBlock),
 * blocks that became leaves by coarsening get the average of their old
 * children; a block with a deeper old subtree starts from zero. */
int sayaka_mac_init_from(sayaka_mac *h, const sayaka_mac *old);
/* The reference's own transfer for a cell state with PROLONG_CENTERED_LINEAR
 * and RESTRICT_AVERAGE, bit for bit: the solution of `old` is averaged down
 * (FillPatch::restrictAll, src/SayakaFillPatch.cpp:378-437), blocks present in
 * both trees keep it, and the new blocks are filled level by level by
 * AmrTree::initNewBlockDataAfterRegrid (src/SayakaRegrid.cpp:987-1105):
 * centered-linear interpolation from the parent
 * (src/SayakaInterpPatch.cpp:228-306), the parent's face ghosts from its
 * same-level neighbours or its physical BC (the types of sayaka_mac_set_bc,
 * values bc_val[face position] as the BCRegister's; NULL = all 0). */
int sayaka_mac_init_new_block_data(sayaka_mac *h, const sayaka_mac *old, const double *bc_val);

/* the library's pending CUDA runtime error on the calling thread (0 =
 * none), without clearing it: every call of this API leaves none behind */
int32_t sayaka_cuda_peek_error(void);

/* ---- self-test of the device solve's integer-pipe conversions (tests) ----
 * narrow[i] = double -> float of d[i] (round to nearest even) and
 * widen[i] = float -> double of f[i], widen0[i] = 0.0 + (double)f[i], each
 * next to the hardware conversion (_hw); no counterpart in the reference */
int sayaka_fp_selftest(const double *d, const float *f, int n, float *narrow, float *narrow_hw, double *widen,
                       double *widen_hw, double *widen0, double *widen0_hw);

/* ---- parity hooks on compact all-block arrays (tests and tools) ---- */
/* the solve's right-hand side (all blocks) */
int sayaka_mac_get_rhs_compact(sayaka_mac *h, double *out);
/* mg_apply_level(L) (src/SayakaMacOperator.cpp:84-137) */
int sayaka_mac_apply_compact(sayaka_mac *h, int32_t L, const double *x, double *y);
/* mg_residual_level(L) (src/SayakaMacUtil.cpp:9-49) */
int sayaka_mac_residual_compact(sayaka_mac *h, int32_t L, const double *x, const double *rhs, double *r);
/* The residual r = rhs - A x of tower L with its norms, allocating no device
 * memory: for callers that cannot call cudaMalloc where they need the norm (a
 * fixed memory pool, a host callback).  This entry point has no counterpart
 * in the reference.  x, rhs, r: DEVICE pointers to compact
 * all-block arrays; norms: DEVICE pointer to 2 doubles, set to {|r|_inf, r.r}
 * over tower L (a NaN in r gives a NaN |r|_inf); r is written on the tower's
 * cells only.  Runs on the handle's device, whatever device is current.
 * Enqueued on stream
 * (a cudaStream_t; NULL = the solver's stream) without host synchronisation.
 * Scratch is a static 128 KiB device array: towers of more than 2,097,152
 * cells are rejected (SAYAKA_BAD_INPUT, see sayaka_mac_last_error).  All calls
 * on a device share that scratch, so calls must not overlap (one stream, or
 * a synchronisation between them).  The first call on a device looks up the
 * scratch address and should come before any stream capture. */
int sayaka_mac_residual_norm_noalloc(sayaka_mac *h, int32_t L, const double *x, const double *rhs, double *r,
                                     double *norms, void *stream);
/* the device solve's own FP64 kernels, for comparison with the reference
 * arithmetic above: which 0 = out = A in on the finest tower with the fast
 * operator (per-cell factors, FMA; mg_apply_level, src/SayakaMacOperator.cpp:84-137);
 * which 1 = one smoothing pass of tower L in mg_smooth_level's order with the
 * fast sweep (launch variant 0..9, -1 the tuned one; in = phi, in2 = rhs);
 * which 2 = one block-hybrid pass (params.smoother 1) over tower L with
 * `variant` (1..1024) red-black sweeps per block (in = phi, frozen outside
 * each block; in2 = rhs); which 3 = out = A x on the finest tower for x = in
 * rounded to FP32, with the double-float operator the BiCGSTAB iteration
 * applies to the FP32 V-cycle's output (in2 unused) */
int sayaka_mac_device_kernel_compact(sayaka_mac *h, int32_t which, int32_t L, int32_t variant, const double *in,
                                     const double *in2, double *out);
/* one mg_smooth_level(L) (src/SayakaMacOperator.cpp:140-159, 1028-1112) */
int sayaka_mac_smooth_compact(sayaka_mac *h, int32_t L, const double *phi, const double *rhs, double *out);
/* mg_restict_wgt for levels finest-1 .. 1 (src/SayakaMacIB.cpp:157-232) */
int sayaka_mac_restrict_compact(sayaka_mac *h, const double *in, double *out);
/* mg_prolong_wgt for levels 2 .. finest (src/SayakaMacIB.cpp:234-283) */
int sayaka_mac_prolong_compact(sayaka_mac *h, const double *in, double *out);
/* mg_precond_level(finest) (src/SayakaMacSolver.cpp:924-949) */
int sayaka_mac_vcycle_compact(sayaka_mac *h, const double *p, double *phat);
/* mg_flux_level on compact arrays; flux is compact face data of dir */
int sayaka_mac_flux_compact(sayaka_mac *h, int32_t dir, const double *phi, double *flux);
/* fixBC with phi as [block][grown box] (ngrow layers) and compact rhs */
int sayaka_mac_fix_bc_compact(sayaka_mac *h, const double *phi_grown, int32_t ngrow, double *rhs);
/* coefficient fields after sync/restriction: which 0 = B[dir], 1 = area
 * fraction[dir], 2 = volume fraction */
int sayaka_mac_get_coef_compact(sayaka_mac *h, int32_t which, int32_t dir, double *out);

#ifdef __cplusplus
}
#endif

#endif /* SAYAKA_GB300_H */
