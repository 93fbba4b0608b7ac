// Device-side data of the MAC solver and the kernel launch interface.
//
// HBM layout (one pool per field, all blocks of all levels, indexed by the
// tree's block id):
//   cell field   : [block][k][j][i]              nb^ndim values per block
//   face field d : [block][..][face index in d]  (nb+1)*nb^(ndim-1) per block,
//                  the reference's face-centred valid-box order
// No ghost cells are stored: every kernel gathers the values a ghost cell
// would hold straight from the owning block (see mac_kernels.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sayaka_gb300 {

enum BCMath { kBCNeumann = 0, kBCDirichlet = 1, kBCSimpleFill = 2 };

// tables shared by every kernel (device pointers)
struct Topo {
  int ndim, nb, ncell;  // ncell = nb^ndim
  int lnb;              // log2(nb) when nb is a power of two, else -1
  int nfb;              // faces per block per direction
  int nblocks;
  const int *neighbor;   // [nblocks*6]
  const int *child;      // [nblocks*8]
  const int *parent;     // [nblocks]
  const int *which_child;// [nblocks]
  const int *fc_neigh;   // [nblocks*6] coarse leaf behind a -1 neighbour
  const int *bc_type;    // [nblocks*6] BCMath of physical faces, -1 otherwise
  int *err = nullptr;    // the solver's error word (a bounded wait that ran out sets it)
};

template <typename T>
struct Coef {
  const T *geom;      // [nblocks*8]: dx[3], ds[3], dv, unused
  const T *tff[3];    // same-level face coefficient ((beta*ds)/dx)*B*a
  const T *bcoef[3];  // face B
  const T *afrac[3];  // IB area fraction
  const T *vf;        // IB volume fraction
  T alpha, beta;
  // relaxation weight of the device V-cycle's red-black updates of fluid
  // cells (1: Gauss-Seidel; the reference-arithmetic kernels ignore it)
  T omega = 1;
  // Constant-coefficient blocks (device solve only; null elsewhere):
  // kUni values per block, [0..2] the same-level face coefficient of every
  // face of direction 0..2 of the block, [3] nonzero when the block is one
  // (every face of direction d has coefficient [d] and every cell vf = 1);
  // FP64 records also hold the factors of the block's interior cells (no
  // face on the block boundary): [4] P and [5] S of the outer operator,
  // [6] sa and [7] ia of the FP64 smoother.  Kernels read these instead of
  // the face arrays and vf, with the same arithmetic in the same order.
  const T *ut = nullptr;
};
constexpr int kUni = 8;

// Halo descriptor of a tower list entry, kHX ints: the ids every face of
// the block reads, precomputed so that a cell's gathers wait on one load
// (the descriptor) instead of a chain through the topology tables:
//   [f]            f < 2*ndim: same-level neighbour (FINE_FINE), coarse leaf
//                  (FINE_CRSE) or -1
//   [kHXInfo]      face types (low 16 bits) | which_child << 16
//   [kHXBlock]     the block id
//   [kHXKids+4f+k] CRSE_FINE face f: the fine child covering transverse
//                  halves k (bit j = half of the j-th transverse dimension)
//   [kHXPar+f]     FINE_FINE face f of a block below level 1: the
//                  neighbour's parent * 8 + its which_child, else -1
//   [kHXPar+6]     the block's own parent * 8 + which_child, or -1
constexpr int kHX = 40;
constexpr int kHXInfo = 6;
constexpr int kHXBlock = 7;
constexpr int kHXKids = 8;
constexpr int kHXPar = 32;

// BiCGSTAB state kept on the device (FP64 scalars and control flags) by the
// graph-captured solve of mac_fast.cu
struct FState {
  double rho, rho1, alpha, omega, beta;
  double rnorm0, rnorm;
  double tol_rel, tol_abs;
  int iter, max_iter;
  int done;     // loop ends (converged, breakdown or max_iter)
  int stat;     // 1 = breakdown
  int conv;     // converged
  int trivial;  // zero initial residual
  // learned correction: on, switched off after a stall, iterations since the
  // best residual, best residual
  int nn_on, nn_off, nn_since, pad_;
  double nn_best;
  // verified convergence: the recursive residual passed and the true
  // residual is being checked; the next iteration restarts from p = r;
  // restarts so far
  int verify, restart, restarts, pad2_;
};

// a block list with per-block packed face types (2 bits per face)
struct BlockList {
  const int *blocks;
  const uint16_t *ftypes;  // may be null for lists that need no face types
  int n;
  // FP64 smoother factors of a tower sublevel list, [entry][cell]:
  // sa = dv*vf/diag, ia = 1/diag (0 where vf = 0); null when not built
  const double *sa = nullptr, *ia = nullptr;
  const int *hx = nullptr;  // halo descriptors [entry][kHX] of tower lists, else null
  // level lists: [entry] parent * 8 + which_child; non-leaf lists:
  // [entry][8] children; null elsewhere
  const int *links = nullptr;
  // a forest of independent problems solved with one BiCGSTAB state per
  // problem (connected component of the tree): comp[block] and the states;
  // kernels leave the blocks of a finished problem alone.  Null otherwise.
  const int *comp = nullptr;
  const FState *stc = nullptr;
};

// chunks of a block list listed problem by problem (one BiCGSTAB state per
// problem): the BiCGSTAB kernels run one CTA per chunk of at most kChunkCells
// cells of one problem
// 16 cells per thread: the batch workload solves in 58.8 ms with 4096-cell
// chunks, 59.5 with 2048 or 8192
constexpr int kChunkCells = 4096;
struct Chunks {
  const int *comp;       // per chunk: its problem
  const int *beg, *end;  // per chunk: first and past-last cell of the list
  const int *c0, *cn;    // per problem: first chunk and number of chunks
};

// the block belongs to a problem whose solve has finished
__host__ __device__ __forceinline__ bool block_off(const BlockList &L, int b) {
  return L.stc && L.stc[L.comp[b]].done;
}

// The dense FP64 bottom solve: one inverse per connected component of the
// level-1 blocks (a forest of independent problems has one per problem),
// rows grouped by component, one CTA tile per 8 rows.
struct BottomDev {
  const double *binv;          // the components' row-major inverses, back to back
  const int *blocks;           // bottom-level block of every ncell rows, in row order
  const int *comp_row0, *comp_n;
  const long long *comp_off;   // start of each component's inverse in binv
  const int *tile_comp, *tile_row0;
  int ntiles, ncell, max_n;
  const int *comp = nullptr;      // per-problem states (see BlockList): rows of finished problems are skipped
  const FState *stc = nullptr;
  const float *binv32 = nullptr;  // FP32 copy of binv for the FP32 V-cycle (bottom level above 1)
  // or, instead, an FP16 copy with one FP32 scale per row (entry = h * scale)
  const unsigned short *binv16 = nullptr;
  const float *rscale = nullptr;
};
constexpr int kBottomTileRows = 8;

// one phase of the cooperative V-cycle program (mac_vcycle.cu)
enum PhaseOp { kPhaseRestrict = 0, kPhaseBottom = 1, kPhaseProlong = 2, kPhaseSmooth = 3, kPhaseOut = 4 };
struct VPhase {
  int op;
  int color;
  int n;
  int pad;
  const int *blocks;
  const uint16_t *ftypes;
  const double *sa, *ia;  // FP64 smoother factors (see BlockList)
};

// ---- launchers (mac_kernels.cu) ----
template <typename T>
void launch_face_coef(const Topo &t, const double *geom64, const T *bcoef[3], const T *afrac[3],
                      double beta, T *tff[3], cudaStream_t s);

// pdl: launch with Programmatic Dependent Launch (see launch.cuh)
template <typename T>
void launch_apply(const Topo &t, const Coef<T> &c, const BlockList &L, const T *x, T *y,
                  const T *rhs /*null: y = Ax; else y = rhs - Ax (masked)*/, const int *guard,
                  cudaStream_t s, bool pdl = false);

template <typename T>
void launch_smooth(const Topo &t, const Coef<T> &c, const BlockList &L, int color, T *phi,
                   const T *rhs, const int *guard, cudaStream_t s, bool pdl = false);
// the device solve's smoother (smooth_cell_fast); `variant` picks the
// launch bounds (0..kRbgsVariants-1), chosen per workload by the autotuner
constexpr int kRbgsVariants = 14;
// error word of the bulk-copy smoother variant (an mbarrier wait timed out);
// read (and cleared) by the host after a solve
// the solver's error word (Topo::err) after its stream is idle; clear: reset it
int rbgs_bulk_error(int *err, cudaStream_t s, bool clear);
template <typename T>
void launch_rbgs(const Topo &t, const Coef<T> &c, const BlockList &L, int color, T *phi,
                   const T *rhs, const int *guard, cudaStream_t s, bool pdl = false,
                 int variant = 0);

template <typename T>
void launch_restrict(const Topo &t, const Coef<T> &c, const BlockList &crse, T *phi,
                     const int *guard, cudaStream_t s, bool pdl = false);

template <typename T>
void launch_prolong(const Topo &t, const Coef<T> &c, const BlockList &fine, T *phi,
                    const int *guard, cudaStream_t s, bool pdl = false);
// prolongation of a level fused with the first red sweep of its sublevel
// (the level's blocks with the tower's face types); same values as
// launch_prolong + launch_rbgs(color 0)
template <typename T>
// X: a list (with halo descriptors) whose red cells are swept in the same
// launch, blocks that neither read nor are read by L's level
// form 1: one warp per block (2D FP32 16x16 blocks; elsewhere the CTA form 0)
void launch_prolong_red(const Topo &t, const Coef<T> &c, const BlockList &L, T *phi, const T *rhs,
                        const int *guard, cudaStream_t s, bool pdl = false,
                        const BlockList &X = BlockList{nullptr, nullptr, 0}, int form = 0);

// block-hybrid Gauss-Seidel pass (Gauss-Seidel inside a block, Jacobi
// between blocks): nsweep red-black sweeps of every block of L from src's
// values into dst (src unchanged); L may hold several sublevels
template <typename T>
void launch_bhgs(const Topo &t, const Coef<T> &c, const BlockList &L, int nsweep, const T *src, T *dst,
                 const T *rhs, const int *guard, cudaStream_t s, bool pdl = false);
template <typename T>
void launch_copy_blocks(const BlockList &L, int ncell, const T *src, T *dst, const int *guard, cudaStream_t s,
                        bool pdl = false);

void launch_flux(const Topo &t, const Coef<double> &c, const BlockList &L, int dir,
                 const double *phi, double *flux, cudaStream_t s);

void launch_fix_bc(const Topo &t, const Coef<double> &c, const BlockList &L,
                   const double *phi_grown, int ngrow, double *rhs, cudaStream_t s);

}  // namespace sayaka_gb300
