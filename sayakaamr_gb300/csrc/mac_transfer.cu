// The solution of a solver on an old tree carried onto the tree after a
// regrid (the cell-data part of AmrTree::initNewBlockDataAfterRegrid,
// src/SayakaRegrid.cpp:987-1105, for the pressure the next solve starts
// from).  Blocks are matched by their root and the child path from it, which
// survives the id repacking of a regrid.  Two transfers:
//
// init_solution_from (injection): every leaf of the new tree gets
//   * a copy of the same block of the old tree, or
//   * injection from its nearest old leaf ancestor when the block was refined
//     (repeated when a regrid refined more than one level), or
//   * the average of its old children when it became a leaf by coarsening,
//   * zero where the old tree had a deeper subtree (a valid initial guess).
//
// init_new_block_data (the reference's own sequence for a cell state with
// PROLONG_CENTERED_LINEAR / RESTRICT_AVERAGE): the old field is averaged
// down (FillPatch::restrictAll, src/SayakaFillPatch.cpp:378-437), every block
// present in both trees keeps its data, and the new blocks are filled level
// by level from their parent by centered-linear interpolation
// (prolongCellBlockData_CenteredLinear, src/SayakaInterpPatch.cpp:228-306)
// with the parent's face ghosts from its same-level neighbours or its
// physical BC (fillBlockBndryAtSameLevel, BCPatch::fillBasicCellBlockBC,
// src/SayakaBoundaryPatch.cpp:139-234).  Same operations in the same order as
// the reference: bit-identical results.
#include <unordered_map>
#include <vector>

#include "dev_alloc.h"
#include "cuda_check.h"
#include "mac_solver.h"
#include "mac_stencil.cuh"
#include "tree.h"

namespace sayaka_gb300 {

namespace {

constexpr int kXT = 256;

// kind 0 copy, 1 injection from an old ancestor `depth` levels up (path: the
// child index at every step, 3 bits each, from the block upward), 2 average
// of the old children, 3 zero
__global__ void __launch_bounds__(kXT) k_transfer(int ndim, int nb, int ncell, int nmap, const int *__restrict__ blk,
                                                const int *__restrict__ kind, const int *__restrict__ src,
                                                const int *__restrict__ wc, const int *__restrict__ kids,
                                                const double *__restrict__ old_sol, double *__restrict__ sol) {
  const long total = (long)nmap * ncell;
  const int half = nb >> 1;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int m = (int)(it / ncell), ci = (int)(it - (long)m * ncell);
    int ijk[3];
    ijk[0] = ci % nb;
    ijk[1] = ndim >= 2 ? (ci / nb) % nb : 0;
    ijk[2] = ndim == 3 ? ci / (nb * nb) : 0;
    double v;
    if (kind[m] == 0) {
      v = old_sol[(long)src[m] * ncell + ci];
    } else if (kind[m] == 1) {
      int pc[3] = {ijk[0], ijk[1], ijk[2]};
      const int depth = kids[m * 8];
      for (int step = 0; step < depth; step++) {
        const int digit = (wc[m] >> (3 * step)) & 7;
        for (int q = 0; q < ndim; q++) pc[q] = ((digit >> q) & 1) * half + (pc[q] >> 1);
      }
      v = old_sol[(long)src[m] * ncell + stencil::encode(pc, nb)];
    } else if (kind[m] == 3) {
      v = 0.0;
    } else {
      int cidx = 0, fbase[3] = {0, 0, 0};
      for (int q = 0; q < ndim; q++) {
        const int sq = ijk[q] >= half ? 1 : 0;
        cidx |= sq << q;
        fbase[q] = 2 * (ijk[q] - sq * half);
      }
      const int F = kids[m * 8 + cidx];
      double sum = 0.0;
      for (int kk = 0; kk < (ndim == 3 ? 2 : 1); kk++)
        for (int jj = 0; jj < 2; jj++)
          for (int ii = 0; ii < 2; ii++) {
            const int fi[3] = {fbase[0] + ii, fbase[1] + jj, ndim == 3 ? fbase[2] + kk : 0};
            sum += old_sol[(long)F * ncell + stencil::encode(fi, nb)];
          }
      v = sum / (double)(1 << ndim);
    }
    sol[(long)blk[m] * ncell + ci] = v;
  }
}

// root id and child path from the root: one 64-bit key per block
std::vector<unsigned long long> path_keys(const TreeTables &t) {
  std::vector<unsigned long long> key(t.num_blocks, 0);
  for (int b = 0; b < t.num_blocks; b++) {
    unsigned long long path = 0;
    int depth = 0, x = b;
    while (t.parent[x] >= 0) {
      path |= (unsigned long long)(t.which_child[x] & 7) << (3 * depth);
      depth++;
      x = t.parent[x];
    }
    key[b] = ((unsigned long long)x << 44) | ((unsigned long long)depth << 39) | path;
  }
  return key;
}

// FillPatch::restrictAll, one level: every listed (non-leaf) block's cells =
// (sum of its 2^d fine cells, k, j, i order, from 0) * (1 / 2^d)
__global__ void __launch_bounds__(kXT) k_avg_down(int ndim, int nb, int ncell, int n, const int *__restrict__ blocks,
                                                const int *__restrict__ child, double *__restrict__ x) {
  const long total = (long)n * ncell;
  const int half = nb >> 1;
  const double wgt = 1.0 / (double)(1 << ndim);
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell), ci = (int)(it - (long)p * ncell);
    const int b = blocks[p];
    int ijk[3];
    ijk[0] = ci % nb;
    ijk[1] = ndim >= 2 ? (ci / nb) % nb : 0;
    ijk[2] = ndim == 3 ? ci / (nb * nb) : 0;
    int cidx = 0, fb[3] = {0, 0, 0};
    for (int q = 0; q < ndim; q++) {
      const int sq = ijk[q] >= half ? 1 : 0;
      cidx |= sq << q;
      fb[q] = 2 * (ijk[q] - sq * half);
    }
    const double *F = x + (long)child[b * 8 + cidx] * ncell;
    double sum = 0.0;
    for (int kk = 0; kk < (ndim == 3 ? 2 : 1); kk++)
      for (int jj = 0; jj < 2; jj++)
        for (int ii = 0; ii < 2; ii++) {
          const int fi[3] = {fb[0] + ii, fb[1] + jj, ndim == 3 ? fb[2] + kk : 0};
          sum = __dadd_rn(sum, F[stencil::encode(fi, nb)]);
        }
    x[(long)b * ncell + ci] = __dmul_rn(sum, wgt);
  }
}

// x_new[dst[i]] = x_old[src[i]], whole blocks
__global__ void __launch_bounds__(kXT) k_copy_blocks(int ncell, int n, const int *__restrict__ dst,
                                                   const int *__restrict__ src, const double *__restrict__ xo,
                                                   double *__restrict__ x) {
  const long total = (long)n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell), ci = (int)(it - (long)p * ncell);
    x[(long)dst[p] * ncell + ci] = xo[(long)src[p] * ncell + ci];
  }
}

struct BcValues {
  double v[6];
};

// the parent's cell at coarse index c, moved by dir = +-1 along q; outside the
// parent, its face ghost: the same-level neighbour's mirrored cell, else the
// physical BC of that face (Neumann: the boundary cell; Dirichlet:
// 2 * value - boundary cell; SimpleFill: the value)
__device__ __forceinline__ double parent_cell(const Topo &t, const int *level, const BcValues &bv, int P,
                                              const int c[3], int q, int dir, const double *x) {
  int a[3] = {c[0], c[1], c[2]};
  a[q] += dir;
  const int nb = t.nb;
  if (a[q] >= 0 && a[q] < nb) return x[(long)P * t.ncell + stencil::encode(a, nb)];
  const int f = 2 * q + (dir > 0 ? 1 : 0);
  const int n = t.neighbor[P * 6 + f];
  if (n >= 0 && level[n] == level[P]) {
    a[q] = dir > 0 ? 0 : nb - 1;
    return x[(long)n * t.ncell + stencil::encode(a, nb)];
  }
  const double vref = x[(long)P * t.ncell + stencil::encode(c, nb)];
  if (n <= kPhysBndry) {
    const int bt = t.bc_type[P * 6 + f];
    if (bt == 1) return __dsub_rn(__dmul_rn(2.0, bv.v[f]), vref);
    if (bt == 2) return bv.v[f];
  }
  return vref;  // Neumann (no same-level neighbour inside the domain cannot occur in a 2:1-balanced tree)
}

// prolongCellBlockData_CenteredLinear of every listed block from its parent
template <int ND>
__global__ void __launch_bounds__(kXT) k_prolong_centered(Topo t, int n, const int *__restrict__ blocks,
                                                        const int *__restrict__ level, BcValues bv, double *x) {
  const int nb = t.nb, ncell = t.ncell, half = nb >> 1;
  const long total = (long)n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell), ci = (int)(it - (long)p * ncell);
    const int b = blocks[p], P = t.parent[b], wc = t.which_child[b];
    int ijk[3], c[3] = {0, 0, 0};
    ijk[0] = ci % nb;
    ijk[1] = (ci / nb) % nb;
    ijk[2] = ND == 3 ? ci / (nb * nb) : 0;
    for (int q = 0; q < ND; q++) c[q] = ((wc >> q) & 1) * half + (ijk[q] >> 1);
    const double c0 = x[(long)P * ncell + stencil::encode(c, nb)];
    double g[3] = {0.0, 0.0, 0.0}, rel[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < ND; q++) {
      const double cp = parent_cell(t, level, bv, P, c, q, 1, x);
      const double cm = parent_cell(t, level, bv, P, c, q, -1, x);
      g[q] = __dmul_rn(0.5, __dsub_rn(cp, cm));
      rel[q] = (ijk[q] & 1) ? 0.25 : -0.25;
    }
    double v = __dadd_rn(c0, __dmul_rn(rel[0], g[0]));
    v = __dadd_rn(v, __dmul_rn(rel[1], g[1]));
    v = __dadd_rn(v, __dmul_rn(rel[2], g[2]));  // 2D: + 0 * 0, as the reference's third term
    x[(long)b * ncell + ci] = v;
  }
}

}  // namespace

int MacGpu::init_solution_from(const MacGpu &old, std::string *why) {
  if (old.device_ != device_) {
    *why = "init_from: the solvers live on different devices";
    return 1;
  }
  if (old.tt_.ndim != tt_.ndim || old.tt_.nb != tt_.nb) {
    *why = "init_from: the trees differ in dimension or block size";
    return 1;
  }
  if (tt_.max_level > 13 || old.tt_.max_level > 13) {
    *why = "init_from: more than 13 levels";
    return 1;
  }
  const std::vector<unsigned long long> ko = path_keys(old.tt_), kn = path_keys(tt_);
  std::unordered_map<unsigned long long, int> where;
  where.reserve(ko.size() * 2);
  for (int b = 0; b < old.tt_.num_blocks; b++) where[ko[b]] = b;
  std::vector<int> blk, kind, src, wc, kids;
  for (int b = 0; b < tt_.num_blocks; b++) {
    if (tt_.node_type[b] != kNodeLeaf) continue;
    auto it = where.find(kn[b]);
    if (it != where.end() && old.tt_.node_type[it->second] == kNodeLeaf) {
      blk.push_back(b), kind.push_back(0), src.push_back(it->second), wc.push_back(0);
      kids.insert(kids.end(), 8, -1);
      continue;
    }
    if (it == where.end()) {  // refined: walk up to the nearest old leaf
      int a = b, depth = 0, path = 0;
      auto ia = where.end();
      while (tt_.parent[a] >= 0 && depth < 10) {
        path |= (tt_.which_child[a] & 7) << (3 * depth);
        depth++;
        a = tt_.parent[a];
        ia = where.find(kn[a]);
        if (ia != where.end()) break;
      }
      if (ia != where.end() && old.tt_.node_type[ia->second] == kNodeLeaf) {
        blk.push_back(b), kind.push_back(1), src.push_back(ia->second), wc.push_back(path);
        kids.push_back(depth);
        kids.insert(kids.end(), 7, -1);
        continue;
      }
    }
    if (it != where.end()) {  // a parent in the old tree whose children were leaves
      const int ob = it->second;
      bool ok = true;
      for (int c = 0; c < (1 << tt_.ndim); c++) {
        const int oc = old.tt_.child[ob * 8 + c];
        ok = ok && oc >= 0 && old.tt_.node_type[oc] == kNodeLeaf;
      }
      if (ok) {
        blk.push_back(b), kind.push_back(2), src.push_back(ob), wc.push_back(0);
        for (int c = 0; c < 8; c++) kids.push_back(c < (1 << tt_.ndim) ? old.tt_.child[ob * 8 + c] : -1);
        continue;
      }
    }
    blk.push_back(b), kind.push_back(3), src.push_back(0), wc.push_back(0);
    kids.insert(kids.end(), 8, -1);
  }
  const int nmap = (int)blk.size();
  const size_t n = (size_t)tt_.num_blocks * ncell_;
  int *d = nullptr;
  const size_t ints = (size_t)nmap * 4 + kids.size();
  CKR_(dev_malloc(&d, std::max<size_t>(ints, 1) * sizeof(int)), 2);
  std::vector<int> pack;
  pack.reserve(ints);
  for (auto *v : {&blk, &kind, &src, &wc, &kids}) pack.insert(pack.end(), v->begin(), v->end());
  CKR_(cudaMemcpyAsync(d, pack.data(), pack.size() * sizeof(int), cudaMemcpyHostToDevice, stream_), 2);
  CKR_(cudaMemsetAsync(vec_[kSOL], 0, n * sizeof(double), stream_), 2);
  // the old solver's solution is complete once its stream is idle
  CKR_(cudaStreamSynchronize(old.stream_), 2);
  const long w = (long)nmap * ncell_;
  if (w > 0)
    k_transfer<<<(int)std::min<long>((w + kXT - 1) / kXT, 152 * 32), kXT, 0, stream_>>>(
        tt_.ndim, tt_.nb, ncell_, nmap, d, d + nmap, d + 2 * nmap, d + 3 * nmap, d + 4 * nmap, old.vec_[kSOL],
        vec_[kSOL]);
  CKR_(cudaGetLastError(), 2);
  CKR_(cudaStreamSynchronize(stream_), 2);
  dev_free(d);
  return 0;
}

int MacGpu::init_new_block_data(const MacGpu &old, const double *bc_val, std::string *why) {
  if (old.device_ != device_) {
    *why = "init_new_block_data: the solvers live on different devices";
    return 1;
  }
  if (old.tt_.ndim != tt_.ndim || old.tt_.nb != tt_.nb || tt_.ndim < 2) {
    *why = "init_new_block_data: the trees differ in dimension or block size";
    return 1;
  }
  if (tt_.max_level > 13 || old.tt_.max_level > 13) {
    *why = "init_new_block_data: more than 13 levels";
    return 1;
  }
  BcValues bv{};
  for (int f = 0; f < 6; f++) bv.v[f] = bc_val ? bc_val[f] : 0.0;
  const std::vector<unsigned long long> ko = path_keys(old.tt_), kn = path_keys(tt_);
  std::unordered_map<unsigned long long, int> where;
  where.reserve(ko.size() * 2);
  for (int b = 0; b < old.tt_.num_blocks; b++) where[ko[b]] = b;
  // host lists: the old tree's non-leaf blocks by level (restriction, finest-1
  // .. 1), the kept blocks (new id, old id), the new blocks by level
  std::vector<int> pack;
  std::vector<std::pair<int, int>> avg_lv;  // (offset, count) per level, in launch order
  int old_finest = 1;
  for (int b = 0; b < old.tt_.num_blocks; b++)
    if (old.tt_.node_type[b] == kNodeLeaf) old_finest = std::max(old_finest, old.tt_.level[b]);
  for (int l = old_finest - 1; l >= 1; l--) {
    const int off = (int)pack.size();
    for (int b = 0; b < old.tt_.num_blocks; b++)
      if (old.tt_.level[b] == l && old.tt_.node_type[b] != kNodeLeaf) pack.push_back(b);
    avg_lv.push_back({off, (int)pack.size() - off});
  }
  const int keep_off = (int)pack.size();
  std::vector<int> keep_src, fresh;
  for (int b = 0; b < tt_.num_blocks; b++) {
    auto it = where.find(kn[b]);
    if (it != where.end()) {
      pack.push_back(b);
      keep_src.push_back(it->second);
    } else {
      fresh.push_back(b);
    }
  }
  const int nkeep = (int)keep_src.size();
  const int src_off = (int)pack.size();
  pack.insert(pack.end(), keep_src.begin(), keep_src.end());
  std::vector<std::pair<int, int>> new_lv;
  for (int l = 2; l <= tt_.max_level; l++) {
    const int off = (int)pack.size();
    for (int b : fresh)
      if (tt_.level[b] == l) pack.push_back(b);
    if ((int)pack.size() > off) new_lv.push_back({off, (int)pack.size() - off});
  }
  const int level_off = (int)pack.size();
  pack.insert(pack.end(), tt_.level.begin(), tt_.level.end());
  const size_t nold = (size_t)old.tt_.num_blocks * ncell_, n = (size_t)tt_.num_blocks * ncell_;
  int *d = nullptr;
  double *tmp = nullptr;
  CKR_(dev_malloc(&d, std::max<size_t>(pack.size(), 1) * sizeof(int)), 2);
  if (dev_malloc(&tmp, std::max<size_t>(nold, 1) * sizeof(double)) != cudaSuccess) {
    dev_free(d);
    *why = "init_new_block_data: out of device memory";
    return 2;
  }
  CKR_(cudaMemcpyAsync(d, pack.data(), pack.size() * sizeof(int), cudaMemcpyHostToDevice, stream_), 2);
  // the old solver's solution is complete once its stream is idle
  CKR_(cudaStreamSynchronize(old.stream_), 2);
  CKR_(cudaMemcpyAsync(tmp, old.vec_[kSOL], nold * sizeof(double), cudaMemcpyDeviceToDevice, stream_), 2);
  auto grid = [](long w) { return (int)std::max<long>(1, std::min<long>((w + kXT - 1) / kXT, 152 * 32)); };
  for (const auto &lv : avg_lv)
    if (lv.second > 0)
      k_avg_down<<<grid((long)lv.second * ncell_), kXT, 0, stream_>>>(tt_.ndim, tt_.nb, ncell_, lv.second,
                                                                     d + lv.first, old.topo_.child, tmp);
  CKR_(cudaMemsetAsync(vec_[kSOL], 0, n * sizeof(double), stream_), 2);
  if (nkeep > 0)
    k_copy_blocks<<<grid((long)nkeep * ncell_), kXT, 0, stream_>>>(ncell_, nkeep, d + keep_off, d + src_off, tmp,
                                                                   vec_[kSOL]);
  for (const auto &lv : new_lv) {
    if (tt_.ndim == 2)
      k_prolong_centered<2><<<grid((long)lv.second * ncell_), kXT, 0, stream_>>>(topo_, lv.second, d + lv.first,
                                                                                 d + level_off, bv, vec_[kSOL]);
    else
      k_prolong_centered<3><<<grid((long)lv.second * ncell_), kXT, 0, stream_>>>(topo_, lv.second, d + lv.first,
                                                                                 d + level_off, bv, vec_[kSOL]);
  }
  CKR_(cudaGetLastError(), 2);
  CKR_(cudaStreamSynchronize(stream_), 2);
  dev_free(tmp);
  dev_free(d);
  return 0;
}

}  // namespace sayaka_gb300
