// The solution of a solver on an old tree carried onto the tree after a
// regrid (the cell data part of AmrTree::initNewBlockDataAfterRegrid,
// src/SayakaRegrid.cpp:987-1105, for the pressure the next solve starts
// from).  Blocks are matched by their root and the child path from it, which
// survives the id repacking of a regrid.  Every leaf of the new tree gets
//   * a copy of the same block of the old tree, or
//   * injection from its nearest old leaf ancestor when the block was refined
//     (the reference's prolongBlock of a new child, repeated when a regrid
//     refined more than one level), or
//   * the average of its old children when it became a leaf by coarsening,
//   * zero where the old tree had a deeper subtree (a valid initial guess).
#include <unordered_map>
#include <vector>

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
  CKR_(cudaMalloc(&d, std::max<size_t>(ints, 1) * sizeof(int)), 2);
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
  cudaFree(d);
  return 0;
}

}  // namespace sayaka_gb300
