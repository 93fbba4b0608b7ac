// Host orchestration of the GPU MAC solver: device pools, block lists,
// coefficient setup, vector kernels / reductions, the V-cycle preconditioner
// and the BiCGSTAB driver.
#include <mutex>

#include "dev_alloc.h"
#include "mac_solver.h"

#include <algorithm>
#include <functional>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "tower.h"
#include "tree.h"

namespace sayaka_gb300 {

// the pool of each device keeps what is freed (release threshold raised once
// per device and process)
static void pool_keep_freed() {
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
  std::lock_guard<std::mutex> lk(mu);
  if (done[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    unsigned long long keep = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  done[dev] = true;
}

cudaError_t dev_malloc_bytes(void **p, size_t bytes) {
  pool_keep_freed();
  const cudaError_t e = cudaMallocAsync(p, bytes, 0);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(0);
}

cudaError_t dev_free(void *p) {
  if (!p) return cudaSuccess;
  const cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return e;
  return cudaFreeAsync(p, 0);
}


#include "cuda_check.h"

namespace {

constexpr int kThreads = 256;
constexpr int kRedBlocks = 2 * 152;

inline int grid_for(long work) {
  long g = (work + kThreads - 1) / kThreads;
  if (g < 1) g = 1;
  if (g > 152 * 32) g = 152 * 32;
  return (int)g;
}

__global__ void k_copy(BlockList L, int ncell, double *dst, const double *src) {
  const long total = (long)L.n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell);
    const long q = (long)L.blocks[p] * ncell + (it - (long)p * ncell);
    dst[q] = src[q];
  }
}
__global__ void k_zero(BlockList L, int ncell, double *dst) {
  const long total = (long)L.n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell);
    dst[(long)L.blocks[p] * ncell + (it - (long)p * ncell)] = 0.0;
  }
}
// out = a*x + b*y (src/SayakaBlockData.cpp:213-261)
__global__ void k_axpby(BlockList L, int ncell, double *out, double a, const double *x, double b, const double *y) {
  const long total = (long)L.n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell);
    const long q = (long)L.blocks[p] * ncell + (it - (long)p * ncell);
    out[q] = a * x[q] + b * y[q];
  }
}
// masked copy r = (vf > 0) ? src : 0
__global__ void k_masked_copy(BlockList L, int ncell, const double *vf, double *dst, const double *src) {
  const long total = (long)L.n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell);
    const long q = (long)L.blocks[p] * ncell + (it - (long)p * ncell);
    dst[q] = vf[q] > 0 ? src[q] - 0.0 : 0.0;
  }
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// MODE 0: sum a*b ; MODE 1: max |a|.  Two-level reduction, the last block
// to finish combines the per-block partials in a fixed order.
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_reduce(BlockList L, int ncell, const double *a, const double *b,
                                                     double *partials, unsigned *counter, double *out) {
  __shared__ double sh[kThreads / 32];
  __shared__ bool last;
  double acc = 0.0;
  const long total = (long)L.n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell);
    const long q = (long)L.blocks[p] * ncell + (it - (long)p * ncell);
    if (MODE == 0)
      acc += a[q] * b[q];
    else
      acc = fmax(acc, fabs(a[q]));
  }
  acc = MODE == 0 ? warp_sum(acc) : warp_max(acc);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < kThreads / 32 ? sh[threadIdx.x] : 0.0;
    v = MODE == 0 ? warp_sum(v) : warp_max(v);
    if (threadIdx.x == 0) {
      partials[blockIdx.x] = v;
      __threadfence();
      const unsigned t = atomicAdd(counter, 1u);
      last = (t == gridDim.x - 1);
    }
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double v = 0.0;
  for (int i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
    const double pv = ((volatile double *)partials)[i];
    v = MODE == 0 ? v + pv : fmax(v, pv);
  }
  v = MODE == 0 ? warp_sum(v) : warp_max(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < kThreads / 32; w++) r = MODE == 0 ? r + sh[w] : fmax(r, sh[w]);
    *out = r;
    *counter = 0;
  }
}

template <typename T>
T *dalloc(size_t n) {
  T *p = nullptr;
  if (dev_malloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
  cudaMemset(p, 0, std::max<size_t>(n, 1) * sizeof(T));
  cudaStreamSynchronize(0);  // zeroed before any stream of the solver touches it
  return p;
}

// halo descriptors of a tower list (see kHX), one thread per entry
__global__ void k_make_hx(int n, int nd, const int *__restrict__ blocks, const uint16_t *__restrict__ fts,
                          const int *__restrict__ neighbor, const int *__restrict__ parent,
                          const int *__restrict__ which_child, const int *__restrict__ child,
                          const int *__restrict__ fc_neigh, int *__restrict__ hx) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const int b = blocks[p];
    const unsigned ft = fts[p];
    int e[kHX];
    for (int k = 0; k < kHX; k++) e[k] = -1;
    e[kHXInfo] = (int)(ft | ((unsigned)which_child[b] << 16));
    e[kHXBlock] = b;
    if (parent[b] >= 0) e[kHXPar + 6] = parent[b] * 8 + which_child[b];
    for (int f = 0; f < 2 * nd; f++) {
      const int ty = (ft >> (2 * f)) & 3, d = f >> 1, s = f & 1;
      if (ty == 0) {
        const int nbr = neighbor[b * 6 + f];
        e[f] = nbr;
        if (parent[nbr] >= 0) e[kHXPar + f] = parent[nbr] * 8 + which_child[nbr];
      }
      if (ty == 2) e[f] = fc_neigh[b * 6 + f];
      if (ty != 3) continue;
      const int N = neighbor[b * 6 + f];
      for (int k = 0; k < (1 << (nd - 1)); k++) {
        int cidx = (1 - s) << d, j = 0;
        for (int q = 0; q < nd; q++)
          if (q != d) cidx |= ((k >> j++) & 1) << q;
        e[kHXKids + f * 4 + k] = child[N * 8 + cidx];
      }
    }
    int *out = hx + (long)p * kHX;
    for (int k = 0; k < kHX; k++) out[k] = e[k];
  }
}

// A TreeData-layout field (per block `ncomp` components of G0 x G1 x G2
// values, G = nb + 2 ngrow in each dimension) and the compact vector of the
// valid cells, one thread per cell, x fastest on both sides
struct TdLayout {
  int nd, nb, ncomp, g, comp;
  long G0, G1, cap;
};
__device__ __forceinline__ long td_at(const TdLayout &L, int b, int i, int j, int k) {
  const long gz = L.nd == 3 ? L.g : 0;
  return (long)b * L.cap * L.ncomp + (long)L.comp * L.cap + (i + L.g) + L.G0 * ((j + L.g) + L.G1 * (k + gz));
}
__global__ void k_td_gather(TdLayout L, long total, int ncell, const double *__restrict__ td, double *__restrict__ out) {
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int b = (int)(it / ncell), ci = (int)(it - (long)b * ncell);
    const int i = ci % L.nb, j = (ci / L.nb) % L.nb, k = L.nd == 3 ? ci / (L.nb * L.nb) : 0;
    out[it] = td[td_at(L, b, i, j, k)];
  }
}
__global__ void k_td_scatter(TdLayout L, long total, int ncell, const double *__restrict__ in, double *__restrict__ td) {
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int b = (int)(it / ncell), ci = (int)(it - (long)b * ncell);
    const int i = ci % L.nb, j = (ci / L.nb) % L.nb, k = L.nd == 3 ? ci / (L.nb * L.nb) : 0;
    td[td_at(L, b, i, j, k)] = in[it];
  }
}

void tree_from_tables(const TreeTables &tt, AmrTree &t) {
  t.init(tt.ndim, tt.nb, tt.min_level, tt.max_level, std::max(tt.num_blocks, 1), false);
  t.num_blocks = tt.num_blocks;
  for (int b = 0; b < tt.num_blocks; b++) {
    TreeNode &n = t.nodes[b];
    n.level = tt.level[b];
    for (int f = 0; f < 6; f++) n.neighbor[f] = tt.neighbor[b * 6 + f];
    for (int c = 0; c < 8; c++) n.child[c] = tt.child[b * 8 + c];
    n.parent = tt.parent[b];
    n.which_child = tt.which_child[b];
    n.node_type = tt.node_type[b];
  }
  for (int l = 1; l <= tt.max_level; l++) t.levels[l].clear();
  for (int b = 0; b < tt.num_blocks; b++)
    if (tt.level[b] >= 1 && tt.level[b] <= tt.max_level) t.levels[tt.level[b]].push_back(b);
}

}  // namespace

void MacGpu::fail(const std::string &m) {
  if (err_.empty()) err_ = m;
}

MacGpu::MacGpu(const TreeTables &tt) : tt_(tt) {
  // every buffer of the solver lives on the device current at construction
  if (cudaGetDevice(&device_) != cudaSuccess) {
    cudaGetLastError();
    device_ = 0;
  }
  const int nd = tt.ndim, nb = tt.nb, nbk = tt.num_blocks;
  if (nd < 2 || nd > 3 || nb < 2 || (nb & 1) || nbk <= 0) {
    fail("bad tree tables (ndim 2|3, even nb, blocks > 0)");
    return;
  }
  ncell_ = nd == 2 ? nb * nb : nb * nb * nb;
  nfb_ = nd == 2 ? (nb + 1) * nb : (nb + 1) * nb * nb;
  finest_ = 0;
  for (int b = 0; b < nbk; b++) finest_ = std::max(finest_, tt.level[b]);
  if (finest_ < 1 || finest_ > tt.max_level) {
    fail("bad block levels");
    return;
  }
  CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));

  // geometry exactly as the reference computes it (src/SayakaTree.h:277-301)
  geom_.assign((size_t)nbk * 8, 0.0);
  for (int b = 0; b < nbk; b++) {
    double dx[3], ds[3] = {1, 1, 1}, v = 1.0;
    for (int d = 0; d < 3; d++) dx[d] = tt.block_len[b * 3 + d];
    for (int d = 0; d < nd; d++) dx[d] /= nb;
    for (int d = 0; d < nd; d++) v *= dx[d];
    for (int d = 0; d < nd; d++) ds[d] = v / dx[d];
    for (int d = 0; d < 3; d++) {
      geom_[b * 8 + d] = dx[d];
      geom_[b * 8 + 3 + d] = ds[d];
    }
    geom_[b * 8 + 6] = v;
  }
  // coarse leaf behind a coarse/fine face: the parent's neighbour
  fc_neigh_.assign((size_t)nbk * 6, -1);
  for (int b = 0; b < nbk; b++)
    for (int f = 0; f < 2 * nd; f++) {
      const int nbr = tt.neighbor[b * 6 + f];
      if (nbr < 0 && nbr > kPhysBndry && tt.parent[b] >= 0) fc_neigh_[b * 6 + f] = tt.neighbor[tt.parent[b] * 6 + f];
    }
  bc_type_.assign((size_t)nbk * 6, -1);
  // the host copies of B and the fractions are filled on demand (pull_coefs)
  host_coef_stale_ = true;

  // towers and level lists
  AmrTree t;
  tree_from_tables(tt, t);
  std::vector<Tower> tw = build_towers(t);
  towers_.resize(tt.max_level + 1);
  // device tables (the halo descriptors below are built from them)
  d_neighbor_ = dalloc<int>((size_t)nbk * 6);
  d_child_ = dalloc<int>((size_t)nbk * 8);
  d_parent_ = dalloc<int>(nbk);
  d_wc_ = dalloc<int>(nbk);
  d_fc_neigh_ = dalloc<int>((size_t)nbk * 6);
  d_bc_type_ = dalloc<int>((size_t)nbk * 6);
  d_err_ = dalloc<int>(1);
  d_geom_ = dalloc<double>((size_t)nbk * 8);
  CK(cudaMemcpy(d_neighbor_, tt.neighbor.data(), (size_t)nbk * 6 * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_child_, tt.child.data(), (size_t)nbk * 8 * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_parent_, tt.parent.data(), (size_t)nbk * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_wc_, tt.which_child.data(), (size_t)nbk * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_fc_neigh_, fc_neigh_.data(), (size_t)nbk * 6 * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_geom_, geom_.data(), (size_t)nbk * 8 * sizeof(double), cudaMemcpyHostToDevice));
  // halo descriptors of a tower list (see kHX), built on the device
  auto make_hx = [&](const int *blk, const uint16_t *fts, int n, int *hx) {
    if (n <= 0) return;
    k_make_hx<<<std::min((n + 255) / 256, 152 * 8), 256, 0, stream_>>>(n, nd, blk, fts, d_neighbor_, d_parent_, d_wc_,
                                                                      d_child_, d_fc_neigh_, hx);
  };
  for (int L = 1; L <= tt.max_level; L++) {
    const Tower &src = tw[L];
    DevTower &dt = towers_[L];
    dt.begin = src.begin;
    dt.end = src.end;
    dt.blocks = src.blocks;
    const int n = (int)src.blocks.size();
    std::vector<uint16_t> ft(n, 0);
    for (int p = 0; p < n; p++) {
      uint16_t v = 0;
      for (int f = 0; f < 2 * nd; f++) v |= (uint16_t)(src.regs[p * 6 + f].type & 3) << (2 * f);
      ft[p] = v;
    }
    dt.all.n = n;
    dt.all.blocks = dalloc<int>(n);
    dt.all.ftypes = dalloc<uint16_t>(n);
    dt.all.hx = dalloc<int>((size_t)n * kHX);
    if (n) {
      CK(cudaMemcpy(dt.all.blocks, src.blocks.data(), n * sizeof(int), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(dt.all.ftypes, ft.data(), n * sizeof(uint16_t), cudaMemcpyHostToDevice));
      make_hx(dt.all.blocks, dt.all.ftypes, n, dt.all.hx);
    }
    // parity-grouped copy of the sublevels the V-cycle smooths (L down to
    // the first empty sublevel, as the per-sublevel loop does)
    int low = L;
    while (low - 1 >= 1 && src.end[low - 1] > src.begin[low - 1]) low--;
    std::vector<int> pb;
    std::vector<uint16_t> pf;
    for (int g = 0; g < 2; g++) {
      if (g == 1) dt.par_split = (int)pb.size();
      for (int l = L - g; l >= low; l -= 2)
        for (int p = src.begin[l]; p < src.end[l]; p++) {
          pb.push_back(src.blocks[p]);
          pf.push_back(ft[p]);
        }
      if (g == 0) dt.par_top = src.end[L] - src.begin[L];
    }
    dt.par.n = (int)pb.size();
    dt.par.blocks = dalloc<int>(pb.size());
    dt.par.ftypes = dalloc<uint16_t>(pb.size());
    dt.par.hx = dalloc<int>(pb.size() * kHX);
    if (!pb.empty()) {
      CK(cudaMemcpy(dt.par.blocks, pb.data(), pb.size() * sizeof(int), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(dt.par.ftypes, pf.data(), pf.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
      make_hx(dt.par.blocks, dt.par.ftypes, (int)pb.size(), dt.par.hx);
    }
  }
  // Independent problems in one tree (a forest: no neighbour, parent or child
  // link between them) each get their own BiCGSTAB state.  Components are
  // numbered in the order of their lowest block id.
  {
    std::vector<int> up(nbk);
    for (int b = 0; b < nbk; b++) up[b] = b;
    std::function<int(int)> root = [&](int b) {
      while (up[b] != b) b = up[b] = up[up[b]];
      return b;
    };
    auto join = [&](int a, int b) {
      if (b < 0 || b >= nbk) return;
      a = root(a);
      b = root(b);
      if (a != b) up[std::max(a, b)] = std::min(a, b);
    };
    for (int b = 0; b < nbk; b++) {
      for (int f = 0; f < 2 * nd; f++) join(b, tt.neighbor[b * 6 + f]);
      join(b, tt.parent[b]);
    }
    comp_of_block_.assign(nbk, 0);
    std::vector<int> id(nbk, -1);
    ncomp_ = 0;
    for (int b = 0; b < nbk; b++) {
      const int r = root(b);
      if (id[r] < 0) id[r] = ncomp_++;
      comp_of_block_[b] = id[r];
    }
  }
  if (ncomp_ > 1 && towers_[finest_].all.n > 0) {
    // the finest tower problem by problem, and its chunks (see Chunks)
    const DevTower &ft = towers_[finest_];
    const int n = ft.all.n;
    std::vector<int> perm(n);
    for (int p = 0; p < n; p++) perm[p] = p;
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) {
      return comp_of_block_[ft.blocks[a]] < comp_of_block_[ft.blocks[b]];
    });
    std::vector<uint16_t> ftypes(n);
    CK(cudaMemcpy(ftypes.data(), ft.all.ftypes, n * sizeof(uint16_t), cudaMemcpyDeviceToHost));
    std::vector<int> pb(n);
    std::vector<uint16_t> pf(n);
    for (int p = 0; p < n; p++) {
      pb[p] = ft.blocks[perm[p]];
      pf[p] = ftypes[perm[p]];
    }
    tlc_.n = n;
    tlc_.blocks = dalloc<int>(n);
    tlc_.ftypes = dalloc<uint16_t>(n);
    tlc_.hx = dalloc<int>((size_t)n * kHX);
    CK(cudaMemcpy(tlc_.blocks, pb.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(tlc_.ftypes, pf.data(), n * sizeof(uint16_t), cudaMemcpyHostToDevice));
    make_hx(tlc_.blocks, tlc_.ftypes, n, tlc_.hx);
    std::vector<int> ccomp, cbeg, cend, c0(ncomp_, 0), cn(ncomp_, 0);
    const long nc = ncell_;
    for (int p = 0; p < n;) {
      const int c = comp_of_block_[pb[p]];
      int q = p;
      while (q < n && comp_of_block_[pb[q]] == c) q++;
      c0[c] = (int)ccomp.size();
      for (long a = (long)p * nc; a < (long)q * nc; a += kChunkCells) {
        ccomp.push_back(c);
        cbeg.push_back((int)a);
        cend.push_back((int)std::min<long>(a + kChunkCells, (long)q * nc));
      }
      cn[c] = (int)ccomp.size() - c0[c];
      p = q;
    }
    nchunks_ = (int)ccomp.size();
    std::vector<int> all;
    for (auto *v : {&ccomp, &cbeg, &cend}) all.insert(all.end(), v->begin(), v->end());
    all.insert(all.end(), c0.begin(), c0.end());
    all.insert(all.end(), cn.begin(), cn.end());
    d_chunk_ = dalloc<int>(all.size());
    CK(cudaMemcpy(d_chunk_, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice));
    d_comp_ = dalloc<int>(nbk);
    CK(cudaMemcpy(d_comp_, comp_of_block_.data(), nbk * sizeof(int), cudaMemcpyHostToDevice));
    d_stc_ = dalloc<FState>(ncomp_);
    d_cpart_ = dalloc<double>((size_t)nchunks_ * 2);
    d_ccnt_ = dalloc<unsigned>(ncomp_);
    CK(cudaMemsetAsync(d_ccnt_, 0, ncomp_ * sizeof(unsigned), stream_));
    CK(cudaMallocHost(&h_stc_, ncomp_ * sizeof(FState)));
  }
  levels_.resize(tt.max_level + 1);
  nonleaf_.resize(tt.max_level + 1);
  level_blocks_.resize(tt.max_level + 1);
  nonleaf_blocks_.resize(tt.max_level + 1);
  for (int l = 1; l <= tt.max_level; l++) {
    level_blocks_[l] = t.levels[l];
    for (int b : t.levels[l])
      if (tt.node_type[b] != kNodeLeaf) nonleaf_blocks_[l].push_back(b);
    for (int k = 0; k < 2; k++) {
      const std::vector<int> &v = k == 0 ? level_blocks_[l] : nonleaf_blocks_[l];
      DevList &dl = k == 0 ? levels_[l] : nonleaf_[l];
      dl.n = (int)v.size();
      dl.blocks = dalloc<int>(v.size());
      if (!v.empty()) CK(cudaMemcpy(dl.blocks, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice));
      // level lists: parent * 8 + which_child; non-leaf lists: children
      std::vector<int> lk;
      for (int b : v) {
        if (k == 0) lk.push_back(tt.parent[b] >= 0 ? tt.parent[b] * 8 + tt.which_child[b] : -1);
        else
          for (int q = 0; q < 8; q++) lk.push_back(tt.child[b * 8 + q]);
      }
      dl.links = dalloc<int>(lk.size());
      if (!lk.empty()) CK(cudaMemcpy(dl.links, lk.data(), lk.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
  }

  for (int d = 0; d < nd; d++) {
    d_bcoef_[d] = dalloc<double>((size_t)nbk * nfb_);
    d_afrac_[d] = dalloc<double>((size_t)nbk * nfb_);
    d_tff_[d] = dalloc<double>((size_t)nbk * nfb_);
  }
  d_vf_ = dalloc<double>((size_t)nbk * ncell_);
  for (int v = 0; v < kNumVec; v++) {
    vec_[v] = dalloc<double>((size_t)nbk * ncell_);
    if (!vec_[v]) {
      fail("out of device memory");
      return;
    }
  }
  d_red_ = dalloc<double>(kRedBlocks + 8);
  d_counter_ = dalloc<unsigned>(4);
  CK(cudaMallocHost(&h_red_, 8 * sizeof(double)));

  topo_.ndim = nd;
  topo_.nb = nb;
  topo_.lnb = (nb & (nb - 1)) == 0 ? __builtin_ctz((unsigned)nb) : -1;
  topo_.ncell = ncell_;
  topo_.nfb = nfb_;
  topo_.nblocks = nbk;
  topo_.neighbor = d_neighbor_;
  topo_.child = d_child_;
  topo_.parent = d_parent_;
  topo_.which_child = d_wc_;
  topo_.fc_neigh = d_fc_neigh_;
  topo_.bc_type = d_bc_type_;
  topo_.err = d_err_;

  c64_.geom = d_geom_;
  for (int d = 0; d < 3; d++) {
    c64_.tff[d] = d_tff_[d];
    c64_.bcoef[d] = d_bcoef_[d];
    c64_.afrac[d] = d_afrac_[d];
  }
  c64_.vf = d_vf_;
  // physical faces without setBC behave as Dirichlet-0 in the reference's
  // release build (src/SayakaMacOperator.cpp:1142-1151); start from that
  for (int b = 0; b < nbk; b++)
    for (int f = 0; f < 2 * nd; f++)
      if (tt.neighbor[b * 6 + f] <= kPhysBndry) bc_type_[b * 6 + f] = kBCDirichlet;
  CK(cudaMemcpy(d_bc_type_, bc_type_.data(), (size_t)nbk * 6 * sizeof(int), cudaMemcpyHostToDevice));
  set_scalars(0.0, 1.0);
}

MacGpu::~MacGpu() {
  auto fr = [](void *p) {
    if (p) dev_free(p);
  };
  for (auto &t : towers_) {
    fr(t.all.blocks);
    fr(t.all.ftypes);
    fr(t.par.blocks);
    fr(t.par.ftypes);
    fr(t.all.hx);
    fr(t.par.hx);
  }
  for (auto &l : levels_) {
    fr(l.blocks);
    fr(l.links);
  }
  for (auto &l : nonleaf_) {
    fr(l.blocks);
    fr(l.links);
  }
  fr(d_neighbor_);
  fr(d_child_);
  fr(d_parent_);
  fr(d_wc_);
  fr(d_fc_neigh_);
  fr(d_bc_type_);
  fr(d_err_);
  fr(d_geom_);
  for (int d = 0; d < 3; d++) {
    fr(d_bcoef_[d]);
    fr(d_afrac_[d]);
    fr(d_tff_[d]);
  }
  fr(d_vf_);
  for (auto *v : vec_) fr(v);
  fr(d_red_);
  fr(d_counter_);
  for (int d = 0; d < 3; d++) {
    fr(d_tff32_[d]);
    fr(d_bcoef32_[d]);
    fr(d_afrac32_[d]);
  }
  fr(d_vf32_);
  fr(d_geom32_);
  fr(d_resid32_);
  fr(d_corr32_);
  fr(d_corr32b_);
  fr(d_corr64b_);
  fr(tlc_.blocks);
  fr(tlc_.ftypes);
  fr(tlc_.hx);
  fr(d_chunk_);
  fr(d_comp_);
  fr(d_stc_);
  fr(d_cpart_);
  fr(d_ccnt_);
  if (h_stc_) cudaFreeHost(h_stc_);
  fr(d_st_);
  fr(d_part_);
  fr(d_opP_);
  for (auto &q : d_sfac_) fr(q);
  for (auto &q : d_pfac_) fr(q);
  for (auto &q : d_face_) fr(q);
  learned_free();
  fr(d_opS_);
  fr(d_opP2_);
  fr(d_opS2_);
  fr(d_uni2_);
  free_coef_lists();
  fr(d_uni64_);
  fr(d_uni32_);
  fr(d_cnt_);
  bottom_free();
  fr(d_phases_);
  fr(d_bar_);
  if (h_st_) cudaFreeHost(h_st_);
  if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
  if (graph_) cudaGraphDestroy(graph_);
  if (h_red_) cudaFreeHost(h_red_);
  if (stream_) cudaStreamDestroy(stream_);
}

// ---------------------------------------------------------------------------
// block lists
BlockList MacGpu::tower_list(int L) const {
  const DevTower &t = towers_[L];
  BlockList r{t.all.blocks, t.all.ftypes, t.all.n};
  r.hx = t.all.hx;
  return attach(r);
}
// lists built while a solve is recorded carry the per-problem states
BlockList MacGpu::attach(BlockList r) const {
  if (solve_lists_ && multi()) {
    r.comp = d_comp_;
    r.stc = d_stc_;
  }
  return r;
}
BlockList MacGpu::sublevel_list(int L, int l) const {
  const DevTower &t = towers_[L];
  const int b = t.begin[l], e = t.end[l];
  BlockList r{t.all.blocks + b, t.all.ftypes + b, e - b};
  r.hx = t.all.hx + (long)b * kHX;
  if (L < (int)d_sfac_.size() && d_sfac_[L]) {
    const long w = (long)t.all.n * ncell_;
    r.sa = d_sfac_[L] + (long)b * ncell_;
    r.ia = d_sfac_[L] + w + (long)b * ncell_;
  }
  return attach(r);
}
BlockList MacGpu::smooth_list(int L) const {
  BlockList r = tower_list(L);
  if (L < (int)d_sfac_.size() && d_sfac_[L]) {
    r.sa = d_sfac_[L];
    r.ia = d_sfac_[L] + (long)r.n * ncell_;
  }
  return r;
}
BlockList MacGpu::parity_list(int L, int g, bool skip_top) const {
  const DevTower &t = towers_[L];
  const int b = g == 0 ? (skip_top ? t.par_top : 0) : t.par_split;
  const int e = g == 0 ? t.par_split : t.par.n;
  BlockList r{t.par.blocks + b, t.par.ftypes + b, e - b};
  r.hx = t.par.hx + (long)b * kHX;
  if (L < (int)d_pfac_.size() && d_pfac_[L]) {
    const long w = (long)t.par.n * ncell_;
    r.sa = d_pfac_[L] + (long)b * ncell_;
    r.ia = d_pfac_[L] + w + (long)b * ncell_;
  }
  return attach(r);
}
BlockList MacGpu::level_list(int l) const {
  BlockList r{levels_[l].blocks, nullptr, levels_[l].n};
  r.links = levels_[l].links;
  return attach(r);
}
BlockList MacGpu::nonleaf_list(int l) const {
  BlockList r{nonleaf_[l].blocks, nullptr, nonleaf_[l].n};
  r.links = nonleaf_[l].links;
  return attach(r);
}

// ---------------------------------------------------------------------------
// coefficients
void MacGpu::set_scalars(double alpha, double beta) {
  alpha_ = alpha;
  beta_ = beta;
  c64_.alpha = alpha;
  c64_.beta = beta;
  if (!coef_uploaded_) {  // the initial coefficients (B = 1, fractions 1)
    init_coefs();
    coef_uploaded_ = true;
    return;
  }
  recompute_face_coef();
  coef_version_++;
}

void MacGpu::recompute_face_coef() {
  const double *b[3] = {d_bcoef_[0], d_bcoef_[1], d_bcoef_[2]};
  const double *a[3] = {d_afrac_[0], d_afrac_[1], d_afrac_[2]};
  double *o[3] = {d_tff_[0], d_tff_[1], d_tff_[2]};
  for (int d = tt_.ndim; d < 3; d++) {
    b[d] = b[0];
    a[d] = a[0];
    o[d] = o[0];
  }
  launch_face_coef<double>(topo_, d_geom_, b, a, beta_, o, stream_);
}

void MacGpu::set_bc_types(const int *bc6) {
  for (int b = 0; b < tt_.num_blocks; b++)
    for (int f = 0; f < 6; f++) {
      const bool phys = f < 2 * tt_.ndim && tt_.neighbor[b * 6 + f] <= kPhysBndry;
      bc_type_[b * 6 + f] = phys ? bc6[b * 6 + f] : -1;
    }
  CK(cudaMemcpy(d_bc_type_, bc_type_.data(), bc_type_.size() * sizeof(int), cudaMemcpyHostToDevice));
  coef_version_++;
}

void MacGpu::get_coef(int which, int dir, double *out) {
  pull_coefs();
  if (which == 0)
    std::memcpy(out, bcoef_[dir].data(), bcoef_[dir].size() * sizeof(double));
  else if (which == 1)
    std::memcpy(out, afrac_[dir].data(), afrac_[dir].size() * sizeof(double));
  else
    std::memcpy(out, vf_.data(), vf_.size() * sizeof(double));
}

// ---------------------------------------------------------------------------
// user vectors
void MacGpu::set_rhs(const double *all, bool dev) {
  CK(cudaMemcpyAsync(vec_[kRHS], all, (size_t)tt_.num_blocks * ncell_ * sizeof(double),
                     dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, stream_));
}
static TdLayout td_layout(int nd, int nb, int ncomp, int ngrow, int comp) {
  TdLayout L{nd, nb, ncomp, ngrow, comp, nb + 2l * ngrow, nd >= 2 ? nb + 2l * ngrow : 1, 0};
  L.cap = L.G0 * L.G1 * (nd == 3 ? nb + 2l * ngrow : 1);
  return L;
}
int MacGpu::set_field_td(const double *td, int ncomp, int ngrow, int comp, bool rhs) {
  const long total = (long)tt_.num_blocks * ncell_;
  k_td_gather<<<grid_for(total), kThreads, 0, stream_>>>(td_layout(tt_.ndim, tt_.nb, ncomp, ngrow, comp), total, ncell_,
                                                         td, vec_[rhs ? kRHS : kSOL]);
  CKR(cudaGetLastError(), 2);
  CKR(cudaStreamSynchronize(stream_), 2);
  return 0;
}
int MacGpu::get_sol_td(double *td, int ncomp, int ngrow, int comp) {
  const long total = (long)tt_.num_blocks * ncell_;
  k_td_scatter<<<grid_for(total), kThreads, 0, stream_>>>(td_layout(tt_.ndim, tt_.nb, ncomp, ngrow, comp), total,
                                                          ncell_, vec_[kSOL], td);
  CKR(cudaGetLastError(), 2);
  CKR(cudaStreamSynchronize(stream_), 2);
  return 0;
}
void MacGpu::set_sol(const double *all, bool dev) {
  CK(cudaMemcpyAsync(vec_[kSOL], all, (size_t)tt_.num_blocks * ncell_ * sizeof(double),
                     dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, stream_));
}
void MacGpu::zero_sol() { CK(cudaMemsetAsync(vec_[kSOL], 0, (size_t)tt_.num_blocks * ncell_ * sizeof(double), stream_)); }
void MacGpu::get_sol(double *all, bool dev) {
  // a failed copy or a failed kernel before it is reported (status
  // SAYAKA_CUDA_ERROR), never returned as stale data with status OK
  CK(cudaMemcpyAsync(all, vec_[kSOL], (size_t)tt_.num_blocks * ncell_ * sizeof(double),
                     dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
}

// ---------------------------------------------------------------------------
// vector ops over block lists
void MacGpu::vcopy(const BlockList &L, double *dst, const double *src) {
  const long w = (long)L.n * ncell_;
  if (w) k_copy<<<grid_for(w), kThreads, 0, stream_>>>(L, ncell_, dst, src);
}
void MacGpu::vzero(const BlockList &L, double *dst) {
  const long w = (long)L.n * ncell_;
  if (w) k_zero<<<grid_for(w), kThreads, 0, stream_>>>(L, ncell_, dst);
}
void MacGpu::vaxpby(const BlockList &L, double *out, double a, const double *x, double b, const double *y) {
  const long w = (long)L.n * ncell_;
  if (w) k_axpby<<<grid_for(w), kThreads, 0, stream_>>>(L, ncell_, out, a, x, b, y);
}
double MacGpu::vdot(const BlockList &L, const double *a, const double *b) {
  const long w = (long)L.n * ncell_;
  const int g = std::min<long>(kRedBlocks, std::max<long>(1, (w + kThreads - 1) / kThreads));
  k_reduce<0><<<g, kThreads, 0, stream_>>>(L, ncell_, a, b, d_red_, d_counter_, d_red_ + kRedBlocks);
  CKR(cudaMemcpyAsync(h_red_, d_red_ + kRedBlocks, sizeof(double), cudaMemcpyDeviceToHost, stream_), 0.0);
  CKR(cudaStreamSynchronize(stream_), 0.0);
  return h_red_[0];
}
double MacGpu::vnorm(const BlockList &L, const double *a) {
  const long w = (long)L.n * ncell_;
  const int g = std::min<long>(kRedBlocks, std::max<long>(1, (w + kThreads - 1) / kThreads));
  k_reduce<1><<<g, kThreads, 0, stream_>>>(L, ncell_, a, a, d_red_, d_counter_, d_red_ + kRedBlocks);
  CKR(cudaMemcpyAsync(h_red_, d_red_ + kRedBlocks, sizeof(double), cudaMemcpyDeviceToHost, stream_), 0.0);
  CKR(cudaStreamSynchronize(stream_), 0.0);
  return h_red_[0];
}

// ---------------------------------------------------------------------------
// MG building blocks (FP64)
void MacGpu::mg_apply(int L, double *out, const double *in, const double *rhs) {
  if (towers_[L].all.n == 0) return;
  launch_apply<double>(topo_, c64_, tower_list(L), in, out, rhs, nullptr, stream_);
}

// mg_smooth_level_usefill: fine -> coarse over the tower's levels, two
// colours each (src/SayakaMacOperator.cpp:1028-1112)
void MacGpu::mg_smooth(int L, double *phi, const double *rhs) {
  if (towers_[L].all.n == 0) return;
  for (int l = L; l >= 1; l--) {
    BlockList sl = sublevel_list(L, l);
    if (sl.n == 0) break;
    for (int rb = 0; rb < 2; rb++) launch_smooth<double>(topo_, c64_, sl, rb, phi, rhs, nullptr, stream_);
  }
}

void MacGpu::mg_restrict(int lc, double *phi) {
  if (lc >= tt_.max_level) return;
  if (levels_[lc].n == 0 || levels_[lc + 1].n == 0) return;
  launch_restrict<double>(topo_, c64_, nonleaf_list(lc), phi, nullptr, stream_);
}

void MacGpu::mg_prolong(int lf, double *phi) {
  if (lf <= 1 || levels_[lf].n == 0) return;
  launch_prolong<double>(topo_, c64_, level_list(lf), phi, nullptr, stream_);
}

// one V-cycle with zero initial guess: sol = M^-1 rhs on tower L
// (src/SayakaMacSolver.cpp:924-949 -> :245-374 with fixed_iter = 1)
void MacGpu::precond(int L, double *sol, const double *rhs) {
  BlockList TL = tower_list(L);
  // SOL = 0; RESID = rhs - L(0) = rhs on fluid cells
  k_masked_copy<<<grid_for((long)TL.n * ncell_), kThreads, 0, stream_>>>(TL, ncell_, d_vf_, vec_[kRESID], rhs);
  vzero(TL, vec_[kCORR]);
  for (int l = L; l >= 2; l--) mg_restrict(l - 1, vec_[kRESID]);
  const int rb = bottom_solve();
  if (rb != 0) {
    // bottom breakdown: the reference skips the up-sweep and returns SOL = 0
    vzero(TL, sol);
    return;
  }
  for (int l = 2; l <= L; l++) {
    mg_prolong(l, vec_[kCORR]);
    for (int s = 0; s < prm_.n_post; s++) mg_smooth(l, vec_[kCORR], vec_[kRESID]);
  }
  // SOL(=0) += CORR ; sol = SOL
  vaxpby(TL, sol, 1.0, vec_[kCORR], 0.0, vec_[kCORR]);
}

// mg_solve_bottom (src/SayakaMacSolver.cpp:164-242): CORR on tower(1) from
// RESID, unpreconditioned BiCGSTAB in its own buffers
int MacGpu::bottom_solve() {
  BlockList T1 = tower_list(1);
  vzero(T1, vec_[kCORR]);
  SolveInfo info;
  const int stat = bicgstab(1, vec_[kCORR], vec_[kRESID], prm_.bot_tol_rel, prm_.bot_tol_abs, prm_.bot_max_iter,
                            false, true, &info);
  return stat;
}

// BiCGSTAB of cg_solve_level (src/SayakaMacSolver.cpp:683-920)
int MacGpu::bicgstab(int L, double *sol, const double *rhs, double tol_rel, double tol_abs, int max_iter,
                     bool use_precond, bool bottom, SolveInfo *info) {
  BlockList TL = tower_list(L);
  double *X0 = vec_[bottom ? kBX0 : kX0], *X = vec_[bottom ? kBX : kX], *R = vec_[bottom ? kBR : kR];
  double *RHAT = vec_[bottom ? kBRHAT : kRHAT], *P = vec_[bottom ? kBP : kP];
  double *S = vec_[bottom ? kBS : kS], *V = vec_[bottom ? kBV : kV], *Tt = vec_[bottom ? kBT : kT];
  double *PHAT = bottom ? P : vec_[kPHAT], *SHAT = bottom ? S : vec_[kSHAT];
  if (L == 1) use_precond = false;

  vcopy(TL, X0, sol);
  mg_apply(L, R, X0, rhs);  // R = rhs - A x0 (masked)
  vcopy(TL, RHAT, R);
  vzero(TL, X);
  const double rnorm0 = vnorm(TL, R);
  info->rnorm0 = rnorm0;
  info->rnorm = rnorm0;
  info->iterations = 0;
  if (!err_.empty()) return -1;
  if (rnorm0 == 0) return 0;

  double rho1 = 0, alpha = 0, omega = 0;
  bool conv = false;
  int stat = 0, iter;
  for (iter = 1; iter <= max_iter; iter++) {
    const double rho = vdot(TL, RHAT, R);
    if (rho == 0) {
      stat = 1;
      break;
    }
    if (iter == 1) {
      vcopy(TL, P, R);
    } else {
      const double beta = (rho / rho1) * (alpha / omega);
      vaxpby(TL, P, 1.0, P, -omega, V);
      vaxpby(TL, P, 1.0, R, beta, P);
    }
    if (use_precond) precond(L, PHAT, P);
    mg_apply(L, V, use_precond ? PHAT : P, nullptr);
    alpha = vdot(TL, RHAT, V);
    if (alpha == 0) {
      stat = 1;
      break;
    }
    alpha = rho / alpha;
    vaxpby(TL, S, 1.0, R, -alpha, V);
    vaxpby(TL, X, 1.0, X, alpha, use_precond ? PHAT : P);
    double rnorm = vnorm(TL, S);
    info->rnorm = rnorm;
    if (rnorm < rnorm0 * tol_rel || rnorm < tol_abs) {
      conv = true;
      break;
    }
    if (use_precond) precond(L, SHAT, S);
    mg_apply(L, Tt, use_precond ? SHAT : S, nullptr);
    const double tds = vdot(TL, Tt, S);
    const double tdt = vdot(TL, Tt, Tt);
    if (tdt == 0) {
      stat = 1;
      break;
    }
    omega = tds / tdt;
    vaxpby(TL, X, 1.0, X, omega, use_precond ? SHAT : S);
    vaxpby(TL, R, 1.0, S, -omega, Tt);
    rnorm = vnorm(TL, R);
    info->rnorm = rnorm;
    if (prm_.verbose && !bottom) fprintf(stderr, "bicgstab iter=%d |r|=%.6e\n", iter, rnorm);
    if (rnorm < rnorm0 * tol_rel + tol_abs) {
      conv = true;
      break;
    }
    if (omega == 0) {
      stat = 1;
      break;
    }
    rho1 = rho;
    if (!err_.empty()) return -1;
  }
  info->iterations = std::min(iter, max_iter);
  if (conv) {
    vaxpby(TL, X0, 1.0, X0, 1.0, X);
    vcopy(TL, sol, X0);
  }
  info->status = stat ? 1 : (conv ? 0 : 2);
  return stat;
}

int MacGpu::cg_solve(SolveInfo *info) {
  if (prm_.bottom == 1 && prm_.use_mg_precond) return cg_solve_device(info);
  auto t0 = std::chrono::steady_clock::now();
  const int stat = bicgstab(finest_, vec_[kSOL], vec_[kRHS], prm_.tol_rel, prm_.tol_abs, prm_.max_iter,
                            prm_.use_mg_precond != 0, false, info);
  cudaStreamSynchronize(stream_);
  info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (!err_.empty()) return -1;
  return stat;
}

// mg_solve (src/SayakaMacSolver.cpp:43-162): stand-alone V-cycles on the
// finest tower with the reference's arithmetic (host-driven, the bottom by
// BiCGSTAB with the bottom tolerances): RESID = RHS - L(SOL), then per
// iteration CORR = 0, restriction of RESID to level 1, bottom solve,
// prolongation and post-smoothing up, SOL += CORR, RESID and its L-inf norm,
// until |r| < |r0| tol_rel + tol_abs or max_iter.  The reference exits on a
// bottom breakdown (status BREAKDOWN here) and runs its preconditioner's
// fixed V-cycle count instead of max_iter once a preconditioned cg_solve set
// it; this entry point always follows max_iter and the tolerance.
int MacGpu::mg_solve(SolveInfo *info) {
  auto t0 = std::chrono::steady_clock::now();
  const int L = finest_;
  const BlockList TL = tower_list(L);
  const size_t n = (size_t)tt_.num_blocks * ncell_;
  double *SOL = vec_[kSOL], *RHS = vec_[kRHS], *RES = vec_[kRESID], *COR = vec_[kCORR];
  mg_apply(L, RES, SOL, RHS);
  const double r0 = vnorm(TL, RES);
  double rn = r0;
  int it = 0, conv = 0, stat = 0;
  for (it = 1; it <= prm_.max_iter && err_.empty(); it++) {
    CKR(cudaMemsetAsync(COR, 0, n * sizeof(double), stream_), -1);
    for (int l = L; l >= 2; l--) mg_restrict(l - 1, RES);
    if (bottom_solve() != 0) {
      stat = 1;
      break;
    }
    for (int l = 2; l <= L; l++) {
      mg_prolong(l, COR);
      for (int s = 0; s < prm_.n_post; s++) mg_smooth(l, COR, RES);
    }
    vaxpby(TL, SOL, 1.0, SOL, 1.0, COR);
    mg_apply(L, RES, SOL, RHS);
    rn = vnorm(TL, RES);
    if (rn < r0 * prm_.tol_rel + prm_.tol_abs) {
      conv = 1;
      break;
    }
  }
  CKR(cudaStreamSynchronize(stream_), -1);
  info->iterations = std::min(it, prm_.max_iter);
  info->rnorm0 = r0;
  info->rnorm = rn;
  info->status = stat ? 1 : (conv ? 0 : 2);
  info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return err_.empty() ? 0 : -1;
}

// relax_solve (src/SayakaMacSolver.cpp:377-452): red-black Gauss-Seidel
// sweeps of the finest tower (mg_smooth_level) on SOL with RHS, the
// residual's L-inf norm after each, until |r| < |r0| tol_rel + tol_abs or
// max_iter (the reference returns 0 either way; status 2 here when the
// tolerance was not met)
int MacGpu::relax_solve(SolveInfo *info) {
  auto t0 = std::chrono::steady_clock::now();
  const int L = finest_;
  const BlockList TL = tower_list(L);
  double *SOL = vec_[kSOL], *RHS = vec_[kRHS], *RES = vec_[kRESID];
  mg_apply(L, RES, SOL, RHS);
  const double r0 = vnorm(TL, RES);
  double rn = r0;
  int it = 0, conv = 0;
  for (it = 1; it <= prm_.max_iter && err_.empty(); it++) {
    mg_smooth(L, SOL, RHS);
    mg_apply(L, RES, SOL, RHS);
    rn = vnorm(TL, RES);
    if (rn < r0 * prm_.tol_rel + prm_.tol_abs) {
      conv = 1;
      break;
    }
  }
  CKR(cudaStreamSynchronize(stream_), -1);
  info->iterations = std::min(it, prm_.max_iter);
  info->rnorm0 = r0;
  info->rnorm = rn;
  info->status = conv ? 0 : 2;
  info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return err_.empty() ? 0 : -1;
}

// ---------------------------------------------------------------------------
// parity hooks (compact all-block arrays on the host)
void MacGpu::apply(int L, const double *x, double *y) {
  const size_t n = (size_t)tt_.num_blocks * ncell_;
  CK(cudaMemcpyAsync(vec_[kP], x, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
  CK(cudaMemsetAsync(vec_[kV], 0, n * sizeof(double), stream_));
  mg_apply(L, vec_[kV], vec_[kP], nullptr);
  CK(cudaMemcpyAsync(y, vec_[kV], n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
}
void MacGpu::residual(int L, const double *x, const double *rhs, double *r) {
  const size_t n = (size_t)tt_.num_blocks * ncell_;
  CK(cudaMemcpyAsync(vec_[kP], x, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
  CK(cudaMemcpyAsync(vec_[kS], rhs, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
  CK(cudaMemsetAsync(vec_[kT], 0, n * sizeof(double), stream_));
  mg_apply(L, vec_[kT], vec_[kP], vec_[kS]);
  CK(cudaMemcpyAsync(r, vec_[kT], n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
}
void MacGpu::smooth(int L, const double *phi, const double *rhs, double *out) {
  const size_t n = (size_t)tt_.num_blocks * ncell_;
  CK(cudaMemcpyAsync(vec_[kCORR], phi, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
  CK(cudaMemcpyAsync(vec_[kRESID], rhs, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
  mg_smooth(L, vec_[kCORR], vec_[kRESID]);
  CK(cudaMemcpyAsync(out, vec_[kCORR], n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
}
void MacGpu::restrict_sweep(const double *in, double *out) {
  const size_t n = (size_t)tt_.num_blocks * ncell_;
  CK(cudaMemcpyAsync(vec_[kRESID], in, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
  for (int l = finest_; l >= 2; l--) mg_restrict(l - 1, vec_[kRESID]);
  CK(cudaMemcpyAsync(out, vec_[kRESID], n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
}
void MacGpu::prolong_sweep(const double *in, double *out) {
  const size_t n = (size_t)tt_.num_blocks * ncell_;
  CK(cudaMemcpyAsync(vec_[kCORR], in, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
  for (int l = 2; l <= finest_; l++) mg_prolong(l, vec_[kCORR]);
  CK(cudaMemcpyAsync(out, vec_[kCORR], n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
}
void MacGpu::vcycle(const double *p, double *phat) {
  const size_t n = (size_t)tt_.num_blocks * ncell_;
  for (int v = 0; v < kNumVec; v++) CK(cudaMemsetAsync(vec_[v], 0, n * sizeof(double), stream_));
  CK(cudaMemcpyAsync(vec_[kP], p, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
  precond(finest_, vec_[kPHAT], vec_[kP]);
  CK(cudaMemcpyAsync(phat, vec_[kPHAT], n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
}
void MacGpu::flux(int dir, const double *phi, double *out) {
  const size_t n = (size_t)tt_.num_blocks * ncell_;
  const size_t nf = (size_t)tt_.num_blocks * nfb_;
  CK(cudaMemcpyAsync(vec_[kP], phi, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
  double *fl = nullptr;
  CK(dev_malloc(&fl, nf * sizeof(double)));
  CK(cudaMemsetAsync(fl, 0, nf * sizeof(double), stream_));
  launch_flux(topo_, c64_, tower_list(finest_), dir, vec_[kP], fl, stream_);
  CK(cudaMemcpyAsync(out, fl, nf * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
  dev_free(fl);
}
void MacGpu::fix_bc(const double *phig, int ng, double *rhs) {
  const int nd = tt_.ndim, G = tt_.nb + 2 * ng;
  const size_t gsz = (size_t)tt_.num_blocks * (nd == 3 ? (size_t)G * G * G : (size_t)G * G);
  const size_t n = (size_t)tt_.num_blocks * ncell_;
  double *dg = nullptr;
  CK(dev_malloc(&dg, gsz * sizeof(double)));
  CK(cudaMemcpyAsync(dg, phig, gsz * sizeof(double), cudaMemcpyHostToDevice, stream_));
  CK(cudaMemcpyAsync(vec_[kTMP], rhs, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
  launch_fix_bc(topo_, c64_, tower_list(finest_), dg, ng, vec_[kTMP], stream_);
  CK(cudaMemcpyAsync(rhs, vec_[kTMP], n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
  dev_free(dg);
}

}  // namespace sayaka_gb300
