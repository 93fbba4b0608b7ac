// The whole V-cycle preconditioner as ONE cooperative launch.
//
// On the benchmark trees every level of the V-cycle is small, so one launch
// per restriction level, per smoother level and colour, and per prolongation
// (about 70 per V-cycle) costs far more in launch and drain latency than in
// memory traffic.  Here the host compiles the V-cycle into a list of phases --
// restrict level l, dense bottom solve, prolong level l, red-black sweep of
// one level of tower l in one colour, copy out -- and a persistent
// cooperative kernel runs them with a grid-wide barrier between consecutive
// phases.  Every phase uses the same cell functions as the per-launch kernels
// (mac_stencil.cuh), so results are bit-identical to the launch-per-level
// V-cycle; fields written inside the kernel are read through L2.
//
// The barrier spins with a bound: a CTA that waits longer than the limit
// raises the error word and every CTA leaves the kernel at its next barrier;
// the host turns the word into a CUDA_ERROR status.  Cooperative launch
// guarantees that all CTAs are resident, so the bound is only a safety net.
#include <vector>

#include "dev_alloc.h"
#include "cuda_check.h"
#include "mac_solver.h"
#include "launch.cuh"
#include "mac_stencil.cuh"

namespace sayaka_gb300 {

namespace {

constexpr int kVT = 256;

// sense-by-generation grid barrier (bounded spin); returns false when the
// kernel must stop (timeout here or in another CTA)
__device__ __forceinline__ bool grid_barrier(unsigned *bar, int *err) {
  __shared__ int bail;
  __syncthreads();
  if (threadIdx.x == 0) {
    bail = 0;
    volatile unsigned *gen = bar + 1;
    const unsigned g = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(bar, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      unsigned long long spins = 0;
      while (*gen == g) {
        if (*(volatile int *)err) {
          bail = 1;
          break;
        }
        if (++spins > (1ull << 24)) {  // ~1 s: never expected with co-resident CTAs
          atomicExch(err, 1);
          bail = 1;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return bail == 0;
}

template <typename T, int ND>
__global__ void __launch_bounds__(kVT) k_vcycle_coop(Topo t, Coef<T> c, const VPhase *__restrict__ phases,
                                                     int nphases, T *resid, T *corr, double *out, BottomDev bd,
                                                     const FState *st, unsigned *bar, int *err) {
  using namespace stencil;
  if (st->done) return;
  extern __shared__ double rv[];
  const int ncell = t.ncell, nhalf = ncell >> 1;
  const long tid = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long nthr = (long)gridDim.x * blockDim.x;
  for (int ph = 0; ph < nphases; ph++) {
    const VPhase P = phases[ph];
    if (P.op == kPhaseRestrict) {
      const long total = (long)P.n * ncell;
      for (long it = tid; it < total; it += nthr) {
        const int p = (int)(it / ncell);
        restrict_cell<T, ND, true>(t, c, P.blocks[p], (int)(it - (long)p * ncell), resid);
      }
    } else if (P.op == kPhaseSmooth) {
      const long total = (long)P.n * nhalf;
      for (long it = tid; it < total; it += nthr) {
        const int p = (int)(it / nhalf);
        int ijk[3];
        color_cell<ND>((int)(it - (long)p * nhalf), t.nb, P.color, ijk);
        smooth_cell_fast<T, ND, true>(t, c, P.blocks[p], P.ftypes[p], ijk, corr, resid,
                                      P.sa ? P.sa + (long)p * ncell : nullptr,
                                      P.ia ? P.ia + (long)p * ncell : nullptr);
      }
    } else if (P.op == kPhaseProlong) {
      const long total = (long)P.n * ncell;
      for (long it = tid; it < total; it += nthr) {
        const int p = (int)(it / ncell);
        prolong_cell<T, ND, true>(t, c, P.blocks[p], (int)(it - (long)p * ncell), corr);
      }
    } else if (P.op == kPhaseBottom) {
      // dense FP64 solve of the level-1 components, tile by tile
      for (int tile = blockIdx.x; tile < bd.ntiles; tile += gridDim.x) bottom_tile<T, true>(bd, tile, resid, corr, rv);
    } else if (out) {  // kPhaseOut: phat (FP64) = 0 + corr over the tower
      const long total = (long)P.n * ncell;
      for (long it = tid; it < total; it += nthr) {
        const int p = (int)(it / ncell);
        const long q = (long)P.blocks[p] * ncell + (it - (long)p * ncell);
        out[q] = 0.0 + (double)__ldcg(&corr[q]);
      }
    }
    if (ph + 1 < nphases && !grid_barrier(bar, err)) return;
  }
}

}  // namespace

// phase program of the V-cycle on tower L (same order as vcycle_device)
void MacGpu::build_vcycle_program() {
  const int L = finest_;
  std::vector<VPhase> v;
  auto push = [&](int op, int color, const BlockList &bl) {
    if (bl.n <= 0 && op != kPhaseBottom) return;
    VPhase p{};
    p.op = op;
    p.color = color;
    p.n = bl.n;
    p.blocks = bl.blocks;
    p.ftypes = bl.ftypes;
    p.sa = bl.sa;
    p.ia = bl.ia;
    v.push_back(p);
  };
  const int LB = bot_level_;
  for (int l = L; l >= LB + 1; l--) {
    if (l - 1 >= tt_.max_level || levels_[l - 1].n == 0 || levels_[l].n == 0) continue;
    push(kPhaseRestrict, 0, nonleaf_list(l - 1));
  }
  n_down_ = (int)v.size();
  push(kPhaseBottom, 0, BlockList{nullptr, nullptr, 0});
  for (int l = LB + 1; l <= L; l++) {
    if (levels_[l].n == 0) continue;
    push(kPhaseProlong, 0, level_list(l));
    for (int s = 0; s < prm_.n_post; s++) {
      if (prm_.sublevel_order == 1) {
        for (int rb = 0; rb < 2; rb++)
          for (int g = 0; g < 2; g++) push(kPhaseSmooth, rb, parity_list(l, g, false));
        continue;
      }
      for (int ll = l; ll >= 1; ll--) {
        BlockList sl = sublevel_list(l, ll);
        if (sl.n == 0) break;
        for (int rb = 0; rb < 2; rb++) push(kPhaseSmooth, rb, sl);
      }
    }
  }
  push(kPhaseOut, 0, tower_list(L));
  if (d_phases_) dev_free(d_phases_);
  d_phases_ = nullptr;
  n_phases_ = (int)v.size();
  h_phases_ = v;
  CK(dev_malloc(&d_phases_, v.size() * sizeof(VPhase)));
  CK(cudaMemcpy(d_phases_, v.data(), v.size() * sizeof(VPhase), cudaMemcpyHostToDevice));
  if (!d_bar_) {
    CK(dev_malloc(&d_bar_, 4 * sizeof(unsigned)));
    CK(cudaMemsetAsync(d_bar_, 0, 4 * sizeof(unsigned), stream_));
  }
  program_npost_ = prm_.n_post;
  program_order_ = prm_.sublevel_order;
  program_bot_ = bot_level_;
}

template <typename T>
void MacGpu::vcycle_coop(T *resid, T *corr, const Coef<T> &c, double *out) {
  const size_t smem = (size_t)std::max(bot_.max_n, 1) * sizeof(double);
  const void *fn = tt_.ndim == 2 ? (const void *)k_vcycle_coop<T, 2> : (const void *)k_vcycle_coop<T, 3>;
  if (coop_grid_ <= 0) {
    if (smem > 48 * 1024) ensure_max_smem(fn, (int)smem);
    int per_sm = 0, dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kVT, smem);
    if (per_sm <= 0) {
      fail("cooperative V-cycle kernel cannot be resident");
      return;
    }
    coop_grid_ = nsm * std::min(per_sm, 2);
  }
  int *err = (int *)(d_bar_ + 2);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(coop_grid_);
  cfg.blockDim = dim3(kVT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream_;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const BottomDev bd = bot_;
  const VPhase *ph = d_phases_;
  const int np = n_phases_;
  const FState *st = d_st_;
  unsigned *bar = d_bar_;
  cudaError_t e;
  if (tt_.ndim == 2)
    e = cudaLaunchKernelEx(&cfg, k_vcycle_coop<T, 2>, topo_, c, ph, np, resid, corr, out, bd, st, bar, err);
  else
    e = cudaLaunchKernelEx(&cfg, k_vcycle_coop<T, 3>, topo_, c, ph, np, resid, corr, out, bd, st, bar, err);
  if (e != cudaSuccess) fail(std::string("cooperative V-cycle launch: ") + cudaGetErrorString(e));
}

template void MacGpu::vcycle_coop<float>(float *, float *, const Coef<float> &, double *);
template void MacGpu::vcycle_coop<double>(double *, double *, const Coef<double> &, double *);

}  // namespace sayaka_gb300

// ---------------------------------------------------------------------------
// V-cycle phases inside ONE thread-block cluster (up to 16 CTAs of 1024
// threads on 16 SMs).  Consecutive phases are separated by the hardware
// cluster barrier (barrier.cluster arrive.release / wait.acquire), which is
// far cheaper than a kernel boundary or a software grid barrier; the dense
// FP64 bottom solve runs as a separate full-GPU launch between the
// restriction program and the prolongation/smoothing program.
#include <cooperative_groups.h>

namespace sayaka_gb300 {

namespace {

constexpr int kCT = 1024;

template <typename T, int ND>
__global__ void __launch_bounds__(kCT, 1) k_vcycle_cluster(Topo t, Coef<T> c, const VPhase *__restrict__ phases,
                                                           int first, int last, T *resid, T *corr, double *out,
                                                           const FState *st) {
  using namespace stencil;
  namespace cg = cooperative_groups;
  if (st->done) return;
  cg::cluster_group cl = cg::this_cluster();
  const int ncell = t.ncell, nhalf = ncell >> 1;
  const long tid = (long)cl.block_rank() * blockDim.x + threadIdx.x;
  const long nthr = (long)cl.num_blocks() * blockDim.x;
  for (int ph = first; ph < last; ph++) {
    const VPhase P = phases[ph];
    if (P.op == kPhaseRestrict) {
      const long total = (long)P.n * ncell;
      for (long it = tid; it < total; it += nthr) {
        const int p = (int)(it / ncell);
        restrict_cell<T, ND, true>(t, c, P.blocks[p], (int)(it - (long)p * ncell), resid);
      }
    } else if (P.op == kPhaseSmooth) {
      const long total = (long)P.n * nhalf;
      for (long it = tid; it < total; it += nthr) {
        const int p = (int)(it / nhalf);
        int ijk[3];
        color_cell<ND>((int)(it - (long)p * nhalf), t.nb, P.color, ijk);
        smooth_cell_fast<T, ND, true>(t, c, P.blocks[p], P.ftypes[p], ijk, corr, resid,
                                      P.sa ? P.sa + (long)p * ncell : nullptr,
                                      P.ia ? P.ia + (long)p * ncell : nullptr);
      }
    } else if (P.op == kPhaseProlong) {
      const long total = (long)P.n * ncell;
      for (long it = tid; it < total; it += nthr) {
        const int p = (int)(it / ncell);
        prolong_cell<T, ND, true>(t, c, P.blocks[p], (int)(it - (long)p * ncell), corr);
      }
    } else if (P.op == kPhaseOut && out) {
      const long total = (long)P.n * ncell;
      for (long it = tid; it < total; it += nthr) {
        const int p = (int)(it / ncell);
        const long q = (long)P.blocks[p] * ncell + (it - (long)p * ncell);
        out[q] = 0.0 + (double)__ldcg(&corr[q]);
      }
    }
    if (ph + 1 < last) cl.sync();
  }
}

}  // namespace

template <typename T>
void MacGpu::vcycle_cluster(T *resid, T *corr, const Coef<T> &c, double *out) {
  auto fn = tt_.ndim == 2 ? k_vcycle_cluster<T, 2> : k_vcycle_cluster<T, 3>;
  if (cluster_size_ <= 0) {
    cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    for (int cs : {16, 8, 4, 2, 1}) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(cs);
      cfg.blockDim = dim3(kCT);
      cudaLaunchAttribute a[1];
      a[0].id = cudaLaunchAttributeClusterDimension;
      a[0].val.clusterDim.x = cs;
      a[0].val.clusterDim.y = 1;
      a[0].val.clusterDim.z = 1;
      cfg.attrs = a;
      cfg.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg) == cudaSuccess && nclusters >= 1) {
        cluster_size_ = cs;
        break;
      }
      cudaGetLastError();
    }
    if (cluster_size_ <= 0) {
      fail("no thread-block cluster fits the V-cycle kernel");
      return;
    }
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cluster_size_);
  cfg.blockDim = dim3(kCT);
  cfg.stream = stream_;
  cudaLaunchAttribute a[1];
  a[0].id = cudaLaunchAttributeClusterDimension;
  a[0].val.clusterDim.x = cluster_size_;
  a[0].val.clusterDim.y = 1;
  a[0].val.clusterDim.z = 1;
  cfg.attrs = a;
  cfg.numAttrs = 1;
  const VPhase *ph = d_phases_;
  const FState *st = d_st_;
  const int *guard = &d_st_->done;
  const bool pdl = prm_.pdl != 0;
  const long lim = prm_.cluster_cells;
  auto cells = [&](const VPhase &q) -> long {
    return q.op == kPhaseSmooth ? (long)q.n * (ncell_ / 2) : (long)q.n * ncell_;
  };
  auto small = [&](int i) { return h_phases_[i].op != kPhaseBottom && cells(h_phases_[i]) <= lim; };
  int i = 0;
  while (i < n_phases_) {
    if (small(i)) {  // a run of small phases: one cluster launch, cluster barriers in between
      int j = i + 1;
      while (j < n_phases_ && small(j)) j++;
      cudaError_t e = cudaLaunchKernelEx(&cfg, fn, topo_, c, ph, i, j, resid, corr, out, st);
      if (e != cudaSuccess) {
        fail(std::string("cluster V-cycle launch: ") + cudaGetErrorString(e));
        return;
      }
      i = j;
      continue;
    }
    const VPhase &P = h_phases_[i];
    const BlockList bl{P.blocks, P.ftypes, P.n, P.sa, P.ia};
    switch (P.op) {
      case kPhaseRestrict: launch_restrict<T>(topo_, c, bl, resid, guard, stream_, pdl); break;
      case kPhaseBottom: bottom_launch<T>(resid, corr); break;
      case kPhaseProlong: launch_prolong<T>(topo_, c, bl, corr, guard, stream_, pdl); break;
      case kPhaseSmooth: launch_rbgs<T>(topo_, c, bl, P.color, corr, resid, guard, stream_, pdl, rbgs_var<T>()); break;
      default:
        if (out) vc_out_launch<T>(bl, corr, out);
        break;
    }
    i++;
  }
}

template void MacGpu::vcycle_cluster<float>(float *, float *, const Coef<float> &, double *);
template void MacGpu::vcycle_cluster<double>(double *, double *, const Coef<double> &, double *);

}  // namespace sayaka_gb300
