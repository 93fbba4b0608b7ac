// Coefficient setup of the MAC solver on the device: the face coefficient B
// (setCoefB, src/SayakaMacCoef.cpp:36-76) and the immersed-boundary
// fractions (setIBFracByLS / calcIBFracByLS, src/SayakaMacIB.cpp:34-154, and
// fractions given directly), each followed by the reference's averaging:
//   1. FLUX_SYNC_AVG over the finest tower, levels finest .. 2
//      (src/SayakaTower.cpp:298-415 with src/SayakaInterpPatch.cpp:627-691):
//      (a) the fine faces of a FINE_CRSE face averaged into the parent's
//          face, (b) the parent's face copied into the CRSE_FINE face of the
//          coarse neighbour;
//   2. AVG restriction of cell data onto the non-leaf blocks, levels
//      finest-1 .. 1 (src/SayakaInterpPatch.cpp:398-444);
//   3. AVG restriction of face data onto the non-leaf blocks, levels
//      finest-1 .. 1 (src/SayakaFillPatch.cpp:401-447).
// Each level step is one launch over precomputed work lists (the tree is
// fixed for a handle), one thread per face or cell written; every value is
// summed in the reference's order, and where the reference writes a face
// twice (the middle face of a non-leaf block, from both children) the
// value written is that of its last write.  Nothing goes through the host:
// a coefficient change costs a few launches instead of host loops and a
// full re-upload.
#include <algorithm>
#include <cstring>

#include "dev_alloc.h"
#include "cuda_check.h"
#include "mac_device.h"
#include "mac_solver.h"
#include "tree.h"

namespace sayaka_gb300 {
namespace {

constexpr int kCT = 256;

__device__ __forceinline__ int face_at(int d, int i, int j, int k, int nb) {
  const int e0 = nb + (d == 0), e1 = nb + (d == 1);
  return i + e0 * (j + e1 * k);
}

struct Faces {
  double *f[3];
};

inline int cgrid(long work) {
  long g = (work + kCT - 1) / kCT;
  return (int)std::max(1l, std::min(g, 152l * 32));
}

// 1(a): items (b, f) of one level: b's face f is FINE_CRSE; its fine face
// values, 2^(nd-1) per parent face, averaged into the parent's face
__global__ void k_sync_up(int nd, int nb, int nfb, const int *__restrict__ items, int n, const int *__restrict__ parent,
                          const int *__restrict__ wc, Faces F, int dmask) {
  const int half = nb >> 1;
  const int per = nd == 3 ? half * half : half;
  const double scale = nd == 3 ? 0.25 : 0.5;
  const long total = (long)n * per;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int k = (int)(it / per), m = (int)(it - (long)k * per);
    const int b = items[2 * k], f = items[2 * k + 1];
    const int dir = f >> 1, side = f & 1;
    if (!((dmask >> dir) & 1)) continue;
    double *A = F.f[dir];
    const int P = parent[b], w = wc[b];
    int off[3] = {0, 0, 0};
    for (int q = 0; q < nd; q++) off[q] = ((w >> q) & 1) * half;
    const int t0 = dir == 0 ? 1 : 0, t1 = dir == 2 ? 1 : 2;
    int cc[3] = {0, 0, 0};
    cc[dir] = side == 0 ? off[dir] : off[dir] + half;
    cc[t0] = off[t0] + m % half;
    if (nd == 3) cc[t1] = off[t1] + m / half;
    double val = 0;
    for (int a1 = 0; a1 <= (nd == 3 ? 1 : 0); a1++)
      for (int a0 = 0; a0 <= 1; a0++) {
        int fi[3];
        fi[dir] = 2 * (cc[dir] - off[dir]);
        fi[t0] = 2 * (cc[t0] - off[t0]) + a0;
        if (nd == 3)
          fi[t1] = 2 * (cc[t1] - off[t1]) + a1;
        else
          fi[2] = 0;
        val += A[(long)b * nfb + face_at(dir, fi[0], fi[1], fi[2], nb)];
      }
    A[(long)P * nfb + face_at(dir, cc[0], cc[1], cc[2], nb)] = val * scale;
  }
}

// 1(b): items (b, f, nbr) of one level: b's face f faces the non-leaf
// block nbr; nbr's opposite face plane copied into b's face plane
__global__ void k_sync_copy(int nd, int nb, int nfb, const int *__restrict__ items, int n, Faces F, int dmask) {
  const int per = nd == 3 ? nb * nb : nb;
  const long total = (long)n * per;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int k = (int)(it / per), m = (int)(it - (long)k * per);
    const int b = items[3 * k], f = items[3 * k + 1], nbr = items[3 * k + 2];
    const int dir = f >> 1, side = f & 1;
    if (!((dmask >> dir) & 1)) continue;
    double *A = F.f[dir];
    const int t0 = dir == 0 ? 1 : 0, t1 = dir == 2 ? 1 : 2;
    int di[3] = {0, 0, 0}, si[3] = {0, 0, 0};
    di[t0] = si[t0] = m % nb;
    if (nd == 3) di[t1] = si[t1] = m / nb;
    di[dir] = side == 0 ? 0 : nb;
    si[dir] = side == 0 ? nb : 0;
    A[(long)b * nfb + face_at(dir, di[0], di[1], di[2], nb)] =
        A[(long)nbr * nfb + face_at(dir, si[0], si[1], si[2], nb)];
  }
}

// 3: every face of the non-leaf blocks of one level from their children;
// the middle face of direction d (written by both children in the
// reference, the upper one last) takes the upper child's value
__global__ void k_restrict_faces(int nd, int nb, int nfb, const int *__restrict__ blocks, int n,
                                 const int *__restrict__ child, Faces F, int dmask) {
  const int half = nb >> 1;
  const double scale = nd == 3 ? 0.25 : 0.5;
  const long total = (long)n * nd * nfb;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int k = (int)(it / ((long)nd * nfb));
    const int r = (int)(it - (long)k * nd * nfb);
    const int dir = r / nfb, fx = r - dir * nfb;
    if (!((dmask >> dir) & 1)) continue;
    double *A = F.f[dir];
    const int b = blocks[k];
    const int e0 = nb + (dir == 0), e1 = nb + (dir == 1);
    int ijk[3] = {fx % e0, (fx / e0) % e1, nd == 3 ? fx / (e0 * e1) : 0};
    int c = 0, off[3] = {0, 0, 0};
    for (int q = 0; q < nd; q++) {
      const int s = ijk[q] >= half ? 1 : 0;
      c |= s << q;
      off[q] = s * half;
    }
    const int C = child[b * 8 + c];
    const int t0 = dir == 0 ? 1 : 0, t1 = dir == 2 ? 1 : 2;
    double val = 0;
    for (int a1 = 0; a1 <= (nd == 3 ? 1 : 0); a1++)
      for (int a0 = 0; a0 <= 1; a0++) {
        int fi[3];
        fi[dir] = 2 * (ijk[dir] - off[dir]);
        fi[t0] = 2 * (ijk[t0] - off[t0]) + a0;
        if (nd == 3)
          fi[t1] = 2 * (ijk[t1] - off[t1]) + a1;
        else
          fi[2] = 0;
        val += A[(long)C * nfb + face_at(dir, fi[0], fi[1], fi[2], nb)];
      }
    A[(long)b * nfb + fx] = val * scale;
  }
}

// 2: every cell of the non-leaf blocks of one level, the average of its
// 2^nd children cells
__global__ void k_restrict_cells(int nd, int nb, int ncell, const int *__restrict__ blocks, int n,
                                 const int *__restrict__ child, double *V) {
  const int half = nb >> 1;
  const double wgt = 1.0 / (1 << nd);
  const long total = (long)n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int k = (int)(it / ncell), ci = (int)(it - (long)k * ncell);
    const int b = blocks[k];
    const int ijk[3] = {ci % nb, (ci / nb) % nb, nd == 3 ? ci / (nb * nb) : 0};
    int c = 0, fb[3] = {0, 0, 0};
    for (int q = 0; q < nd; q++) {
      const int s = ijk[q] >= half ? 1 : 0;
      c |= s << q;
      fb[q] = 2 * (ijk[q] - s * half);
    }
    const int C = child[b * 8 + c];
    double sum = 0;
    for (int kk = 0; kk < (nd == 3 ? 2 : 1); kk++)
      for (int jj = 0; jj < 2; jj++)
        for (int ii = 0; ii < 2; ii++)
          sum += V[(long)C * ncell + (fb[0] + ii) + nb * ((fb[1] + jj) + nb * (fb[2] + kk))];
    V[(long)b * ncell + ci] = sum * wgt;
  }
}

// binary fractions of the finest tower's blocks from a level set held with
// ng ghost layers (src/SayakaMacIB.cpp:99-154): a cell is fluid when
// ls > 0, a face open when the cells on both sides are
__global__ void k_ls_frac(int nd, int nb, int ncell, int nfb, const int *__restrict__ blocks, int n,
                          const double *__restrict__ ls, int ng, double *vf, Faces F) {
  const int G = nb + 2 * ng;
  const long gsz = nd == 3 ? (long)G * G * G : (long)G * G;
  const int per = ncell + nd * nfb;
  const long total = (long)n * per;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int k = (int)(it / per), r = (int)(it - (long)k * per);
    const int b = blocks[k];
    auto L = [&](int i, int j, int kz) {
      return ls[(long)b * gsz + (i + ng) + (long)G * ((j + ng) + (long)G * (nd == 3 ? kz + ng : 0))];
    };
    if (r < ncell) {
      const int i = r % nb, j = (r / nb) % nb, kz = nd == 3 ? r / (nb * nb) : 0;
      vf[(long)b * ncell + r] = L(i, j, kz) <= 0 ? 0.0 : 1.0;
      continue;
    }
    const int q = r - ncell, d = q / nfb, fx = q - d * nfb;
    const int e0 = nb + (d == 0), e1 = nb + (d == 1);
    const int i = fx % e0, j = (fx / e0) % e1, kz = nd == 3 ? fx / (e0 * e1) : 0;
    const int ii = d == 0, jj = d == 1, kk = d == 2;
    const bool solid = L(i - ii, j - jj, kz - kk) <= 0 || L(i, j, kz) <= 0;
    F.f[d][(long)b * nfb + fx] = solid ? 0.0 : 1.0;
  }
}

}  // namespace

// the work lists of the FLUX_SYNC_AVG steps, per level l = 2 .. finest:
// up[l] (b, f) for the FINE_CRSE faces of the finest tower's level-l
// blocks, copy[l] (b, f, nbr) for the faces of its level-(l-1) blocks that
// face a non-leaf block
void MacGpu::build_coef_lists() {
  if (coef_lists_) return;
  const int nd = tt_.ndim;
  const DevTower &tw = towers_[finest_];
  d_sync_up_.assign(finest_ + 1, nullptr);
  d_sync_copy_.assign(finest_ + 1, nullptr);
  n_sync_up_.assign(finest_ + 1, 0);
  n_sync_copy_.assign(finest_ + 1, 0);
  for (int l = finest_; l >= 2; l--) {
    std::vector<int> up, cp;
    for (int p = tw.begin[l]; p < tw.end[l]; p++) {
      const int b = tw.blocks[p];
      for (int f = 0; f < 2 * nd; f++) {
        const int nbr = tt_.neighbor[b * 6 + f];
        if (nbr < 0 && nbr > kPhysBndry) {
          up.push_back(b);
          up.push_back(f);
        }
      }
    }
    if (l - 1 < finest_)
      for (int p = tw.begin[l - 1]; p < tw.end[l - 1]; p++) {
        const int b = tw.blocks[p];
        for (int f = 0; f < 2 * nd; f++) {
          const int nbr = tt_.neighbor[b * 6 + f];
          if (nbr >= 0 && tt_.node_type[nbr] != kNodeLeaf) {
            cp.push_back(b);
            cp.push_back(f);
            cp.push_back(nbr);
          }
        }
      }
    auto up_dev = [&](const std::vector<int> &v, int *&d) {
      if (v.empty()) return;
      if (dev_malloc(&d, v.size() * sizeof(int)) != cudaSuccess) {
        fail("out of device memory (coefficient lists)");
        return;
      }
      CK(cudaMemcpy(d, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice));
    };
    up_dev(up, d_sync_up_[l]);
    up_dev(cp, d_sync_copy_[l]);
    n_sync_up_[l] = (int)up.size() / 2;
    n_sync_copy_[l] = (int)cp.size() / 3;
  }
  coef_lists_ = err_.empty();
}

void MacGpu::free_coef_lists() {
  for (auto *p : d_sync_up_)
    if (p) dev_free(p);
  for (auto *p : d_sync_copy_)
    if (p) dev_free(p);
  d_sync_up_.clear();
  d_sync_copy_.clear();
  if (d_ls_) dev_free(d_ls_);
  d_ls_ = nullptr;
  coef_lists_ = false;
}

// steps 1 and 3 on the face arrays of the directions in dmask, step 2 on
// the cell array V when given, in the reference's order (1, 2, 3)
void MacGpu::coef_average(int dmask, double *const F[3], double *V) {
  build_coef_lists();
  if (!err_.empty()) return;
  const int nd = tt_.ndim, nb = tt_.nb;
  Faces fa{{F[0], F[1], F[2]}};
  const int half = nb >> 1;
  const int up_per = nd == 3 ? half * half : half, cp_per = nd == 3 ? nb * nb : nb;
  if (dmask)
    for (int l = finest_; l >= 2; l--) {
      if (n_sync_up_[l])
        k_sync_up<<<cgrid((long)n_sync_up_[l] * up_per), kCT, 0, stream_>>>(nd, nb, nfb_, d_sync_up_[l], n_sync_up_[l],
                                                                             d_parent_, d_wc_, fa, dmask);
      if (n_sync_copy_[l])
        k_sync_copy<<<cgrid((long)n_sync_copy_[l] * cp_per), kCT, 0, stream_>>>(nd, nb, nfb_, d_sync_copy_[l],
                                                                                 n_sync_copy_[l], fa, dmask);
    }
  for (int l = finest_ - 1; l >= 1 && V; l--) {
    const int n = nonleaf_[l].n;
    if (n) k_restrict_cells<<<cgrid((long)n * ncell_), kCT, 0, stream_>>>(nd, nb, ncell_, nonleaf_[l].blocks, n,
                                                                          d_child_, V);
  }
  for (int l = finest_ - 1; l >= 1 && dmask; l--) {
    const int n = nonleaf_[l].n;
    if (n)
      k_restrict_faces<<<cgrid((long)n * nd * nfb_), kCT, 0, stream_>>>(nd, nb, nfb_, nonleaf_[l].blocks, n, d_child_,
                                                                        fa, dmask);
  }
  CK(cudaGetLastError());
}

// after the coefficient arrays changed on the device
void MacGpu::coef_changed() {
  recompute_face_coef();
  coef_version_++;
  host_coef_stale_ = true;
}

// setCoefB for direction dir from B on every block (the finest tower's
// blocks are taken; the averaging overwrites every other block's faces)
void MacGpu::set_coef_b_leaf(int dir, const double *face_all) {
  CK(cudaMemcpyAsync(d_bcoef_[dir], face_all, (size_t)tt_.num_blocks * nfb_ * sizeof(double), cudaMemcpyHostToDevice,
                     stream_));
  coef_average(1 << dir, d_bcoef_, nullptr);
  coef_changed();
}

// fractions given on every block (setIBFrac with the fine values): the
// finest tower's blocks are taken, then synchronised and restricted
void MacGpu::set_ib_frac_leaf(const double *vol_all, const double *const area_all[3]) {
  CK(cudaMemcpyAsync(d_vf_, vol_all, (size_t)tt_.num_blocks * ncell_ * sizeof(double), cudaMemcpyHostToDevice,
                     stream_));
  for (int d = 0; d < tt_.ndim; d++)
    CK(cudaMemcpyAsync(d_afrac_[d], area_all[d], (size_t)tt_.num_blocks * nfb_ * sizeof(double),
                       cudaMemcpyHostToDevice, stream_));
  coef_average((1 << tt_.ndim) - 1, d_afrac_, d_vf_);
  coef_changed();
}

// binary fractions from a level set (every block's grown box, ng >= 1
// ghost layers, ls <= 0 solid; host or, with dev, device memory), computed
// on the finest tower's blocks
void MacGpu::set_ib_frac_by_ls(const double *ls, int ng, bool dev) {
  const int nd = tt_.ndim, G = tt_.nb + 2 * ng;
  const size_t gsz = nd == 3 ? (size_t)G * G * G : (size_t)G * G;
  const size_t bytes = (size_t)tt_.num_blocks * gsz * sizeof(double);
  const double *src = ls;
  if (!dev) {  // staged in a device buffer kept for the next call
    if (bytes > ls_cap_) {
      CK(cudaStreamSynchronize(stream_));
      if (d_ls_) dev_free(d_ls_);
      d_ls_ = nullptr;
      ls_cap_ = 0;
      if (dev_malloc(&d_ls_, bytes) != cudaSuccess) {
        fail("out of device memory (level set)");
        return;
      }
      ls_cap_ = bytes;
    }
    CK(cudaMemcpyAsync(d_ls_, ls, bytes, cudaMemcpyHostToDevice, stream_));
    src = d_ls_;
  }
  const DevTower &tw = towers_[finest_];
  Faces fa{{d_afrac_[0], d_afrac_[1], d_afrac_[2]}};
  const long work = (long)tw.all.n * (ncell_ + nd * nfb_);
  if (work)
    k_ls_frac<<<cgrid(work), kCT, 0, stream_>>>(nd, tt_.nb, ncell_, nfb_, tw.all.blocks, tw.all.n, src, ng, d_vf_,
                                                fa);
  coef_average((1 << nd) - 1, d_afrac_, d_vf_);
  coef_changed();
}

// the host copies of B, the area and the volume fractions (allocated on
// first use) brought up to date with the device arrays
void MacGpu::pull_coefs() {
  const int nd = tt_.ndim;
  const size_t nf = (size_t)tt_.num_blocks * nfb_, nc = (size_t)tt_.num_blocks * ncell_;
  if (vf_.size() != nc) {
    for (int d = 0; d < 3; d++) {
      bcoef_[d].assign(d < nd ? nf : 1, 0.0);
      afrac_[d].assign(d < nd ? nf : 1, 0.0);
    }
    vf_.assign(nc, 0.0);
    host_coef_stale_ = true;
  }
  if (!host_coef_stale_) return;
  for (int d = 0; d < nd; d++) {
    CK(cudaMemcpyAsync(bcoef_[d].data(), d_bcoef_[d], nf * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    CK(cudaMemcpyAsync(afrac_[d].data(), d_afrac_[d], nf * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  }
  CK(cudaMemcpyAsync(vf_.data(), d_vf_, nc * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
  host_coef_stale_ = false;
}

void MacGpu::pull_block_coefs(const std::vector<int> &blocks, std::vector<double> &vf,
                              std::vector<double> (&bc)[3], std::vector<double> (&af)[3]) {
  const int nd = tt_.ndim, n = (int)blocks.size();
  vf.assign((size_t)n * ncell_, 0.0);
  for (int d = 0; d < 3; d++) {
    bc[d].assign(d < nd ? (size_t)n * nfb_ : 0, 0.0);
    af[d].assign(d < nd ? (size_t)n * nfb_ : 0, 0.0);
  }
  for (int p = 0; p < n; p++) {
    const size_t fo = (size_t)blocks[p] * nfb_, co = (size_t)blocks[p] * ncell_;
    for (int d = 0; d < nd; d++) {
      CK(cudaMemcpyAsync(&bc[d][(size_t)p * nfb_], d_bcoef_[d] + fo, nfb_ * sizeof(double), cudaMemcpyDeviceToHost,
                         stream_));
      CK(cudaMemcpyAsync(&af[d][(size_t)p * nfb_], d_afrac_[d] + fo, nfb_ * sizeof(double), cudaMemcpyDeviceToHost,
                         stream_));
    }
    CK(cudaMemcpyAsync(&vf[(size_t)p * ncell_], d_vf_ + co, ncell_ * sizeof(double), cudaMemcpyDeviceToHost,
                       stream_));
  }
  CK(cudaStreamSynchronize(stream_));
}

__global__ void k_fill(long n, double v, double *a) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) a[i] = v;
}

// B = 1 and every fraction 1, set on the device (no host upload)
void MacGpu::init_coefs() {
  const long nf = (long)tt_.num_blocks * nfb_, nc = (long)tt_.num_blocks * ncell_;
  for (int d = 0; d < tt_.ndim; d++) {
    k_fill<<<cgrid(nf), kCT, 0, stream_>>>(nf, 1.0, d_bcoef_[d]);
    k_fill<<<cgrid(nf), kCT, 0, stream_>>>(nf, 1.0, d_afrac_[d]);
  }
  k_fill<<<cgrid(nc), kCT, 0, stream_>>>(nc, 1.0, d_vf_);
  CK(cudaGetLastError());
  coef_changed();
}

}  // namespace sayaka_gb300
