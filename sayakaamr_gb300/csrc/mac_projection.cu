// The steps of a projection method on either side of the pressure solve,
// on the device:
//  * before: the solve's right-hand side from the face velocity,
//      rhs = sum_d (scale/dh_d) * (w_d u_d(i+1) - w_d u_d(i)),
//    scale = -1/dt in src/Test7.h:587-609 (calc_pres_rhs_block), 1 with the
//    optional face weight w = 1/rho in src/Test6.h:798-830
//    (calc_block_rhs_value); every block, accumulated over d from 0 in that
//    order, so the result is the reference's bit for bit;
//  * after: the velocity correction of src/Test7.h:634-645 (corr_vel),
//      u_dir += dt * mg_flux_level(finest, dir, p)
//    on the finest tower's blocks (TreeData::AddEqual over the valid faces),
//    with p the solver's solution, which stays on the device.
#include "dev_alloc.h"
#include "cuda_check.h"
#include "mac_solver.h"
#include "mac_stencil.cuh"

namespace sayaka_gb300 {

namespace {

constexpr int kPT = 256;

struct FaceSet {
  const double *u[3];
  const double *w[3];  // all null: no weighting
};

template <int ND>
__global__ void __launch_bounds__(kPT) k_div_rhs(Topo t, const double *__restrict__ geom, FaceSet fs, double scale,
                                               double *__restrict__ rhs) {
  using namespace stencil;
  const int total = t.nblocks * t.ncell;
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < total; it += gridDim.x * blockDim.x) {
    const int b = it / t.ncell, ci = it - b * t.ncell;
    int ijk[3];
    decode<ND>(ci, t.nb, ijk);
    double acc = 0.0;
#pragma unroll
    for (int d = 0; d < ND; d++) {
      const long fb = (long)b * t.nfb;
      const long fl = fb + face_index(d, ijk, 0, t.nb), fr = fb + face_index(d, ijk, 1, t.nb);
      double ul = fs.u[d][fl], ur = fs.u[d][fr];
      if (fs.w[d]) {
        ul *= fs.w[d][fl];
        ur *= fs.w[d][fr];
      }
      acc += scale / geom[b * 8 + d] * (ur - ul);
    }
    rhs[it] = acc;
  }
}

// u += dt * flux on every face of the list's blocks
__global__ void __launch_bounds__(kPT) k_face_axpy(BlockList L, int nfb, double dt, const double *__restrict__ flux,
                                                 double *__restrict__ u) {
  const int total = L.n * nfb;
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < total; it += gridDim.x * blockDim.x) {
    const int p = it / nfb;
    const long q = (long)L.blocks[p] * nfb + (it - p * nfb);
    u[q] += dt * flux[q];
  }
}

inline int pgrid(long work) { return (int)std::max<long>(1, std::min<long>((work + kPT - 1) / kPT, 152 * 32)); }

}  // namespace

double *MacGpu::face_scratch(int k) {
  if ((int)d_face_.size() < 7) d_face_.resize(7, nullptr);
  if (!d_face_[k]) {
    const size_t nf = (size_t)tt_.num_blocks * nfb_;
    if (dev_malloc(&d_face_[k], nf * sizeof(double)) != cudaSuccess) {
      d_face_[k] = nullptr;
      fail("out of device memory (face fields)");
    }
  }
  return d_face_[k];
}

void MacGpu::rhs_from_div(const double *const *u_all, const double *const *w_all, double scale) {
  const size_t nf = (size_t)tt_.num_blocks * nfb_;
  FaceSet fs{};
  for (int d = 0; d < tt_.ndim; d++) {
    double *du = face_scratch(d);
    if (!du) return;
    CK(cudaMemcpyAsync(du, u_all[d], nf * sizeof(double), cudaMemcpyHostToDevice, stream_));
    fs.u[d] = du;
    if (w_all) {
      double *dw = face_scratch(3 + d);
      if (!dw) return;
      CK(cudaMemcpyAsync(dw, w_all[d], nf * sizeof(double), cudaMemcpyHostToDevice, stream_));
      fs.w[d] = dw;
    }
  }
  const long w = (long)tt_.num_blocks * ncell_;
  if (tt_.ndim == 2)
    k_div_rhs<2><<<pgrid(w), kPT, 0, stream_>>>(topo_, d_geom_, fs, scale, vec_[kRHS]);
  else
    k_div_rhs<3><<<pgrid(w), kPT, 0, stream_>>>(topo_, d_geom_, fs, scale, vec_[kRHS]);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(stream_));
}

void MacGpu::correct_vel(int dir, double dt, double *u_all) {
  const size_t nf = (size_t)tt_.num_blocks * nfb_;
  double *fl = face_scratch(6), *du = face_scratch(0);
  if (!fl || !du) return;
  const BlockList TL = tower_list(finest_);
  launch_flux(topo_, c64_, TL, dir, vec_[kSOL], fl, stream_);
  CK(cudaMemcpyAsync(du, u_all, nf * sizeof(double), cudaMemcpyHostToDevice, stream_));
  k_face_axpy<<<pgrid((long)TL.n * nfb_), kPT, 0, stream_>>>(TL, nfb_, dt, fl, du);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(u_all, du, nf * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  CK(cudaStreamSynchronize(stream_));
}

void MacGpu::get_rhs(double *all) {
  CK(cudaMemcpyAsync(all, vec_[kRHS], (size_t)tt_.num_blocks * ncell_ * sizeof(double), cudaMemcpyDeviceToHost,
                     stream_));
  CK(cudaStreamSynchronize(stream_));
}

}  // namespace sayaka_gb300
