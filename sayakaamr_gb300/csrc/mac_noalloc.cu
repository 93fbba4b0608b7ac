// Residual and its norms with no device allocation.
//
// Some callers cannot call cudaMalloc at the point where they need a residual
// norm: a time-stepping loop that runs inside a pre-sized memory pool (any
// allocation would break the pool's accounting or fail outright), a host
// callback that must not take the driver's allocation locks, or a code that
// checks convergence of an outer iteration between solver calls and has
// already handed all free memory to its own fields.  For them this file gives
// a variant of the fused residual kernel of the solve prologue (k_apply_red,
// mode 2: r = rhs - A x on a tower, |r|_inf and r.r) whose per-CTA partials
// and arrival counter live in a file-scope static device array instead of
// buffers from cudaMalloc.  The solver's own coefficient and table buffers,
// made when the solver was created, are only read.
//
// Limits and rules:
// * scratch: 2 doubles per CTA for at most kNaMaxCtas CTAs of kNaThreads
//   threads, one thread per cell, so towers of at most kNaMaxCtas*kNaThreads
//   cells; larger towers are rejected before any launch;
// * the arrival counter (the word after the partials) must be zero when a
//   launch starts: it is zero when the module loads, and the last CTA of every
//   launch sets it back to zero;
// * the scratch is shared by every call on the device: two calls in flight at
//   the same time (on different streams, host threads or solver handles)
//   race on it and give wrong norms, so callers serialise them (same stream,
//   or a synchronisation between them);
// * the first call on a device looks up the scratch address with
//   cudaGetSymbolAddress and loads the kernels' code; that first call should
//   come before any stream capture.
#include <mutex>
#include <string>

#include "mac_solver.h"
#include "mac_stencil.cuh"

namespace sayaka_gb300 {

namespace {

constexpr int kNaThreads = 256;
constexpr int kNaMaxCtas = 8192;                     // 2,097,152 cells
constexpr int kNaScratchDoubles = 2 * kNaMaxCtas + 32;  // partials, counter word, padding to 256 B
constexpr int kNaMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNaScratchDoubles];

__device__ __forceinline__ double na_wsum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// max that keeps NaN (fmax drops it): a residual with a NaN in it must
// report a NaN |r|_inf, as the device solve's norms do
__device__ __forceinline__ double na_max(double a, double b) { return (a != a || b != b) ? a + b : fmax(a, b); }
__device__ __forceinline__ double na_wmax(double v) {
  for (int o = 16; o > 0; o >>= 1) v = na_max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// one thread per cell of the tower: r = vf > 0 ? rhs - A x : 0, then
// out[0] = max |r|, out[1] = sum r*r (CTA partials combined in CTA order by
// the last CTA to arrive)
template <int ND>
__global__ void __launch_bounds__(kNaThreads) k_resid_norm_na(Topo t, Coef<double> c, BlockList L,
                                                              const double *__restrict__ x,
                                                              const double *__restrict__ rhs, double *__restrict__ r,
                                                              double *out, double *scratch) {
  __shared__ double sh[2][kNaThreads / 32];
  __shared__ bool last;
  double m = 0.0, s = 0.0;
  const int ncell = t.ncell;
  const long total = (long)L.n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell);
    const int ci = (int)(it - (long)p * ncell);
    const double ax = stencil::apply_cell<double, ND>(t, c, L.blocks[p], L.ftypes[p], ci, x);
    const long q = (long)L.blocks[p] * ncell + ci;
    const double rv = c.vf[q] > 0 ? rhs[q] - ax : 0.0;
    r[q] = rv;
    m = na_max(m, fabs(rv));
    s += rv * rv;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  m = na_wmax(m);
  s = na_wsum(s);
  if (lane == 0) {
    sh[0][w] = m;
    sh[1][w] = s;
  }
  __syncthreads();
  unsigned *counter = reinterpret_cast<unsigned *>(scratch + 2 * kNaMaxCtas);
  if (threadIdx.x == 0) {
    double bm = 0.0, bs = 0.0;
    for (int i = 0; i < kNaThreads / 32; i++) {
      bm = na_max(bm, sh[0][i]);
      bs += sh[1][i];
    }
    scratch[2 * blockIdx.x] = bm;
    scratch[2 * blockIdx.x + 1] = bs;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  m = 0.0;
  s = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    m = na_max(m, ((volatile double *)scratch)[2 * b]);
    s += ((volatile double *)scratch)[2 * b + 1];
  }
  __syncthreads();
  m = na_wmax(m);
  s = na_wsum(s);
  if (lane == 0) {
    sh[0][w] = m;
    sh[1][w] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double fm = 0.0, fs = 0.0;
    for (int i = 0; i < kNaThreads / 32; i++) {
      fm = na_max(fm, sh[0][i]);
      fs += sh[1][i];
    }
    out[0] = fm;
    out[1] = fs;
    atomicExch(counter, 0u);  // ready for the next launch
  }
}

std::mutex g_na_mutex;
double *g_na_ptr[kNaMaxDevices] = {};

// scratch address on the current device, looked up once per device
double *noalloc_scratch(std::string *why) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    *why = std::string("no current CUDA device: ") + cudaGetErrorString(e);
    return nullptr;
  }
  if (dev < 0 || dev >= kNaMaxDevices) {
    *why = "device index " + std::to_string(dev) + " beyond the " + std::to_string(kNaMaxDevices) +
           " devices the no-alloc residual tracks";
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_ptr[dev]) {
    double *p = nullptr;
    e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      *why = std::string("cudaGetSymbolAddress of the no-alloc scratch: ") + cudaGetErrorString(e);
      return nullptr;
    }
    // load the kernels' code now, so later calls only launch
    cudaFuncAttributes fa;
    for (const void *fn : {(const void *)k_resid_norm_na<2>, (const void *)k_resid_norm_na<3>}) {
      e = cudaFuncGetAttributes(&fa, fn);
      if (e != cudaSuccess) {
        *why = std::string("loading the no-alloc residual kernel: ") + cudaGetErrorString(e);
        return nullptr;
      }
    }
    g_na_ptr[dev] = p;
  }
  return g_na_ptr[dev];
}

}  // namespace

int MacGpu::residual_norm_noalloc(int L, const double *x, const double *rhs, double *r, double *out,
                                  cudaStream_t s, std::string *why) {
  if (L < 1 || L > finest_ || !x || !rhs || !r || !out) {
    *why = "residual_norm_noalloc: L must be in [1, finest level] and every pointer non-null";
    return 1;
  }
  const BlockList TL = tower_list(L);
  const long cells = (long)TL.n * ncell_;
  const long ctas = (cells + kNaThreads - 1) / kNaThreads;
  if (ctas > kNaMaxCtas) {
    *why = "residual_norm_noalloc: tower " + std::to_string(L) + " has " + std::to_string(cells) +
           " cells; the static scratch holds partials for " + std::to_string(kNaMaxCtas) + " CTAs of " +
           std::to_string(kNaThreads) + " threads, at most " + std::to_string((long)kNaMaxCtas * kNaThreads) +
           " cells";
    return 1;
  }
  double *scratch = noalloc_scratch(why);
  if (!scratch) return 2;
  const int grid = (int)std::max<long>(1, ctas);
  if (tt_.ndim == 2)
    k_resid_norm_na<2><<<grid, kNaThreads, 0, s>>>(topo_, c64_, TL, x, rhs, r, out, scratch);
  else
    k_resid_norm_na<3><<<grid, kNaThreads, 0, s>>>(topo_, c64_, TL, x, rhs, r, out, scratch);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    *why = std::string("residual_norm_noalloc launch: ") + cudaGetErrorString(e);
    return 2;
  }
  return 0;
}

}  // namespace sayaka_gb300
