// Learned block correction of the device solve's FP32 V-cycle (2D blocks of
// 8x8 or 16x16 cells): feature assembly, FP32 training forward/backward,
// Adam, BF16 tensor-core inference, and the collection of training pairs from
// the plain solver's own iterates.  The network and its inputs are described
// in mac_learned.h.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "dev_alloc.h"
#include "cuda_check.h"
#include "mac_learned.h"
#include "mac_solver.h"
#include "mac_stencil.cuh"
#include "launch.cuh"

namespace sayaka_gb300 {

using namespace learned;

namespace {

__device__ __forceinline__ float wmaxf(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float wsumf(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide max over NC threads (NC a multiple of 32)
template <int NC>
__device__ __forceinline__ float block_max(float v, float *red) {
  v = wmaxf(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float m = 0.f;
  for (int i = 0; i < NC / 32; i++) m = fmaxf(m, red[i]);
  __syncthreads();
  return m;
}

// block-wide sum (fixed order over warps)
template <int NC>
__device__ __forceinline__ float block_sum(float v, float *red) {
  v = wsumf(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float m = 0.f;
  for (int i = 0; i < NC / 32; i++) m += red[i];
  __syncthreads();
  return m;
}

// v minus its least-squares fit by {1, x, y} over the block (the basis is
// orthogonal on the full nb x nb grid): the block-local part of a field,
// with the block's constant and linear trend left to the V-cycle
template <int NB>
__device__ __forceinline__ float local_part(float v, float *red) {
  constexpr int NC = NB * NB;
  const float xi = (float)(threadIdx.x % NB) - 0.5f * (NB - 1), yj = (float)(threadIdx.x / NB) - 0.5f * (NB - 1);
  const float sxx = (float)NB * (float)(NB * (NB * NB - 1)) / 12.f;  // sum of xi^2 over the block
  const float a0 = block_sum<NC>(v, red) / (float)NC;
  const float a1 = block_sum<NC>(v * xi, red) / sxx;
  const float a2 = block_sum<NC>(v * yj, red) / sxx;
  return v - a0 - a1 * xi - a2 * yj;
}

// input features of one cell: r1/s, log10(B averaged over the cell's faces)/3, vf
template <int NB>
__device__ __forceinline__ void cell_features(const Topo &t, const Coef<float> &c, int b, int ci, float r1, float s,
                                              float *f) {
  const int i = ci % NB, j = ci / NB;
  const long fb = (long)b * t.nfb;
  const float bx = c.bcoef[0][fb + i + (NB + 1) * j] + c.bcoef[0][fb + i + 1 + (NB + 1) * j];
  const float by = c.bcoef[1][fb + i + NB * j] + c.bcoef[1][fb + i + NB * (j + 1)];
  const float bavg = 0.25f * (bx + by);
  f[0] = r1 / s;
  f[1] = log10f(fmaxf(bavg, 1e-12f)) * (1.0f / 3.0f);
  f[2] = c.vf[(long)b * NB * NB + ci];
}

// ---- training pairs: the features of r1 and, per block, the data of the
// block-local operator the loss uses: aux = [sa][dv*vf][x-face T][y-face T]
template <int NB>
__global__ void k_nn_pairs(Topo t, Coef<float> c, BlockList L, const float *__restrict__ r1,
                           const float *__restrict__ err, const double *__restrict__ sa, float *feat, float *aux,
                           int off, int stride) {
  constexpr int NC = NB * NB, NF = (NB + 1) * NB, AUXN = 3 * NC + 2 * NF;
  __shared__ float red[NC / 32];
  // sample blockIdx.x is list entry off + blockIdx.x * stride
  const int p = off + blockIdx.x * stride, ci = threadIdx.x, o = blockIdx.x;
  const int b = L.blocks[p];
  const long q = (long)b * NC + ci;
  const float rv = r1[q];
  const float m = block_max<NC>(fabsf(rv), red);
  const float s = m > 0.f ? m : 1.f;
  float f[3];
  cell_features<NB>(t, c, b, ci, rv, s, f);
  for (int k = 0; k < 3; k++) feat[((long)o * 3 + k) * NC + ci] = f[k];
  float *ax = aux + (long)o * AUXN;
  ax[ci] = (float)sa[(long)p * NC + ci];
  ax[NC + ci] = c.geom[b * 8 + 6] * c.vf[q];
  for (int k = threadIdx.x; k < NF; k += blockDim.x) {
    ax[2 * NC + k] = c.tff[0][(long)b * t.nfb + k];
    ax[2 * NC + NF + k] = c.tff[1][(long)b * t.nfb + k];
  }
  // the error the V-cycle left (x* - x - z), block-local part, in units of s
  ax[2 * NC + 2 * NF + ci] = local_part<NB>(c.vf[q] > 0.f ? err[q] / s : 0.f, red);
}

// (K u)_c = sum over the cell's faces of T_f (u_c - u_nb), u = 0 outside the
// block (u in a padded tile with a zero halo); tx [j][i+s], ty [j+s][i]
template <int NB>
__device__ __forceinline__ float local_K(const float *u, const float *tx, const float *ty, int i, int j) {
  constexpr int P = NB + 2;
  const int pc = (j + 1) * P + (i + 1);
  const float uc = u[pc];
  return tx[i + (NB + 1) * j] * (uc - u[pc - 1]) + tx[i + 1 + (NB + 1) * j] * (uc - u[pc + 1]) +
         ty[i + NB * j] * (uc - u[pc - P]) + ty[i + NB * (j + 1)] * (uc - u[pc + P]);
}

// ---- FP32 forward for training: activations and the loss gradient, for
// the correction u = sa * P(y) of one block.  Loss 0 (residual): the
// residual the correction leaves under the block-local operator A = D^-1 K
// (K symmetric: face coefficients T, zero outside the block; D = dv*vf):
//   L = inv_norm * sum (r1/s - A u)^2,
// dL/du = K (D^-1 g) with g = -2 inv_norm (r1/s - A u), dL/dy = P(sa dL/du).
// Loss 1 (error): the distance to the block-local part of the error the
// V-cycle left, e = P(x* - x - z) / s (stored with the pair):
//   L = inv_norm * sum (u - e)^2,  dL/dy = P(sa * 2 inv_norm (u - e)).
template <int NB>
__global__ void __launch_bounds__(NB *NB) k_nn_fwd(const float *__restrict__ W, const float *__restrict__ feat,
                                                   const float *__restrict__ aux, const int *__restrict__ idx,
                                                   float *h1g, float *h2g, float *dyg, float *loss, float inv_norm,
                                                   int mode) {
  constexpr int NC = NB * NB, P = NB + 2, PP = P * P, NF = (NB + 1) * NB, AUXN = 3 * NC + 2 * NF;
  extern __shared__ float sm[];
  float *x0 = sm;             // [3][P][P]
  float *h1 = x0 + 3 * PP;    // [32][P][P]
  float *h2 = h1 + kC * PP;   // [32][P][P]
  float *w = h2 + kC * PP;    // [kNParam]
  float *ax = w + kNParam;    // [AUXN]
  float *ut = ax + AUXN;      // [P][P] u, then D^-1 g
  __shared__ float red[NC / 32];
  const int s = idx[blockIdx.x];
  const int ci = threadIdx.x, i = ci % NB, j = ci / NB, pc = (j + 1) * P + (i + 1);
  for (int k = threadIdx.x; k < kNParam; k += blockDim.x) w[k] = W[k];
  for (int k = threadIdx.x; k < AUXN; k += blockDim.x) ax[k] = aux[(long)s * AUXN + k];
  for (int k = threadIdx.x; k < (3 + 2 * kC) * PP; k += blockDim.x) sm[k] = 0.f;
  for (int k = threadIdx.x; k < PP; k += blockDim.x) ut[k] = 0.f;
  __syncthreads();
  for (int c = 0; c < 3; c++) x0[c * PP + pc] = feat[((long)s * 3 + c) * NC + ci];
  __syncthreads();
  for (int co = 0; co < kC; co++) {
    float a = w[kOB1 + co];
    for (int cin = 0; cin < kCin; cin++)
      for (int tp = 0; tp < 9; tp++) a += w[kOW1 + (co * kCin + cin) * 9 + tp] * x0[cin * PP + pc + (tp / 3 - 1) * P + (tp % 3 - 1)];
    h1[co * PP + pc] = fmaxf(a, 0.f);
  }
  __syncthreads();
  for (int co = 0; co < kC; co++) {
    float a = w[kOB2 + co];
    for (int cin = 0; cin < kC; cin++)
      for (int tp = 0; tp < 9; tp++) a += w[kOW2 + (co * kC + cin) * 9 + tp] * h1[cin * PP + pc + (tp / 3 - 1) * P + (tp % 3 - 1)];
    h2[co * PP + pc] = fmaxf(a, 0.f);
  }
  __syncthreads();
  float y = w[kOB3];
  for (int cin = 0; cin < kC; cin++)
    for (int tp = 0; tp < 9; tp++) y += w[kOW3 + cin * 9 + tp] * h2[cin * PP + pc + (tp / 3 - 1) * P + (tp % 3 - 1)];
  for (int co = 0; co < kC; co++) {
    h1g[((long)blockIdx.x * kC + co) * NC + ci] = h1[co * PP + pc];
    h2g[((long)blockIdx.x * kC + co) * NC + ci] = h2[co * PP + pc];
  }
  const float *sav = ax, *dvvf = ax + NC, *tx = ax + 2 * NC, *ty = ax + 2 * NC + NF, *tg = ax + 2 * NC + 2 * NF;
  y = local_part<NB>(y, red);
  float res, dldu;
  if (mode == 1) {
    res = sav[ci] * y - tg[ci];
    dldu = 2.f * inv_norm * res;
  } else {
    ut[pc] = sav[ci] * y;
    __syncthreads();
    const float au = dvvf[ci] > 0.f ? local_K<NB>(ut, tx, ty, i, j) / dvvf[ci] : 0.f;
    res = x0[pc] - au;
    const float gv = -2.f * inv_norm * res;
    __syncthreads();
    ut[pc] = dvvf[ci] > 0.f ? gv / dvvf[ci] : 0.f;
    __syncthreads();
    dldu = local_K<NB>(ut, tx, ty, i, j);
  }
  // the projection is symmetric: the gradient goes back through it unchanged
  dyg[(long)blockIdx.x * NC + ci] = local_part<NB>(sav[ci] * dldu, red);
  float l = wsumf(res * res * inv_norm);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l;
  __syncthreads();
  if (threadIdx.x == 0) {
    float tot = 0.f;
    for (int k = 0; k < NC / 32; k++) tot += red[k];
    atomicAdd(loss, tot);
  }
}

// ---- FP32 backward: weight gradients accumulated into G
template <int NB>
__global__ void __launch_bounds__(NB *NB) k_nn_bwd(const float *__restrict__ W, const float *__restrict__ feat,
                                                   const int *__restrict__ idx, const float *__restrict__ h1g,
                                                   const float *__restrict__ h2g, const float *__restrict__ dyg,
                                                   float *G) {
  constexpr int NC = NB * NB, P = NB + 2, PP = P * P;
  extern __shared__ float sm[];
  float *x0 = sm;             // [3][P][P]
  float *h1 = x0 + 3 * PP;    // [32][P][P]
  float *h2 = h1 + kC * PP;   // [32][P][P], later dh1
  float *dh2 = h2 + kC * PP;  // [32][P][P]
  float *dy = dh2 + kC * PP;  // [P][P]
  float *w = dy + PP;         // [kNParam]
  const int s = idx[blockIdx.x];
  const int ci = threadIdx.x, i = ci % NB, j = ci / NB, pc = (j + 1) * P + (i + 1);
  for (int k = threadIdx.x; k < kNParam; k += blockDim.x) w[k] = W[k];
  for (int k = threadIdx.x; k < (3 + 3 * kC + 1) * PP; k += blockDim.x) sm[k] = 0.f;
  __syncthreads();
  for (int c = 0; c < 3; c++) x0[c * PP + pc] = feat[((long)s * 3 + c) * NC + ci];
  for (int c = 0; c < kC; c++) {
    h1[c * PP + pc] = h1g[((long)blockIdx.x * kC + c) * NC + ci];
    h2[c * PP + pc] = h2g[((long)blockIdx.x * kC + c) * NC + ci];
  }
  dy[pc] = dyg[(long)blockIdx.x * NC + ci];
  __syncthreads();
  // output layer: dW3, db3
  for (int e = threadIdx.x; e < kC * 9; e += blockDim.x) {
    const int cin = e / 9, tp = e % 9, off = (tp / 3 - 1) * P + (tp % 3 - 1);
    float a = 0.f;
    for (int q = 0; q < NC; q++) {
      const int pq = (q / NB + 1) * P + (q % NB + 1);
      a += dy[pq] * h2[cin * PP + pq + off];
    }
    atomicAdd(&G[kOW3 + e], a);
  }
  if (threadIdx.x == 0) {
    float a = 0.f;
    for (int q = 0; q < NC; q++) a += dy[(q / NB + 1) * P + (q % NB + 1)];
    atomicAdd(&G[kOB3], a);
  }
  // dh2 = (W3^T * dy) masked by ReLU
  for (int c = 0; c < kC; c++) {
    float a = 0.f;
    for (int tp = 0; tp < 9; tp++) a += w[kOW3 + c * 9 + tp] * dy[pc - (tp / 3 - 1) * P - (tp % 3 - 1)];
    dh2[c * PP + pc] = h2[c * PP + pc] > 0.f ? a : 0.f;
  }
  __syncthreads();
  // hidden layer: dW2, db2
  for (int e = threadIdx.x; e < kC * kC * 9; e += blockDim.x) {
    const int co = e / (kC * 9), cin = (e / 9) % kC, tp = e % 9, off = (tp / 3 - 1) * P + (tp % 3 - 1);
    float a = 0.f;
    for (int q = 0; q < NC; q++) {
      const int pq = (q / NB + 1) * P + (q % NB + 1);
      a += dh2[co * PP + pq] * h1[cin * PP + pq + off];
    }
    atomicAdd(&G[kOW2 + e], a);
  }
  for (int co = threadIdx.x; co < kC; co += blockDim.x) {
    float a = 0.f;
    for (int q = 0; q < NC; q++) a += dh2[co * PP + (q / NB + 1) * P + (q % NB + 1)];
    atomicAdd(&G[kOB2 + co], a);
  }
  // dh1 = (W2^T * dh2) masked by ReLU, into h2's space
  float *dh1 = h2;
  __syncthreads();
  for (int cin = 0; cin < kC; cin++) {
    float a = 0.f;
    for (int co = 0; co < kC; co++)
      for (int tp = 0; tp < 9; tp++)
        a += w[kOW2 + (co * kC + cin) * 9 + tp] * dh2[co * PP + pc - (tp / 3 - 1) * P - (tp % 3 - 1)];
    dh1[cin * PP + pc] = h1[cin * PP + pc] > 0.f ? a : 0.f;
  }
  __syncthreads();
  // input layer: dW1, db1
  for (int e = threadIdx.x; e < kC * kCin * 9; e += blockDim.x) {
    const int co = e / (kCin * 9), cin = (e / 9) % kCin, tp = e % 9, off = (tp / 3 - 1) * P + (tp % 3 - 1);
    float a = 0.f;
    for (int q = 0; q < NC; q++) {
      const int pq = (q / NB + 1) * P + (q % NB + 1);
      a += dh1[co * PP + pq] * x0[cin * PP + pq + off];
    }
    atomicAdd(&G[kOW1 + e], a);
  }
  for (int co = threadIdx.x; co < kC; co += blockDim.x) {
    float a = 0.f;
    for (int q = 0; q < NC; q++) a += dh1[co * PP + (q / NB + 1) * P + (q % NB + 1)];
    atomicAdd(&G[kOB1 + co], a);
  }
}

__global__ void k_adam(float *w, float *g, float *m, float *v, int n, float lr, float b1, float b2, float c1,
                       float c2) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const float gk = g[k];
    const float mk = b1 * m[k] + (1.f - b1) * gk;
    const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    w[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + 1e-8f);
    g[k] = 0.f;
  }
}

// w2 FP32 [out][in][tap] -> BF16 [tap][out][in] (the B operand layout)
__global__ void k_w2_bf16(const float *W, __nv_bfloat16 *o) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < kC * kC * 9; k += gridDim.x * blockDim.x) {
    const int tp = k / (kC * kC), co = (k / kC) % kC, cin = k % kC;
    o[k] = __float2bfloat16_rn(W[kOW2 + (co * kC + cin) * 9 + tp]);
  }
}

// A forest solved with one BiCGSTAB state per problem switches the
// correction off problem by problem: a block is left alone once its
// problem's solve has finished or its correction has stalled.
__device__ __forceinline__ bool nn_block_off(const BlockList &L, int b) {
  if (!L.stc) return false;
  const FState &q = L.stc[L.comp[b]];
  return q.done || q.nn_off;
}

// ---- inference: r1 = resid - A corr on the tower (skipped once stalled)
template <int ND>
__global__ void __launch_bounds__(256) k_nn_resid(Topo t, Coef<float> c, BlockList L, const float *__restrict__ corr,
                                                  const float *__restrict__ resid, float *__restrict__ r1,
                                                  const FState *st) {
  if (st->done || st->nn_off) return;
  const int total = L.n * t.ncell;
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < total; it += gridDim.x * blockDim.x) {
    const int p = it / t.ncell, ci = it - p * t.ncell;
    const int b = L.blocks[p];
    if (nn_block_off(L, b)) continue;
    const long q = (long)b * t.ncell + ci;
    const float a = stencil::apply_cell<float, ND>(t, c, b, L.ftypes[p], ci, corr);
    r1[q] = c.vf[q] > 0 ? resid[q] - a : 0.f;
  }
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// The network on one block staged in shared memory (x0 [3][P][P] holds the
// features with a zero halo); returns y of the calling thread's cell.  The
// 32 -> 32 layer runs as an implicit GEMM on tensor cores (M = cells, N = 32,
// K = 9 taps x 32 channels, BF16 operands, FP32 accumulation), the small
// layers on the FP32 pipes.
template <int NB>
__device__ __forceinline__ float nn_tail_bf16(const float *__restrict__ W, const __nv_bfloat16 *__restrict__ w2bf,
                                              float *x0, unsigned char *rest) {
  constexpr int P = NB + 2, PP = P * P, CS = 40;  // channel stride of the BF16 tile (padded)
  float *h2 = reinterpret_cast<float *>(rest);   // [32][P][P] FP32
  float *ws = h2 + kC * PP;                        // w1, b1 | b2 | w3, b3
  float *w1 = ws, *b1 = ws + kC * kCin * 9, *b2 = b1 + kC, *w3 = b2 + kC, *b3 = w3 + kC * 9;
  __nv_bfloat16 *h1 = reinterpret_cast<__nv_bfloat16 *>(b3 + 1);  // [P*P][CS]
  __nv_bfloat16 *wb = h1 + PP * CS;                                // [9][32][32]
  const int ci = threadIdx.x, pc = (ci / NB + 1) * P + (ci % NB + 1);
  for (int k = threadIdx.x; k < kC * kCin * 9 + kC; k += blockDim.x) ws[k] = W[kOW1 + k];
  for (int k = threadIdx.x; k < kC; k += blockDim.x) b2[k] = W[kOB2 + k];
  for (int k = threadIdx.x; k < kC * 9 + 1; k += blockDim.x) w3[k] = W[kOW3 + k];
  for (int k = threadIdx.x; k < 9 * kC * kC / 2; k += blockDim.x)
    reinterpret_cast<uint32_t *>(wb)[k] = reinterpret_cast<const uint32_t *>(w2bf)[k];
  for (int k = threadIdx.x; k < PP * CS / 2; k += blockDim.x) reinterpret_cast<uint32_t *>(h1)[k] = 0u;
  for (int k = threadIdx.x; k < kC * PP; k += blockDim.x) h2[k] = 0.f;
  __syncthreads();
  // input layer (FP32) -> BF16 tile [pixel][channel]
  for (int co = 0; co < kC; co++) {
    float a = b1[co];
    for (int cin = 0; cin < kCin; cin++)
      for (int tp = 0; tp < 9; tp++) a += w1[(co * kCin + cin) * 9 + tp] * x0[cin * PP + pc + (tp / 3 - 1) * P + (tp % 3 - 1)];
    h1[pc * CS + co] = __float2bfloat16_rn(fmaxf(a, 0.f));
  }
  __syncthreads();
  // hidden layer: warp w owns cells [32w, 32w+32) = two m16 tiles, all four
  // n8 tiles of the 32 output channels
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  float acc[2][4][4];
  for (int mt = 0; mt < 2; mt++)
    for (int nt = 0; nt < 4; nt++)
      for (int r = 0; r < 4; r++) acc[mt][nt][r] = 0.f;
  int prow[2][2];  // padded pixel of fragment rows g and g+8 of each m tile
  for (int mt = 0; mt < 2; mt++)
    for (int hh = 0; hh < 2; hh++) {
      const int cell = warp * 32 + mt * 16 + g + 8 * hh;
      prow[mt][hh] = (cell / NB + 1) * P + (cell % NB + 1);
    }
  const uint32_t *h1w = reinterpret_cast<const uint32_t *>(h1);
  const uint32_t *wbw = reinterpret_cast<const uint32_t *>(wb);
  for (int tp = 0; tp < 9; tp++) {
    const int off = (tp / 3 - 1) * P + (tp % 3 - 1);
    for (int kh = 0; kh < 2; kh++) {
      const int k0 = kh * 16 + 2 * tq;  // channel of the fragment's first column pair
      uint32_t bfr[4][2];
      for (int nt = 0; nt < 4; nt++) {
        const int n = nt * 8 + g;
        bfr[nt][0] = wbw[((tp * kC + n) * kC + k0) >> 1];
        bfr[nt][1] = wbw[((tp * kC + n) * kC + k0 + 8) >> 1];
      }
      for (int mt = 0; mt < 2; mt++) {
        const int r0 = (prow[mt][0] + off) * CS + k0, r1i = (prow[mt][1] + off) * CS + k0;
        const uint32_t a0 = h1w[r0 >> 1], a1 = h1w[r1i >> 1], a2 = h1w[(r0 + 8) >> 1], a3 = h1w[(r1i + 8) >> 1];
        for (int nt = 0; nt < 4; nt++) mma_bf16(acc[mt][nt], a0, a1, a2, a3, bfr[nt][0], bfr[nt][1]);
      }
    }
  }
  for (int mt = 0; mt < 2; mt++)
    for (int nt = 0; nt < 4; nt++)
      for (int r = 0; r < 4; r++) {
        const int pix = prow[mt][r >> 1];
        const int n = nt * 8 + 2 * tq + (r & 1);
        h2[n * PP + pix] = fmaxf(acc[mt][nt][r] + b2[n], 0.f);
      }
  __syncthreads();
  float y = b3[0];
  for (int cin = 0; cin < kC; cin++)
    for (int tp = 0; tp < 9; tp++) y += w3[cin * 9 + tp] * h2[cin * PP + pc + (tp / 3 - 1) * P + (tp % 3 - 1)];
  return y;
}

// ---- the 32 -> 32 layer of 16x16 blocks on the 5th-generation tensor
// cores (tcgen05.mma, accumulator in tensor memory).  The layer is an
// implicit GEMM over the block's padded 18x18 pixel grid,
//   D[pixel][out] = sum over taps t, channels k of h1[pixel + off_t][k] * W_t[out][k],
// with the rows taken on the padded grid itself (halo columns included), so
// that every tap's A operand is one shared-memory matrix shifted by off_t
// pixels and no im2col copy is made.  Three M = 128 tiles cover the
// interior pixels 19 .. 304; rows that fall on halo pixels are discarded.
// h1 and the weights are stored in the canonical no-swizzle K-major layout:
// [channel chunk of 8][row][8 channels] BF16, so that one core matrix (8
// rows x 16 bytes) is contiguous, 8-row groups are SBO = 128 bytes apart and
// channel chunks LBO = rows * 16 bytes apart.  One thread issues the 54 MMAs
// (3 tiles x 9 taps x 2 K-steps of 16); their completion arrives on an
// mbarrier; each warp then reads its lane quarter of the accumulators with
// tcgen05.ld.  Every wait is bounded: on a timeout the kernel raises
// g_nn_err, waits (bounded) once more and frees its tensor memory.
namespace tc05 {
constexpr int P = 18, PP = P * P;
constexpr int kRow0 = P + 1;      // first interior pixel
constexpr int kTiles = 3;         // M = 128 tiles from kRow0
constexpr int kPixA = 424;        // rows of the A matrix: >= kRow0 + 3*128 + P + 1, a multiple of 8
constexpr int kCols = 128;        // tensor-memory columns: 3 tiles x 32 (power of two)
constexpr uint32_t kLboA = kPixA * 16, kLboB = kC * 16, kSbo = 128;
// instruction descriptor of kind::f16: FP32 accumulator (bit 4), BF16 A and
// B (bits 7, 10), both K-major, N = 32 (bits 17-22: N >> 3), M = 128
// (bits 24-28: M >> 4)
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kC >> 3) << 17) | ((128u >> 4) << 24);
constexpr long kWaitLimit = 1l << 22;

// shared-memory matrix descriptor, no swizzle (bits 0-13 address >> 4,
// 16-29 LBO >> 4, 32-45 SBO >> 4, bit 46 the descriptor version)
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long i = 0; i < kWaitLimit; i++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
}  // namespace tc05

__device__ int g_nn_err;  // a tensor-core wait timed out (read and cleared by the host)

template <int NB>
constexpr size_t tc_smem() {
  return sizeof(float) * (3 * tc05::PP + 1232 + kC * tc05::PP) + 128 + (size_t)4 * tc05::kPixA * 16 +
         (size_t)9 * 4 * kC * 16 + 64;
}

// the tcgen05 form of nn_tail_bf16 for 16x16 blocks (same inputs, same
// output; the hidden layer's products are summed in another order)
__device__ __forceinline__ float nn_tail_tc05(const float *__restrict__ W, const __nv_bfloat16 *__restrict__ w2bf,
                                              float *x0, unsigned char *rest) {
  using namespace tc05;
  constexpr int NB = 16;
  float *ws = reinterpret_cast<float *>(rest);  // w1, b1 | b2 | w3, b3 (1217 floats, 1232 reserved)
  float *w1 = ws, *b1 = ws + kC * kCin * 9, *b2 = b1 + kC, *w3 = b2 + kC, *b3 = w3 + kC * 9;
  float *h2 = ws + 1232;  // [32][PP] FP32
  unsigned char *base = reinterpret_cast<unsigned char *>(h2 + kC * PP);
  base += (128 - (smem_u32(base) & 127)) & 127;  // 128-byte aligned operand area
  __nv_bfloat16 *ha = reinterpret_cast<__nv_bfloat16 *>(base);                    // [4][kPixA][8]
  __nv_bfloat16 *wb = reinterpret_cast<__nv_bfloat16 *>(base + 4 * kPixA * 16);  // [9][4][32][8]
  uint64_t *bar = reinterpret_cast<uint64_t *>(base + 4 * kPixA * 16 + 9 * 4 * kC * 16);
  uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
  const int ci = threadIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int pc = (ci / NB + 1) * P + (ci % NB + 1);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  for (int k = threadIdx.x; k < kC * kCin * 9 + kC; k += blockDim.x) ws[k] = W[kOW1 + k];
  for (int k = threadIdx.x; k < kC; k += blockDim.x) b2[k] = W[kOB2 + k];
  for (int k = threadIdx.x; k < kC * 9 + 1; k += blockDim.x) w3[k] = W[kOW3 + k];
  // w2bf is [tap][out][in]; wb is [tap][in / 8][out][in % 8]
  for (int k = threadIdx.x; k < 9 * kC * kC; k += blockDim.x) {
    const int tp = k / (kC * kC), o = (k / kC) % kC, i = k % kC;
    wb[((tp * 4 + (i >> 3)) * kC + o) * 8 + (i & 7)] = w2bf[k];
  }
  for (int k = threadIdx.x; k < 4 * kPixA * 8 / 2; k += blockDim.x) reinterpret_cast<uint32_t *>(ha)[k] = 0u;
  for (int k = threadIdx.x; k < kC * PP; k += blockDim.x) h2[k] = 0.f;
  __syncthreads();
  // input layer (FP32) -> BF16 A matrix
  for (int co = 0; co < kC; co++) {
    float a = b1[co];
    for (int cin = 0; cin < kCin; cin++)
      for (int tp = 0; tp < 9; tp++) a += w1[(co * kCin + cin) * 9 + tp] * x0[cin * PP + pc + (tp / 3 - 1) * P + (tp % 3 - 1)];
    ha[((co >> 3) * kPixA + pc) * 8 + (co & 7)] = __float2bfloat16_rn(fmaxf(a, 0.f));
  }
  // generic-proxy writes of the operands made visible to the tensor core
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *slot;
  if (threadIdx.x == 0) {
    const uint32_t a0 = smem_u32(ha), b0 = smem_u32(wb);
    for (int t = 0; t < kTiles; t++)
      for (int tp = 0; tp < 9; tp++) {
        const int off = (tp / 3 - 1) * P + (tp % 3 - 1);
        for (int kh = 0; kh < 2; kh++) {
          const uint64_t ad = sdesc(a0 + (uint32_t)(kRow0 + 128 * t + off) * 16 + kh * 2 * kLboA, kLboA, kSbo);
          const uint64_t bd = sdesc(b0 + (uint32_t)tp * 4 * kC * 16 + kh * 2 * kLboB, kLboB, kSbo);
          const uint32_t acc = (tp | kh) ? 1u : 0u;
          asm volatile(
              "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem + 32 * t),
              "l"(ad), "l"(bd), "r"(kIdesc), "r"(acc));
        }
      }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
  }
  bool ok = mbar_wait(smem_u32(bar), 0);
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(&g_nn_err, 1);
    ok = mbar_wait(smem_u32(bar), 0) && false;  // drain (bounded), the results are not used
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    const int q = warp & 3;
    for (int t = warp < 4 ? 0 : 1; t < kTiles; t += 2) {
      uint32_t r[32];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
          "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(tmem + ((uint32_t)(32 * q) << 16) + 32 * t));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      const int pix = kRow0 + 128 * t + 32 * q + lane;
      const int py = pix / P, px = pix - py * P;
      if (py >= 1 && py <= NB && px >= 1 && px <= NB)
        for (int n = 0; n < kC; n++) h2[n * PP + pix] = fmaxf(__uint_as_float(r[n]) + b2[n], 0.f);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
  }
  float y = b3[0];
  for (int cin = 0; cin < kC; cin++)
    for (int tp = 0; tp < 9; tp++) y += w3[cin * 9 + tp] * h2[cin * PP + pc + (tp / 3 - 1) * P + (tp % 3 - 1)];
  return y;
}

// inference inside the solve: corr += s * sa * net(features of r1), one CTA
// per block of the finest tower, one thread per cell
template <int NB, bool TC = false>
__global__ void __launch_bounds__(NB *NB) k_nn_infer(Topo t, Coef<float> c, BlockList L, const float *__restrict__ W,
                                                     const __nv_bfloat16 *__restrict__ w2bf,
                                                     const float *__restrict__ r1, const double *__restrict__ sa,
                                                     float *__restrict__ corr, const FState *st) {
  constexpr int NC = NB * NB, P = NB + 2, PP = P * P;
  extern __shared__ __align__(16) unsigned char smraw[];
  float *x0 = reinterpret_cast<float *>(smraw);  // [3][P][P]
  __shared__ float red[NC / 32];
  if (st->done || st->nn_off) return;
  const int p = blockIdx.x, ci = threadIdx.x, pc = (ci / NB + 1) * P + (ci % NB + 1);
  const int b = L.blocks[p];
  if (nn_block_off(L, b)) return;  // uniform over the CTA
  const long q = (long)b * NC + ci;
  for (int k = threadIdx.x; k < 3 * PP; k += blockDim.x) x0[k] = 0.f;
  const float rv = r1[q];
  const float m = block_max<NC>(fabsf(rv), red);
  const float s = m > 0.f ? m : 1.f;
  float f[3];
  cell_features<NB>(t, c, b, ci, rv, s, f);
  for (int k = 0; k < 3; k++) x0[k * PP + pc] = f[k];
  float y0;
  if constexpr (TC)
    y0 = nn_tail_tc05(W, w2bf, x0, smraw + 3 * PP * sizeof(float));
  else
    y0 = nn_tail_bf16<NB>(W, w2bf, x0, smraw + 3 * PP * sizeof(float));
  const float y = local_part<NB>(y0, red);
  corr[q] += s * (float)sa[(long)p * NC + ci] * y;
}

// the tensor-core forward on explicit feature blocks (test hook)
template <int NB, bool TC = false>
__global__ void __launch_bounds__(NB *NB) k_nn_forward(const float *__restrict__ W,
                                                       const __nv_bfloat16 *__restrict__ w2bf,
                                                       const float *__restrict__ feat, float *__restrict__ y) {
  constexpr int NC = NB * NB, P = NB + 2, PP = P * P;
  extern __shared__ __align__(16) unsigned char smraw[];
  float *x0 = reinterpret_cast<float *>(smraw);
  const int ci = threadIdx.x, pc = (ci / NB + 1) * P + (ci % NB + 1);
  for (int k = threadIdx.x; k < 3 * PP; k += blockDim.x) x0[k] = 0.f;
  __syncthreads();
  for (int k = 0; k < 3; k++) x0[k * PP + pc] = feat[((long)blockIdx.x * 3 + k) * NC + ci];
  if constexpr (TC)
    y[(long)blockIdx.x * NC + ci] = nn_tail_tc05(W, w2bf, x0, smraw + 3 * PP * sizeof(float));
  else
    y[(long)blockIdx.x * NC + ci] = nn_tail_bf16<NB>(W, w2bf, x0, smraw + 3 * PP * sizeof(float));
}

template <int NB>
constexpr size_t fwd_smem() {
  return sizeof(float) * ((3 + 2 * kC) * (NB + 2) * (NB + 2) + kNParam + 3 * NB * NB + 2 * (NB + 1) * NB +
                          (NB + 2) * (NB + 2));
}
template <int NB>
constexpr size_t bwd_smem() {
  return sizeof(float) * ((3 + 3 * kC + 1) * (NB + 2) * (NB + 2) + kNParam);
}
template <int NB>
constexpr size_t infer_smem() {
  return sizeof(float) * ((3 + kC) * (NB + 2) * (NB + 2) + kC * kCin * 9 + kC + kC + kC * 9 + 1) +
         sizeof(__nv_bfloat16) * ((size_t)(NB + 2) * (NB + 2) * 40 + 9 * kC * kC) + 16;
}

}  // namespace

// the tensor-core wait error word (g_nn_err): its value, cleared when asked
int nn_tc_error(bool clear) {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_nn_err, sizeof(int)) != cudaSuccess) return -1;
  if (clear && v) {
    const int z = 0;
    if (cudaMemcpyToSymbol(g_nn_err, &z, sizeof(int)) != cudaSuccess) return -1;
  }
  return v;
}

static void set_smem_attrs() {
  ensure_max_smem((const void *)k_nn_fwd<16>, (int)fwd_smem<16>());
  ensure_max_smem((const void *)k_nn_bwd<16>, (int)bwd_smem<16>());
  ensure_max_smem((const void *)k_nn_fwd<8>, (int)fwd_smem<8>());
  ensure_max_smem((const void *)k_nn_bwd<8>, (int)bwd_smem<8>());
  ensure_max_smem((const void *)k_nn_infer<16>, (int)infer_smem<16>());
  ensure_max_smem((const void *)k_nn_infer<8>, (int)infer_smem<8>());
  ensure_max_smem((const void *)k_nn_forward<16>, (int)infer_smem<16>());
  ensure_max_smem((const void *)k_nn_forward<8>, (int)infer_smem<8>());
  ensure_max_smem((const void *)k_nn_infer<16, true>, (int)tc_smem<16>());
  ensure_max_smem((const void *)k_nn_forward<16, true>, (int)tc_smem<16>());
}

// ---------------------------------------------------------------------------
// host side

bool MacGpu::learned_supported() const { return tt_.ndim == 2 && (tt_.nb == 8 || tt_.nb == 16); }

void MacGpu::learned_init(unsigned seed) {
  LearnedState &L = ls_;
  L.nb = tt_.nb;
  auto fa = [&](float *&p, size_t n) {
    if (!p && dev_malloc(&p, n * sizeof(float)) != cudaSuccess) {
      p = nullptr;
      fail("out of device memory (learned)");
    }
  };
  fa(L.w, kNParam);
  fa(L.g, kNParam);
  fa(L.m, kNParam);
  fa(L.v, kNParam);
  fa(L.loss, 1);
  if (!L.w2bf && dev_malloc(&L.w2bf, 9 * kC * kC * sizeof(uint16_t)) != cudaSuccess) fail("out of device memory");
  if (!err_.empty()) return;
  // He initialisation; the output layer starts at zero, so the untrained
  // correction is zero and the preconditioner is the plain V-cycle
  std::mt19937 rng(seed);
  std::vector<float> w(kNParam, 0.f);
  std::normal_distribution<float> n1(0.f, std::sqrt(2.f / (kCin * 9))), n2(0.f, std::sqrt(2.f / (kC * 9)));
  for (int k = kOW1; k < kOB1; k++) w[k] = n1(rng);
  for (int k = kOW2; k < kOB2; k++) w[k] = n2(rng);
  CK(cudaMemcpyAsync(L.w, w.data(), kNParam * sizeof(float), cudaMemcpyHostToDevice, stream_));
  CK(cudaMemsetAsync(L.g, 0, kNParam * sizeof(float), stream_));
  CK(cudaMemsetAsync(L.m, 0, kNParam * sizeof(float), stream_));
  CK(cudaMemsetAsync(L.v, 0, kNParam * sizeof(float), stream_));
  L.step = 0;
  L.trained = false;
  learned_sync_bf16();
}

void MacGpu::learned_sync_bf16() {
  k_w2_bf16<<<36, 256, 0, stream_>>>(ls_.w, reinterpret_cast<__nv_bfloat16 *>(ls_.w2bf));
  CK(cudaGetLastError());
}

int MacGpu::learned_set_weights(const float *w, int n) {
  if (n != kNParam) return -1;
  if (!ls_.w) learned_init(1);
  CKR_(cudaMemcpyAsync(ls_.w, w, kNParam * sizeof(float), cudaMemcpyHostToDevice, stream_), -1);
  learned_sync_bf16();
  ls_.trained = true;
  return err_.empty() ? 0 : -1;
}

int MacGpu::learned_get_weights(float *w, int n) {
  if (n != kNParam || !ls_.w) return -1;
  CKR_(cudaMemcpyAsync(w, ls_.w, kNParam * sizeof(float), cudaMemcpyDeviceToHost, stream_), -1);
  CKR_(cudaStreamSynchronize(stream_), -1);
  return 0;
}

// reserve room for `more` training blocks
void MacGpu::learned_reserve(int more) {
  LearnedState &L = ls_;
  const int need = L.nsamp + more;
  if (need <= L.cap) return;
  const int cap = std::max(need, 2 * L.cap);
  const size_t nc = (size_t)ncell_;
  const size_t na = aux_len();
  float *f = nullptr, *a = nullptr;
  if (dev_malloc(&f, (size_t)cap * 3 * nc * sizeof(float)) != cudaSuccess ||
      dev_malloc(&a, (size_t)cap * na * sizeof(float)) != cudaSuccess) {
    if (f) dev_free(f);
    fail("out of device memory (training set)");
    return;
  }
  if (L.nsamp) {
    CK(cudaMemcpyAsync(f, L.feat, (size_t)L.nsamp * 3 * nc * sizeof(float), cudaMemcpyDeviceToDevice, stream_));
    CK(cudaMemcpyAsync(a, L.aux, (size_t)L.nsamp * na * sizeof(float), cudaMemcpyDeviceToDevice, stream_));
  }
  if (L.feat) dev_free(L.feat);
  if (L.aux) dev_free(L.aux);
  L.feat = f;
  L.aux = a;
  L.cap = cap;
}

void MacGpu::learned_free() {
  LearnedState &L = ls_;
  for (float *p : {L.w, L.g, L.m, L.v, L.loss, L.feat, L.aux, L.r1, L.scale})
    if (p) dev_free(p);
  if (L.w2bf) dev_free(L.w2bf);
  L = LearnedState{};
}

// the FP32 V-cycle's output on the finest tower for residual r (tower cells)
void MacGpu::learned_vcycle(float *r, float *z) {
  const int L = finest_;
  CK(cudaMemsetAsync(d_st_, 0, sizeof(FState), stream_));
  // the V-cycle reads its residual from d_resid32_ and writes d_corr32_
  const size_t n = (size_t)tt_.num_blocks * ncell_;
  CK(cudaMemcpyAsync(d_resid32_, r, n * sizeof(float), cudaMemcpyDeviceToDevice, stream_));
  vcycle_device<float>(L, d_resid32_, d_corr32_, c32_, nullptr);
  CK(cudaMemcpyAsync(z, d_corr32_, n * sizeof(float), cudaMemcpyDeviceToDevice, stream_));
}

namespace {
// e = x* - x_k (FP64 -> FP32) on the tower cells; everything else 0
__global__ void k_err32(BlockList L, int ncell, const double *xs, const double *xk, float *e) {
  const int total = L.n * ncell;
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < total; it += gridDim.x * blockDim.x) {
    const int p = it / ncell;
    const long q = (long)L.blocks[p] * ncell + (it - p * ncell);
    e[q] = (float)(xs[q] - xk[q]);
  }
}
__global__ void k_sub32(BlockList L, int ncell, const float *a, const float *b, float *o) {
  const int total = L.n * ncell;
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < total; it += gridDim.x * blockDim.x) {
    const int p = it / ncell;
    const long q = (long)L.blocks[p] * ncell + (it - p * ncell);
    o[q] = a[q] - b[q];
  }
}
inline int lgrid(long w) { return (int)std::max<long>(1, std::min<long>((w + 255) / 256, 152 * 16)); }
}  // namespace

// Training pairs from the plain solver: one device solve of the current
// right-hand side from x0 = 0 with the plain FP32 V-cycle, tightened to
// tol_rel 1e-12, records every iterate x_k; then, with x* the converged
// solution, e = x* - x_k, r = A e (FP32), z = V(r), r1 = r - A z, e1 = e - z
// become one training block per tower block.
int MacGpu::learned_collect(int max_iters, int max_samples) {
  if (!learned_supported()) {
    fail("learned correction: 2D blocks of 8 or 16 cells only");
    return -1;
  }
  if (!ls_.w) learned_init(1);
  SolverParams save = prm_;
  prm_.precision = 1;
  prm_.use_mg_precond = 1;
  prm_.bottom = 1;
  prm_.graph = 0;
  prm_.learned = 0;
  prm_.tol_rel = 1e-12;
  prm_.tol_abs = 0.0;
  prm_.max_iter = std::max(1, max_iters);
  if (prepare_device() != 0) {
    prm_ = save;
    return -1;
  }
  ensure_smooth_factors();  // sa scales the pairs
  const size_t n = (size_t)tt_.num_blocks * ncell_;
  std::vector<double *> rec;
  record_ = &rec;
  zero_sol();
  const int rc = enqueue_solve();
  record_ = nullptr;
  prm_ = save;
  if (rc != 0) {
    for (double *p : rec) dev_free(p);
    return -1;
  }
  CKR_(cudaStreamSynchronize(stream_), -1);
  const int L = finest_;
  const BlockList TL = tower_list(L);
  const long w = (long)TL.n * ncell_;
  float *e = nullptr, *r = nullptr, *z = nullptr, *r1 = nullptr;
  dev_malloc(&e, n * sizeof(float));
  dev_malloc(&r, n * sizeof(float));
  dev_malloc(&z, n * sizeof(float));
  dev_malloc(&r1, n * sizeof(float));
  if (!e || !r || !z || !r1) {
    fail("out of device memory (collection)");
    return -1;
  }
  cudaMemsetAsync(e, 0, n * sizeof(float), stream_);
  cudaMemsetAsync(r, 0, n * sizeof(float), stream_);
  // at most max_samples pairs: every stride-th block of each iterate, the
  // offset moving from iterate to iterate
  const long all = (long)rec.size() * TL.n;
  const int stride = max_samples > 0 && all > max_samples ? (int)((all + max_samples - 1) / max_samples) : 1;
  long want = 0;
  for (size_t k = 0; k < rec.size(); k++) {
    const int off = (int)((k * 7) % stride);
    want += off < TL.n ? (TL.n - off + stride - 1) / stride : 0;
  }
  learned_reserve((int)want);
  const double *sa = d_sfac_.size() > (size_t)L ? d_sfac_[L] : nullptr;
  int kit = 0;
  for (double *xk : rec) {
    const int off = (int)((kit++ * 7) % stride);
    const int cnt = off < TL.n ? (TL.n - off + stride - 1) / stride : 0;
    if (!err_.empty() || !sa) break;
    k_err32<<<lgrid(w), 256, 0, stream_>>>(TL, ncell_, vec_[kSOL], xk, e);
    launch_apply<float>(topo_, c32_, TL, e, r, nullptr, nullptr, stream_);
    learned_vcycle(r, z);
    launch_apply<float>(topo_, c32_, TL, z, r1, r, nullptr, stream_);
    k_sub32<<<lgrid(w), 256, 0, stream_>>>(TL, ncell_, e, z, e);
    const long o = (long)ls_.nsamp * ncell_, oa = (long)ls_.nsamp * aux_len();
    if (cnt > 0) {
      if (tt_.nb == 16)
        k_nn_pairs<16><<<cnt, 256, 0, stream_>>>(topo_, c32_, TL, r1, e, sa, ls_.feat + 3 * o, ls_.aux + oa, off,
                                                 stride);
      else
        k_nn_pairs<8><<<cnt, 64, 0, stream_>>>(topo_, c32_, TL, r1, e, sa, ls_.feat + 3 * o, ls_.aux + oa, off,
                                               stride);
      CKR_(cudaGetLastError(), -1);
    }
    ls_.nsamp += cnt;
  }
  CKR_(cudaStreamSynchronize(stream_), -1);
  for (double *p : rec) dev_free(p);
  dev_free(e);
  dev_free(r);
  dev_free(z);
  dev_free(r1);
  // the collection solve overwrote the solution: leave a zero guess
  zero_sol();
  return err_.empty() ? (int)rec.size() : -1;
}

// one gradient of the loss over the blocks idx[0..nblk) (accumulated into g),
// returns the loss; the activations go to the scratch vectors
float MacGpu::learned_grad(const int *d_idx, int nblk, float inv_norm, float *h1, float *h2, float *dy) {
  CKR_(cudaMemsetAsync(ls_.loss, 0, sizeof(float), stream_), 0.f);
  if (ls_.nb == 16) {
    k_nn_fwd<16><<<nblk, 256, fwd_smem<16>(), stream_>>>(ls_.w, ls_.feat, ls_.aux, d_idx, h1, h2, dy,
                                                         ls_.loss, inv_norm, prm_.learned_loss);
    k_nn_bwd<16><<<nblk, 256, bwd_smem<16>(), stream_>>>(ls_.w, ls_.feat, d_idx, h1, h2, dy, ls_.g);
  } else {
    k_nn_fwd<8><<<nblk, 64, fwd_smem<8>(), stream_>>>(ls_.w, ls_.feat, ls_.aux, d_idx, h1, h2, dy,
                                                      ls_.loss, inv_norm, prm_.learned_loss);
    k_nn_bwd<8><<<nblk, 64, bwd_smem<8>(), stream_>>>(ls_.w, ls_.feat, d_idx, h1, h2, dy, ls_.g);
  }
  CKR_(cudaGetLastError(), 0.f);
  float l = 0.f;
  CKR_(cudaMemcpyAsync(&l, ls_.loss, sizeof(float), cudaMemcpyDeviceToHost, stream_), 0.f);
  CKR_(cudaStreamSynchronize(stream_), 0.f);
  return l;
}

// Adam over the training set in shuffled minibatches; returns the mean loss
// of the last epoch (per block), or -1
float MacGpu::learned_train(int epochs, float lr, int batch, unsigned seed) {
  if (!ls_.w || ls_.nsamp == 0) return -1.f;
  set_smem_attrs();
  batch = std::max(1, std::min(batch, ls_.nsamp));
  const size_t nc = (size_t)ncell_;
  float *h1 = nullptr, *h2 = nullptr, *dy = nullptr;
  int *d_idx = nullptr;
  dev_malloc(&h1, (size_t)batch * kC * nc * sizeof(float));
  dev_malloc(&h2, (size_t)batch * kC * nc * sizeof(float));
  dev_malloc(&dy, (size_t)batch * nc * sizeof(float));
  dev_malloc(&d_idx, (size_t)ls_.nsamp * sizeof(int));
  if (!h1 || !h2 || !dy || !d_idx) {
    fail("out of device memory (training)");
    return -1.f;
  }
  std::mt19937 rng(seed);
  std::vector<int> idx(ls_.nsamp);
  float last = 0.f;
  for (int ep = 0; ep < epochs && err_.empty(); ep++) {
    for (int k = 0; k < ls_.nsamp; k++) idx[k] = k;
    std::shuffle(idx.begin(), idx.end(), rng);
    CKR_(cudaMemcpyAsync(d_idx, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice, stream_), -1.f);
    double tot = 0.0;
    for (int s0 = 0; s0 < ls_.nsamp; s0 += batch) {
      const int nblk = std::min(batch, ls_.nsamp - s0);
      const float inv = 1.f / (float)nblk;
      tot += learned_grad(d_idx + s0, nblk, inv, h1, h2, dy) * nblk;
      ls_.step++;
      const float b1 = 0.9f, b2 = 0.999f;
      k_adam<<<41, 256, 0, stream_>>>(ls_.w, ls_.g, ls_.m, ls_.v, kNParam, lr, b1, b2,
                                      1.f - std::pow(b1, (float)ls_.step), 1.f - std::pow(b2, (float)ls_.step));
    }
    last = (float)(tot / ls_.nsamp);
  }
  CKR_(cudaStreamSynchronize(stream_), -1.f);
  dev_free(h1);
  dev_free(h2);
  dev_free(dy);
  dev_free(d_idx);
  learned_sync_bf16();
  ls_.trained = true;
  return err_.empty() ? last : -1.f;
}

// mean loss (per block) of the collected pairs under the current weights:
// the training forward over the whole set, no update (the gradient it
// accumulates is discarded)
float MacGpu::learned_eval() {
  if (!ls_.w || ls_.nsamp == 0) return -1.f;
  set_smem_attrs();
  const int batch = std::min(256, ls_.nsamp);
  const size_t nc = (size_t)ncell_;
  float *h1 = nullptr, *h2 = nullptr, *dy = nullptr;
  int *d_idx = nullptr;
  dev_malloc(&h1, (size_t)batch * kC * nc * sizeof(float));
  dev_malloc(&h2, (size_t)batch * kC * nc * sizeof(float));
  dev_malloc(&dy, (size_t)batch * nc * sizeof(float));
  dev_malloc(&d_idx, (size_t)ls_.nsamp * sizeof(int));
  if (!h1 || !h2 || !dy || !d_idx) {
    fail("out of device memory (evaluation)");
    return -1.f;
  }
  std::vector<int> idx(ls_.nsamp);
  for (int k = 0; k < ls_.nsamp; k++) idx[k] = k;
  CKR_(cudaMemcpyAsync(d_idx, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice, stream_), -1.f);
  double tot = 0.0;
  for (int s0 = 0; s0 < ls_.nsamp; s0 += batch) {
    const int nblk = std::min(batch, ls_.nsamp - s0);
    tot += learned_grad(d_idx + s0, nblk, 1.f / (float)nblk, h1, h2, dy) * nblk;
  }
  CKR_(cudaMemsetAsync(ls_.g, 0, kNParam * sizeof(float), stream_), -1.f);
  CKR_(cudaStreamSynchronize(stream_), -1.f);
  dev_free(h1);
  dev_free(h2);
  dev_free(dy);
  dev_free(d_idx);
  return err_.empty() ? (float)(tot / ls_.nsamp) : -1.f;
}

// loss and gradient of explicit training blocks (a test hook): feat
// [n][3][ncell] and aux [n][aux_len()] on the host; grad [kNParam]
float MacGpu::learned_loss_grad(const float *feat, const float *aux, int n, float *grad) {
  if (!ls_.w) learned_init(1);
  set_smem_attrs();
  const int keep = ls_.nsamp;
  ls_.nsamp = 0;
  learned_reserve(n);
  const size_t nc = (size_t)ncell_;
  CKR_(cudaMemcpyAsync(ls_.feat, feat, (size_t)n * 3 * nc * sizeof(float), cudaMemcpyHostToDevice, stream_), -1.f);
  CKR_(cudaMemcpyAsync(ls_.aux, aux, (size_t)n * aux_len() * sizeof(float), cudaMemcpyHostToDevice, stream_),
       -1.f);
  ls_.nsamp = n;
  float *h1 = nullptr, *h2 = nullptr, *dy = nullptr;
  int *d_idx = nullptr;
  dev_malloc(&h1, (size_t)n * kC * nc * sizeof(float));
  dev_malloc(&h2, (size_t)n * kC * nc * sizeof(float));
  dev_malloc(&dy, (size_t)n * nc * sizeof(float));
  dev_malloc(&d_idx, (size_t)n * sizeof(int));
  std::vector<int> idx(n);
  for (int k = 0; k < n; k++) idx[k] = k;
  cudaMemcpyAsync(d_idx, idx.data(), n * sizeof(int), cudaMemcpyHostToDevice, stream_);
  CKR_(cudaMemsetAsync(ls_.g, 0, kNParam * sizeof(float), stream_), -1.f);
  const float l = learned_grad(d_idx, n, 1.f / (float)n, h1, h2, dy);
  CKR_(cudaMemcpyAsync(grad, ls_.g, kNParam * sizeof(float), cudaMemcpyDeviceToHost, stream_), -1.f);
  CKR_(cudaStreamSynchronize(stream_), -1.f);
  CKR_(cudaMemsetAsync(ls_.g, 0, kNParam * sizeof(float), stream_), -1.f);
  dev_free(h1);
  dev_free(h2);
  dev_free(dy);
  dev_free(d_idx);
  // the explicit blocks replaced the training set
  (void)keep;
  ls_.nsamp = 0;
  return l;
}

// the tensor-core forward of explicit feature blocks (test hook)
int MacGpu::learned_forward(const float *feat, int n, float *y) {
  if (!ls_.w) learned_init(1);
  set_smem_attrs();
  const size_t nc = (size_t)ncell_;
  float *df = nullptr, *dy = nullptr;
  if (dev_malloc(&df, (size_t)n * 3 * nc * sizeof(float)) != cudaSuccess ||
      dev_malloc(&dy, (size_t)n * nc * sizeof(float)) != cudaSuccess) {
    if (df) dev_free(df);
    fail("out of device memory");
    return -1;
  }
  CKR_(cudaMemcpyAsync(df, feat, (size_t)n * 3 * nc * sizeof(float), cudaMemcpyHostToDevice, stream_), -1);
  if (ls_.nb == 16) {
    if (prm_.learned_tc05)
      k_nn_forward<16, true><<<n, 256, tc_smem<16>(), stream_>>>(ls_.w, (const __nv_bfloat16 *)ls_.w2bf, df, dy);
    else
      k_nn_forward<16><<<n, 256, infer_smem<16>(), stream_>>>(ls_.w, (const __nv_bfloat16 *)ls_.w2bf, df, dy);
  } else {
    k_nn_forward<8><<<n, 64, infer_smem<8>(), stream_>>>(ls_.w, (const __nv_bfloat16 *)ls_.w2bf, df, dy);
  }
  CKR_(cudaGetLastError(), -1);
  CKR_(cudaMemcpyAsync(y, dy, (size_t)n * nc * sizeof(float), cudaMemcpyDeviceToHost, stream_), -1);
  CKR_(cudaStreamSynchronize(stream_), -1);
  dev_free(df);
  dev_free(dy);
  if (nn_tc_error(true) > 0) {
    fail("learned correction: a tensor-core wait timed out");
    return -1;
  }
  return 0;
}

// buffers and kernel attributes of the correction, set up before a graph
// capture (no allocation happens inside the captured iteration)
void MacGpu::learned_prepare() {
  set_smem_attrs();
  if (ls_.r1) return;
  const size_t n = (size_t)tt_.num_blocks * ncell_;
  if (dev_malloc(&ls_.r1, n * sizeof(float)) != cudaSuccess) {
    ls_.r1 = nullptr;
    fail("out of device memory (learned)");
    return;
  }
  CK(cudaMemsetAsync(ls_.r1, 0, n * sizeof(float), stream_));
}

// the correction inside the device iteration: r1 = resid - A corr, then
// corr += s * sa * net(...) on every block of the finest tower
void MacGpu::learned_apply(float *resid, float *corr) {
  const int L = finest_;
  const BlockList TL = tower_list(L);
  const long w = (long)TL.n * ncell_;
  if (!ls_.r1) {
    fail("learned correction used before its buffers were prepared");
    return;
  }
  const double *sa = d_sfac_[L];
  launch_k(false, k_nn_resid<2>, lgrid(w), 256, 0, stream_, topo_, c32_, TL, (const float *)corr,
           (const float *)resid, ls_.r1, (const FState *)d_st_);
  if (ls_.nb == 16)
    if (prm_.learned_tc05)
      launch_k(false, k_nn_infer<16, true>, TL.n, 256, tc_smem<16>(), stream_, topo_, c32_, TL, (const float *)ls_.w,
               (const __nv_bfloat16 *)ls_.w2bf, (const float *)ls_.r1, sa, corr, (const FState *)d_st_);
    else
      launch_k(false, k_nn_infer<16>, TL.n, 256, infer_smem<16>(), stream_, topo_, c32_, TL, (const float *)ls_.w,
               (const __nv_bfloat16 *)ls_.w2bf, (const float *)ls_.r1, sa, corr, (const FState *)d_st_);
  else
    launch_k(false, k_nn_infer<8>, TL.n, 64, infer_smem<8>(), stream_, topo_, c32_, TL, (const float *)ls_.w,
             (const __nv_bfloat16 *)ls_.w2bf, (const float *)ls_.r1, sa, corr, (const FState *)d_st_);
}

}  // namespace sayaka_gb300
