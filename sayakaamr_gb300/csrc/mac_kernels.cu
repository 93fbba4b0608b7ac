// Stencil, smoother and inter-level transfer kernels of the MAC solver.
//
// Every kernel works on one block list (a tower, one level of a tower, or a
// tree level) in a single launch, one thread per (block, cell).  Values that
// the reference obtains through ghost-cell fills and coarse/fine flux
// registers are gathered directly:
//   FINE_FINE face : the neighbour block's boundary cell
//                    (src/SayakaFillPatch.cpp:92-190)
//   FINE_CRSE face : the coarse leaf behind the parent's face, injected
//                    (src/SayakaFillPatch.cpp:192-299, src/SayakaInterpPatch.cpp:157-189)
//   CRSE_FINE face : sum over the fine faces of T_fine * phi_fine, i.e. the
//                    fine-side save + RESTRICT_SUM + copy of
//                    src/SayakaTower.cpp:298-415, src/SayakaInterpPatch.cpp:627-691
// The arithmetic is written operation by operation in the reference's order
// (src/SayakaMacOperator.cpp:1115-1459) and this file is compiled without
// FMA contraction, so FP64 results are bit-identical to the reference's.
#include <algorithm>
#include <cstdint>

#include "mac_device.h"
#include "mac_stencil.cuh"
#include "launch.cuh"

namespace sayaka_gb300 {

namespace {

constexpr int kThreads = 256;
using namespace stencil;

// ---------------------------------------------------------------------------
// MAC operator L(phi) = (phi_c*sum T - sum T*phi_nb) / (dv*vf)
// (src/SayakaMacOperator.cpp:1325-1459); residual variant
// r = rhs - L(phi) (src/SayakaMacUtil.cpp:9-49)
template <typename T, int ND>
__global__ void __launch_bounds__(kThreads) k_apply(Topo t, Coef<T> c, BlockList L, const T *__restrict__ x,
                                                    T *__restrict__ y, const T *__restrict__ rhs, const int *guard) {
  pdl_enter();
  if (guard && *guard) return;
  const int ncell = t.ncell;
  const long total = (long)L.n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell);
    const int ci = (int)(it - (long)p * ncell);
    const int b = L.blocks[p];
    if (block_off(L, b)) continue;
    const long q = (long)b * ncell + ci;
    T out = apply_cell<T, ND>(t, c, b, L.ftypes[p], ci, x);
    if (rhs) out = c.vf[q] > 0 ? rhs[q] - out : (T)0;
    y[q] = out;
  }
}

// ---------------------------------------------------------------------------
// red-black Gauss-Seidel, one colour over one level of a tower
// (src/SayakaMacOperator.cpp:1191-1323).  Colour = (i+j+k)%2 in block-local
// indices; nb is even so colours match across same-level block faces.
template <typename T, int ND>
__global__ void __launch_bounds__(kThreads) k_smooth(Topo t, Coef<T> c, BlockList L, int color, T *__restrict__ phi,
                                                     const T *__restrict__ rhs, const int *guard) {
  pdl_enter();
  if (guard && *guard) return;
  const int nhalf = t.ncell >> 1;
  const long total = (long)L.n * nhalf;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / nhalf);
    int ijk[3];
    color_cell<ND>((int)(it - (long)p * nhalf), t.nb, color, ijk);
    smooth_cell<T, ND>(t, c, L.blocks[p], L.ftypes[p], ijk, phi, rhs);
  }
}

// the device solve's smoother (smooth_cell_fast): blockIdx.y walks the
// blocks of the list, blockIdx.x the chunks of a block's half cells, so the
// block id and face types are uniform across a CTA and no thread divides
template <typename T, int ND, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_rbgs(Topo t, Coef<T> c, BlockList L, int color,
                                                         T *__restrict__ phi, const T *__restrict__ rhs,
                                                         const int *guard) {
  pdl_enter();
  if (guard && *guard) return;
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= (t.ncell >> 1)) return;
  int ijk[3];
  color_cell_fast<ND>(h, t, color, ijk);
  for (int p = blockIdx.y; p < L.n; p += gridDim.y) {
    const long fo = (long)p * t.ncell;
    if (L.stc && block_off(L, L.hx ? L.hx[(long)p * kHX + kHXBlock] : L.blocks[p])) continue;
    if (L.hx) {
      const int *e = L.hx + (long)p * kHX;
      smooth_cell_fast<T, ND>(t, c, e[kHXBlock], (uint16_t)(e[kHXInfo] & 0xffff), ijk, phi, rhs,
                              L.sa ? L.sa + fo : nullptr, L.ia ? L.ia + fo : nullptr, e);
    } else {
      smooth_cell_fast<T, ND>(t, c, L.blocks[p], L.ftypes[p], ijk, phi, rhs, L.sa ? L.sa + fo : nullptr,
                              L.ia ? L.ia + fo : nullptr);
    }
  }
}

// the same sweep with CPT cells per thread, the same cell of CPT blocks
// (entries p, p + G, ..., G = gridDim.y): every cell's operands are gathered
// before any is updated, so that a thread keeps CPT cells' loads in flight
// (smooth_gather / smooth_update: the values of smooth_cell_fast)
template <typename T, int ND, int MINB, int CPT>
__global__ void __launch_bounds__(kThreads, MINB) k_rbgs_ilp(Topo t, Coef<T> c, BlockList L, int color,
                                                             T *__restrict__ phi, const T *__restrict__ rhs,
                                                             const int *guard) {
  pdl_enter();
  if (guard && *guard) return;
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= (t.ncell >> 1)) return;
  int ijk[3];
  color_cell_fast<ND>(h, t, color, ijk);
  const int G = gridDim.y;
  for (int p0 = blockIdx.y; p0 < L.n; p0 += CPT * G) {
    SmoothOps<T, ND> o[CPT];
    bool on[CPT];
#pragma unroll
    for (int k = 0; k < CPT; k++) {
      const int p = p0 + k * G;
      on[k] = false;
      if (p >= L.n) continue;
      const long fo = (long)p * t.ncell;
      const int *e = L.hx ? L.hx + (long)p * kHX : nullptr;
      const int b = e ? e[kHXBlock] : L.blocks[p];
      if (L.stc && block_off(L, b)) continue;
      const uint16_t ft = e ? (uint16_t)(e[kHXInfo] & 0xffff) : L.ftypes[p];
      smooth_gather<T, ND>(t, c, b, ft, ijk, phi, rhs, L.sa ? L.sa + fo : nullptr, L.ia ? L.ia + fo : nullptr, e,
                           o[k]);
      on[k] = true;
    }
#pragma unroll
    for (int k = 0; k < CPT; k++)
      if (on[k]) smooth_update<T, ND>(c, o[k], phi);
  }
}

// (fluid: block b is known to have vf = 1 everywhere)
template <typename T, int ND>
__device__ __forceinline__ T prolonged_value(const Topo &t, const Coef<T> &c, int b, const int ijk[3],
                                             const T *__restrict__ phi, int pw = -1, bool fluid = false) {
  const int nb = t.nb, half = nb >> 1;
  const int P = pw >= 0 ? pw >> 3 : t.parent[b], wc = pw >= 0 ? pw & 7 : t.which_child[b];
  int pc[3] = {0, 0, 0};
  for (int q = 0; q < ND; q++) pc[q] = ((wc >> q) & 1) * half + (ijk[q] >> 1);
  const long q = (long)b * t.ncell + encode(ijk, nb);
  return (fluid || c.vf[q] > 0) ? phi[(long)P * t.ncell + encode(pc, nb)] : (T)0;
}

// One warp updates the cells of colour `color` of one 16x16 block of a 2D
// FP32 sweep, any block: lane l holds row l/2, columns 8(l%2) .. +7 in
// registers, v[] (PROLONG: the block's values prolonged from its parent,
// masked by vf, as k_prolong_red's tile; else phi), neighbours inside the
// block from registers and shuffles, every boundary face by its type as
// smooth_cell_fast and k_prolong_red take it (same-level: the neighbour's
// value, prolonged from its own parent when PROLONG; coarse/fine: the
// coarse ghost or the fine-side sum; physical: the diagonal term), face
// coefficients from the block record or the face arrays; the whole block is
// written back.  Per cell the operations are those of smooth_cell_fast /
// k_prolong_red in the same order: the same bits.
template <bool PROLONG>
__device__ __forceinline__ void warp_block16(const Topo &t, const Coef<float> &c, int b, uint16_t ft, const int *e,
                                             int color, float *__restrict__ phi, const float *__restrict__ rhs,
                                             int lane) {
  constexpr int NB = 16, NC = 256;
  const int j = lane >> 1, hh = lane & 1, c0 = 8 * hh;
  const long cb = (long)b * NC, fb = (long)b * t.nfb;
  const float *u = uniform_of(c, b);
  float v[8];
  if constexpr (PROLONG) {
    const int pw = e ? e[kHXPar + 6] : t.parent[b] * 8 + t.which_child[b];
    const int P = pw >> 3, wc = pw & 7;
    const float4 q4 = *reinterpret_cast<const float4 *>(phi + (long)P * NC + (8 * ((wc >> 1) & 1) + (j >> 1)) * NB +
                                                         8 * (wc & 1) + 4 * hh);
    const float pv[4] = {q4.x, q4.y, q4.z, q4.w};
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = (u || c.vf[cb + j * NB + c0 + k] > 0) ? pv[k >> 1] : 0.f;
  } else {
    const float4 *src = reinterpret_cast<const float4 *>(phi + cb + j * NB + c0);
    const float4 p0 = src[0], p1 = src[1];
    v[0] = p0.x, v[1] = p0.y, v[2] = p0.z, v[3] = p0.w, v[4] = p1.x, v[5] = p1.y, v[6] = p1.z, v[7] = p1.w;
  }
  const float4 *rsrc = reinterpret_cast<const float4 *>(rhs + cb + j * NB + c0);
  const float4 r0 = rsrc[0], r1 = rsrc[1];
  const float r[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
  const float dv = geom(c, b, 6);
  const float from_left = __shfl_up_sync(0xffffffffu, v[7], 1);
  const float from_right = __shfl_down_sync(0xffffffffu, v[0], 1);
  const int par = (color + j) & 1;
  // value across boundary face f of cell ijk (same-level, coarse/fine)
  auto across = [&](int f, const int ijk[3], int ty) -> float {
    if (ty == 0) {
      const int n = e ? e[f] : t.neighbor[b * 6 + f];
      int ni[3] = {ijk[0], ijk[1], 0};
      ni[f >> 1] = (f & 1) ? 0 : NB - 1;
      if constexpr (PROLONG)
        return prolonged_value<float, 2>(t, c, n, ni, phi, e ? e[kHXPar + f] : -1);
      else
        return phi[(long)n * NC + ni[0] + NB * ni[1]];
    }
    return fine_crse_ghost<float, 2, false>(t, b, f, ijk, phi, e);
  };
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const float dnk = __shfl_up_sync(0xffffffffu, v[k], 2);
    const float upk = __shfl_down_sync(0xffffffffu, v[k], 2);
    if ((k & 1) != par) continue;
    const int i = c0 + k;
    const int ijk[3] = {i, j, 0};
    float diag = c.alpha * dv;
    float off = 0.f;
#pragma unroll
    for (int f = 0; f < 4; f++) {
      const int d = f >> 1, sd = f & 1;
      const bool bnd = d == 0 ? (sd ? i == NB - 1 : i == 0) : (sd ? j == NB - 1 : j == 0);
      const int fx = d == 0 ? i + sd + (NB + 1) * j : i + NB * (j + sd);
      if (!bnd) {
        const float coef = u ? u[d] : c.tff[d][fb + fx];
        float nbv;
        if (f == 0)
          nbv = k > 0 ? v[k - 1] : from_left;
        else if (f == 1)
          nbv = k < 7 ? v[k + 1] : from_right;
        else if (f == 2)
          nbv = dnk;
        else
          nbv = upk;
        diag += coef;
        off = fma_t(coef, nbv, off);
        continue;
      }
      const int ty = face_type_of(ft, f);
      if (ty == 0) {
        const float coef = u ? u[d] : c.tff[d][fb + fx];
        diag += coef;
        off = fma_t(coef, across(f, ijk, 0), off);
      } else if (ty == 1) {
        if (t.bc_type[b * 6 + f] != kBCNeumann) diag += (u ? u[d] : c.tff[d][fb + fx]) * 2.0f;
      } else if (ty == 2) {
        const float coef = cf_coef(c, t, b, d, fx, 1.5f);
        diag += coef;
        off = fma_t(coef, across(f, ijk, 2), off);
      } else {
        diag += cf_coef(c, t, b, d, fx, 0.75f);
        off = fma_t(1.0f, crse_fine_sum<float, 2, false>(t, c, b, f, ijk, phi, e), off);
      }
    }
    const float vfv = u ? 1.0f : c.vf[cb + j * NB + i];
    v[k] = (vfv > 0.f && diag > 0.f) ? relax(c.omega, fast_div(fma_t(r[k] * dv, vfv, off), diag), v[k]) : 0.f;
  }
  float4 *dst = reinterpret_cast<float4 *>(phi + cb + j * NB + c0);
  dst[0] = make_float4(v[0], v[1], v[2], v[3]);
  dst[1] = make_float4(v[4], v[5], v[6], v[7]);
}

// prolongation of a level fused with its first red sweep (k_prolong_red's
// values), 2D FP32 16x16 blocks, one warp per block of L, then one warp per
// block of X for the red sweep of the coarser same-parity sublevels
template <int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_prolong_red_warp16(Topo t, Coef<float> c, BlockList L,
                                                                       float *__restrict__ phi,
                                                                       const float *__restrict__ rhs,
                                                                       const int *guard, BlockList X) {
  pdl_enter();
  if (guard && *guard) return;
  const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
  for (int p = blockIdx.x * warps + (threadIdx.x >> 5); p < L.n + X.n; p += gridDim.x * warps) {
    const bool top = p < L.n;
    const BlockList &Q = top ? L : X;
    const int q = top ? p : p - L.n;
    const int *e = Q.hx ? Q.hx + (long)q * kHX : nullptr;
    const int b = e ? e[kHXBlock] : Q.blocks[q];
    if (Q.stc && block_off(Q, b)) continue;  // uniform over the warp
    const uint16_t ft = e ? (uint16_t)(e[kHXInfo] & 0xffff) : Q.ftypes[q];
    if (top)
      warp_block16<true>(t, c, b, ft, e, 0, phi, rhs, lane);
    else
      warp_block16<false>(t, c, b, ft, e, 0, phi, rhs, lane);
  }
}

// The 2D sweep of 16x16 blocks with one warp per block: lane l holds row
// l/2, columns 8(l%2) .. 8(l%2)+7 of phi and rhs in registers (two 16-byte
// loads each), neighbours inside the block come from the lane's own
// registers and from lanes l-1, l+1 (columns) and l-2, l+2 (rows) by
// shuffles, and the block is written back whole (the cells of the other
// colour with their unchanged values) with two 16-byte stores per lane.  The
// fast path takes constant-coefficient blocks (a block record) whose faces
// are all same-level or physical; their halo cells are loaded from the
// neighbour block (one value per lane for the side faces, two 16-byte loads
// for the bottom and top rows).  Any other block is swept cell by cell with
// smooth_cell_fast.  Per cell the arithmetic is smooth_cell_fast's, face by
// face in the same order, so every path gives the same bits.
template <int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_rbgs_warp16(Topo t, Coef<float> c, BlockList L, int color,
                                                                float *__restrict__ phi, const float *__restrict__ rhs,
                                                                const int *guard) {
  pdl_enter();
  if (guard && *guard) return;
  constexpr int NB = 16, NC = 256;
  const int lane = threadIdx.x & 31;
  const int warps = blockDim.x >> 5;
  const int j = lane >> 1, hh = lane & 1, c0 = 8 * hh;
  for (int p = blockIdx.x * warps + (threadIdx.x >> 5); p < L.n; p += gridDim.x * warps) {
    const int *e = L.hx ? L.hx + (long)p * kHX : nullptr;
    const int b = e ? e[kHXBlock] : L.blocks[p];
    if (L.stc && block_off(L, b)) continue;  // uniform over the warp
    const uint16_t ft = e ? (uint16_t)(e[kHXInfo] & 0xffff) : L.ftypes[p];
    const float *u = uniform_of(c, b);
    bool fast = u != nullptr;
#pragma unroll
    for (int f = 0; f < 4; f++) fast = fast && face_type_of(ft, f) <= 1;
    if (!fast) {
      // four cells of the colour per lane, as k_rbgs does them (measured
      // faster for these blocks than warp_block16's register form)
      for (int k = 0; k < 4; k++) {
        const int h = lane * 4 + k;  // half-cell index 0..127
        int ijk[3];
        color_cell_fast<2>(h, t, color, ijk);
        smooth_cell_fast<float, 2>(t, c, b, ft, ijk, phi, rhs, nullptr, nullptr, e);
      }
      continue;
    }
    const long cb = (long)b * NC;
    const float4 *src = reinterpret_cast<const float4 *>(phi + cb + j * NB + c0);
    const float4 *rsrc = reinterpret_cast<const float4 *>(rhs + cb + j * NB + c0);
    const float4 p0 = src[0], p1 = src[1], r0 = rsrc[0], r1 = rsrc[1];
    float v[8] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w};
    const float r[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
    const int ty[4] = {face_type_of(ft, 0), face_type_of(ft, 1), face_type_of(ft, 2), face_type_of(ft, 3)};
    // halo values (same-level faces only; physical faces have no off-diagonal term)
    float hl = 0.f, hr = 0.f;
    if (hh == 0 && ty[0] == 0) {
      const int n = e ? e[0] : t.neighbor[b * 6 + 0];
      hl = phi[(long)n * NC + j * NB + (NB - 1)];
    }
    if (hh == 1 && ty[1] == 0) {
      const int n = e ? e[1] : t.neighbor[b * 6 + 1];
      hr = phi[(long)n * NC + j * NB];
    }
    float hv[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if ((j == 0 && ty[2] == 0) || (j == NB - 1 && ty[3] == 0)) {
      const int f = j == 0 ? 2 : 3;
      const int n = e ? e[f] : t.neighbor[b * 6 + f];
      const int row = j == 0 ? NB - 1 : 0;
      const float4 *hs = reinterpret_cast<const float4 *>(phi + (long)n * NC + row * NB + c0);
      const float4 a0 = hs[0], a1 = hs[1];
      hv[0] = a0.x, hv[1] = a0.y, hv[2] = a0.z, hv[3] = a0.w, hv[4] = a1.x, hv[5] = a1.y, hv[6] = a1.z, hv[7] = a1.w;
    }
    const float dv = geom(c, b, 6);
    const float T0 = u[0], T1 = u[1];
    const bool dir[4] = {t.bc_type[b * 6 + 0] != kBCNeumann, t.bc_type[b * 6 + 1] != kBCNeumann,
                         t.bc_type[b * 6 + 2] != kBCNeumann, t.bc_type[b * 6 + 3] != kBCNeumann};
    // neighbours across lanes: v[7] of the left half, v[0] of the right half
    const float from_left = __shfl_up_sync(0xffffffffu, v[7], 1);
    const float from_right = __shfl_down_sync(0xffffffffu, v[0], 1);
    const int par = (color + j) & 1;  // column parity of this row's cells of the colour
#pragma unroll
    for (int k = 0; k < 8; k++) {
      // rows j-1 and j+1 from lanes l-2 and l+2; their column-k cell has the
      // other colour (their row parity differs), so it is still the old value
      // even after those lanes updated their own cells in place
      const float dnk = __shfl_up_sync(0xffffffffu, v[k], 2);
      const float upk = __shfl_down_sync(0xffffffffu, v[k], 2);
      if ((k & 1) != par) continue;
      const int i = c0 + k;
      float diag = c.alpha * dv;
      float off = 0.f;
      // f = 0: left
      if (i > 0 || ty[0] == 0) {
        const float nbv = k > 0 ? v[k - 1] : (hh == 1 ? from_left : hl);
        diag += T0;
        off = fma_t(T0, nbv, off);
      } else if (dir[0]) {
        diag += T0 * 2.0f;
      }
      // f = 1: right
      if (i < NB - 1 || ty[1] == 0) {
        const float nbv = k < 7 ? v[k + 1] : (hh == 0 ? from_right : hr);
        diag += T0;
        off = fma_t(T0, nbv, off);
      } else if (dir[1]) {
        diag += T0 * 2.0f;
      }
      // f = 2: down
      if (j > 0 || ty[2] == 0) {
        const float nbv = j > 0 ? dnk : hv[k];
        diag += T1;
        off = fma_t(T1, nbv, off);
      } else if (dir[2]) {
        diag += T1 * 2.0f;
      }
      // f = 3: up
      if (j < NB - 1 || ty[3] == 0) {
        const float nbv = j < NB - 1 ? upk : hv[k];
        diag += T1;
        off = fma_t(T1, nbv, off);
      } else if (dir[3]) {
        diag += T1 * 2.0f;
      }
      v[k] = diag > 0.f ? relax(c.omega, fast_div(fma_t(r[k] * dv, 1.0f, off), diag), v[k]) : 0.f;
    }
    float4 *dst = reinterpret_cast<float4 *>(phi + cb + j * NB + c0);
    dst[0] = make_float4(v[0], v[1], v[2], v[3]);
    dst[1] = make_float4(v[4], v[5], v[6], v[7]);
  }
}

// the cell-by-cell sweep of one block (four cells of the colour per lane)
__device__ __forceinline__ void warp16_slow_block(const Topo &t, const Coef<float> &c, int b, uint16_t ft, int color,
                                               float *__restrict__ phi, const float *__restrict__ rhs, const int *e,
                                               int lane) {
  for (int k = 0; k < 4; k++) {
    const int h = lane * 4 + k;
    int ijk[3];
    color_cell_fast<2>(h, t, color, ijk);
    smooth_cell_fast<float, 2>(t, c, b, ft, ijk, phi, rhs, nullptr, nullptr, e);
  }
}

// k_rbgs_warp16 with every load of a block issued before its first branch:
// the descriptor (two vector loads), then at once the block record, dv, the
// face BC types, phi and rhs and the halo values (their ids and face types
// come with the descriptor), and only then the problem's done flag, the
// fast-path test and the sweep.  The latency of a block is then about three
// dependent loads (descriptor, data, done flag) instead of six.  Same
// arithmetic, same bits.  Needs the list's halo descriptors.
template <int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_rbgs_warp16_flat(Topo t, Coef<float> c, BlockList L, int color,
                                                                     float *__restrict__ phi,
                                                                     const float *__restrict__ rhs,
                                                                     const int *guard) {
  pdl_enter();
  if (guard && *guard) return;
  constexpr int NB = 16, NC = 256;
  const int lane = threadIdx.x & 31;
  const int warps = blockDim.x >> 5;
  const int j = lane >> 1, hh = lane & 1, c0 = 8 * hh;
  for (int p = blockIdx.x * warps + (threadIdx.x >> 5); p < L.n; p += gridDim.x * warps) {
    const int *e = L.hx + (long)p * kHX;
    const int4 nb4 = *reinterpret_cast<const int4 *>(e);           // face neighbours 0..3
    const int2 ib = *reinterpret_cast<const int2 *>(e + kHXInfo);  // info, block
    const int b = ib.y;
    const uint16_t ft = (uint16_t)(ib.x & 0xffff);
    const int ty[4] = {face_type_of(ft, 0), face_type_of(ft, 1), face_type_of(ft, 2), face_type_of(ft, 3)};
    const long cb = (long)b * NC;
    // ---- every load of the block
    const int comp = L.stc ? L.comp[b] : 0;
    const float4 rec = c.ut ? *reinterpret_cast<const float4 *>(c.ut + (long)b * kUni) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float dv = geom(c, b, 6);
    const int2 bc01 = *reinterpret_cast<const int2 *>(t.bc_type + b * 6);
    const int2 bc23 = *reinterpret_cast<const int2 *>(t.bc_type + b * 6 + 2);
    const int par = (color + j) & 1;  // column parity of this row's cells of the colour
    const float4 *src = reinterpret_cast<const float4 *>(phi + cb + j * NB + c0);
    const float4 *rsrc = reinterpret_cast<const float4 *>(rhs + cb + j * NB + c0);
    const float4 p0 = src[0], p1 = src[1], r0 = rsrc[0], r1 = rsrc[1];
    float hl = 0.f, hr = 0.f;
    if (hh == 0 && ty[0] == 0) hl = phi[(long)nb4.x * NC + j * NB + (NB - 1)];
    if (hh == 1 && ty[1] == 0) hr = phi[(long)nb4.y * NC + j * NB];
    float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0;
    if ((j == 0 && ty[2] == 0) || (j == NB - 1 && ty[3] == 0)) {
      const int n = j == 0 ? nb4.z : nb4.w;
      const float4 *hs = reinterpret_cast<const float4 *>(phi + (long)n * NC + (j == 0 ? NB - 1 : 0) * NB + c0);
      a0 = hs[0];
      a1 = hs[1];
    }
    // ---- then the decisions
    if (L.stc && L.stc[comp].done) continue;  // uniform over the warp
    bool fast = c.ut != nullptr && __float_as_uint(rec.w) != 0u;
#pragma unroll
    for (int f = 0; f < 4; f++) fast = fast && ty[f] <= 1;
    if (!fast) {
      warp16_slow_block(t, c, b, ft, color, phi, rhs, e, lane);
      continue;
    }
    float v[8] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w};
    // rhs and the halo row of the colour's four cells only (cell k = 2q + par)
    const float rs[4] = {par ? r0.y : r0.x, par ? r0.w : r0.z, par ? r1.y : r1.x, par ? r1.w : r1.z};
    const float hs4[4] = {par ? a0.y : a0.x, par ? a0.w : a0.z, par ? a1.y : a1.x, par ? a1.w : a1.z};
    const float T0 = rec.x, T1 = rec.y;
    const bool dir[4] = {bc01.x != kBCNeumann, bc01.y != kBCNeumann, bc23.x != kBCNeumann, bc23.y != kBCNeumann};
    const float from_left = __shfl_up_sync(0xffffffffu, v[7], 1);
    const float from_right = __shfl_down_sync(0xffffffffu, v[0], 1);
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const float dnk = __shfl_up_sync(0xffffffffu, v[k], 2);
      const float upk = __shfl_down_sync(0xffffffffu, v[k], 2);
      if ((k & 1) != par) continue;
      const int i = c0 + k;
      float diag = c.alpha * dv;
      float off = 0.f;
      if (i > 0 || ty[0] == 0) {
        const float nbv = k > 0 ? v[k - 1] : (hh == 1 ? from_left : hl);
        diag += T0;
        off = fma_t(T0, nbv, off);
      } else if (dir[0]) {
        diag += T0 * 2.0f;
      }
      if (i < NB - 1 || ty[1] == 0) {
        const float nbv = k < 7 ? v[k + 1] : (hh == 0 ? from_right : hr);
        diag += T0;
        off = fma_t(T0, nbv, off);
      } else if (dir[1]) {
        diag += T0 * 2.0f;
      }
      if (j > 0 || ty[2] == 0) {
        const float nbv = j > 0 ? dnk : hs4[k >> 1];
        diag += T1;
        off = fma_t(T1, nbv, off);
      } else if (dir[2]) {
        diag += T1 * 2.0f;
      }
      if (j < NB - 1 || ty[3] == 0) {
        const float nbv = j < NB - 1 ? upk : hs4[k >> 1];
        diag += T1;
        off = fma_t(T1, nbv, off);
      } else if (dir[3]) {
        diag += T1 * 2.0f;
      }
      v[k] = diag > 0.f ? relax(c.omega, fast_div(fma_t(rs[k >> 1] * dv, 1.0f, off), diag), v[k]) : 0.f;
    }
    float4 *dst = reinterpret_cast<float4 *>(phi + cb + j * NB + c0);
    dst[0] = make_float4(v[0], v[1], v[2], v[3]);
    dst[1] = make_float4(v[4], v[5], v[6], v[7]);
  }
}

// ---------------------------------------------------------------------------
// volume-weighted restriction onto the non-leaf blocks of a level:
// coarse = avg(fine*vf_fine)/vf_coarse (src/SayakaMacIB.cpp:157-232 with
// src/SayakaInterpPatch.cpp:398-444)
template <typename T, int ND>
__global__ void __launch_bounds__(kThreads) k_restrict(Topo t, Coef<T> c, BlockList L, T *__restrict__ phi,
                                                       const int *guard) {
  pdl_enter();
  if (guard && *guard) return;
  const int ncell = t.ncell;
  const long total = (long)L.n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell);
    if (block_off(L, L.blocks[p])) continue;
    restrict_cell<T, ND>(t, c, L.blocks[p], (int)(it - (long)p * ncell), phi, L.links ? L.links + (long)p * 8 : nullptr);
  }
}

// masked injection onto every block of a level (src/SayakaMacIB.cpp:234-283)
template <typename T, int ND>
__global__ void __launch_bounds__(kThreads) k_prolong(Topo t, Coef<T> c, BlockList L, T *__restrict__ phi,
                                                      const int *guard) {
  pdl_enter();
  if (guard && *guard) return;
  const int ncell = t.ncell;
  const long total = (long)L.n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell);
    if (block_off(L, L.blocks[p])) continue;
    prolong_cell<T, ND>(t, c, L.blocks[p], (int)(it - (long)p * ncell), phi, L.links ? L.links[p] : -1);
  }
}

// same-level face coefficient ((beta*ds)/dx)*B*a for every face of every block
template <typename T>
__global__ void k_face_coef(Topo t, const double *geom64, const T *b0, const T *b1, const T *b2, const T *a0,
                            const T *a1, const T *a2, double beta, T *t0, T *t1, T *t2) {
  const long per = (long)t.nfb;
  const long total = (long)t.nblocks * per * t.ndim;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int d = (int)(it / ((long)t.nblocks * per));
    const long r = it - (long)d * t.nblocks * per;
    const int b = (int)(r / per);
    const T *B = d == 0 ? b0 : (d == 1 ? b1 : b2);
    const T *A = d == 0 ? a0 : (d == 1 ? a1 : a2);
    T *O = d == 0 ? t0 : (d == 1 ? t1 : t2);
    const T ds = (T)geom64[b * 8 + 3 + d], dx = (T)geom64[b * 8 + d];
    T v = (T)beta * ds / dx;
    v = v * B[r];
    v = v * A[r];
    O[r] = v;
  }
}

// face flux -(phi_hi - phi_lo)/h on every face of direction `dir` of a tower
// (src/SayakaMacOperator.cpp:161-239 and :929-1025): FINE_BC faces get 0,
// FINE_CRSE faces use h = 1.5 dx with the injected coarse ghost, CRSE_FINE
// faces the average of the fine FINE_CRSE fluxes behind them (FLUX_SYNC_AVG).
template <int ND>
__global__ void k_flux(Topo t, Coef<double> c, BlockList L, int dir, const double *__restrict__ phi,
                       double *__restrict__ flux) {
  const int nb = t.nb, ncell = t.ncell, nfb = t.nfb;
  const long total = (long)L.n * nfb;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / nfb);
    const int fxi = (int)(it - (long)p * nfb);
    const int *hxe = L.hx ? L.hx + (long)p * kHX : nullptr;
    const int b = hxe ? hxe[kHXBlock] : L.blocks[p];
    const uint16_t ft = hxe ? (uint16_t)(hxe[kHXInfo] & 0xffff) : L.ftypes[p];
    // decode the face-centred index: dimension dir has nb+1 entries
    const int e0 = nb + (dir == 0), e1 = nb + (dir == 1);
    int fi[3];
    fi[0] = fxi % e0;
    fi[1] = ND >= 2 ? (fxi / e0) % e1 : 0;
    fi[2] = ND == 3 ? fxi / (e0 * e1) : 0;
    const int m = fi[dir];
    const double dh = c.geom[b * 8 + dir];
    const long cb = (long)b * ncell;
    double out;
    if (m > 0 && m < nb) {
      int hi[3] = {fi[0], fi[1], fi[2]}, lo[3] = {fi[0], fi[1], fi[2]};
      lo[dir] = m - 1;
      out = -(phi[cb + encode(hi, nb)] - phi[cb + encode(lo, nb)]) / dh;
    } else {
      const int s = m == 0 ? 0 : 1;
      const int f = 2 * dir + s;
      const int ty = face_type_of(ft, f);
      int own[3] = {fi[0], fi[1], fi[2]};
      own[dir] = s == 0 ? 0 : nb - 1;
      const double po = phi[cb + encode(own, nb)];
      if (ty == 1) {
        out = 0;
      } else if (ty == 0) {
        const double g = same_level_ghost(t, b, f, own, phi);
        out = s == 0 ? -(po - g) / dh : -(g - po) / dh;
      } else if (ty == 2) {
        const double g = fine_crse_ghost<double, ND>(t, b, f, own, phi);
        const double h = dh * 1.5;
        out = s == 0 ? -(po - g) / h : -(g - po) / h;
      } else {
        // average of the fine FINE_CRSE fluxes on this face
        const int N = t.neighbor[b * 6 + f];
        const int half = nb >> 1;
        int cidx = (1 - s) << dir, base[3] = {0, 0, 0}, tq[2] = {0, 0}, nt = 0;
        for (int q = 0; q < ND; q++) {
          if (q == dir) continue;
          const int sq = own[q] >= half ? 1 : 0;
          cidx |= sq << q;
          base[q] = 2 * (own[q] - sq * half);
          tq[nt++] = q;
        }
        const int F = t.child[N * 8 + cidx];
        const double dhf = c.geom[F * 8 + dir] * 1.5;
        int fc[3];
        fc[dir] = s == 1 ? 0 : nb - 1;
        double sum = 0;
        for (int a1 = 0; a1 < (ND == 3 ? 2 : 1); a1++)
          for (int a0 = 0; a0 < 2; a0++) {
            fc[tq[0]] = base[tq[0]] + a0;
            if (ND == 3) fc[tq[1]] = base[tq[1]] + a1;
            if (ND == 2) fc[2] = 0;
            const double pf = phi[(long)F * ncell + encode(fc, nb)];
            // the fine block's ghost toward b is b's boundary cell `own`
            const double fl = s == 1 ? -(pf - po) / dhf : -(po - pf) / dhf;
            sum += fl;
          }
        out = sum * (ND == 3 ? 0.25 : 0.5);
      }
    }
    flux[(long)b * nfb + fxi] = out;
  }
}

// Dirichlet / SimpleFill lift of the right-hand side from BC values held in
// the ghost layer of phi (src/SayakaMacOperator.cpp:1470-1594)
template <int ND>
__global__ void k_fix_bc(Topo t, Coef<double> c, BlockList L, const double *__restrict__ phig, int ng,
                         double *__restrict__ rhs) {
  const int nb = t.nb, ncell = t.ncell;
  const int G = nb + 2 * ng;
  const long gstride = ND == 3 ? (long)G * G * G : (long)G * G;
  const long total = (long)L.n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell);
    const int ci = (int)(it - (long)p * ncell);
    const int *hxe = L.hx ? L.hx + (long)p * kHX : nullptr;
    const int b = hxe ? hxe[kHXBlock] : L.blocks[p];
    const uint16_t ft = hxe ? (uint16_t)(hxe[kHXInfo] & 0xffff) : L.ftypes[p];
    int ijk[3];
    decode<ND>(ci, nb, ijk);
    const double dv = c.geom[b * 8 + 6];
    const long q = (long)b * ncell + ci;
    double r = rhs[q];
    for (int f = 0; f < 2 * ND; f++) {
      if (face_type_of(ft, f) != 1) continue;
      const int d = f >> 1, s = f & 1;
      if (ijk[d] != (s ? nb - 1 : 0)) continue;
      const int bct = t.bc_type[b * 6 + f];
      auto gidx = [&](int i, int j, int k) {
        return (long)b * gstride + (i + ng) + (long)G * ((j + ng) + (long)G * (ND == 3 ? k + ng : 0));
      };
      const double p0 = phig[gidx(ijk[0], ijk[1], ijk[2])];
      int gi[3] = {ijk[0], ijk[1], ijk[2]};
      gi[d] += s ? 1 : -1;
      const double p1 = phig[gidx(gi[0], gi[1], gi[2])];
      const int fx = face_index(d, ijk, s, nb);
      double coef = c.beta * c.geom[b * 8 + 3 + d] / c.geom[b * 8 + d];
      coef *= c.bcoef[d][(long)b * t.nfb + fx];
      coef *= c.afrac[d][(long)b * t.nfb + fx];
      double corr = 0;
      if (bct == kBCDirichlet) {
        const double pbc = 0.5 * (p0 + p1);
        corr = pbc * 2.0 * coef;
      } else if (bct == kBCSimpleFill) {
        const double pbc = p1;
        corr = pbc * 2.0 * coef;
      }
      const double vfv = c.vf[q];
      if (vfv > 0) {
        corr /= (dv * vfv);
        r += corr;
      }
    }
    rhs[q] = r;
  }
}

inline int grid_for(long work) {
  long g = (work + kThreads - 1) / kThreads;
  if (g < 1) g = 1;
  if (g > 152 * 32) g = 152 * 32;
  return (int)g;
}

}  // namespace

template <typename T>
void launch_face_coef(const Topo &t, const double *geom64, const T *bcoef[3], const T *afrac[3], double beta,
                      T *tff[3], cudaStream_t s) {
  const long work = (long)t.nblocks * t.nfb * t.ndim;
  if (work == 0) return;
  k_face_coef<T><<<grid_for(work), kThreads, 0, s>>>(t, geom64, bcoef[0], bcoef[1], bcoef[2], afrac[0], afrac[1],
                                                     afrac[2], beta, tff[0], tff[1], tff[2]);
}

template <typename T>
void launch_apply(const Topo &t, const Coef<T> &c, const BlockList &L, const T *x, T *y, const T *rhs,
                  const int *guard, cudaStream_t s, bool pdl) {
  const long work = (long)L.n * t.ncell;
  if (work == 0) return;
  if (t.ndim == 2)
    launch_k(pdl, k_apply<T, 2>, grid_for(work), kThreads, 0, s, t, c, L, x, y, rhs, guard);
  else
    launch_k(pdl, k_apply<T, 3>, grid_for(work), kThreads, 0, s, t, c, L, x, y, rhs, guard);
}

// The same sweep with the block staged in shared memory: one CTA per block
// of the list loads the block's phi tile (full sectors) and, once per
// boundary face cell of the sweep's colour, the face's contribution
// (diagonal part hc, off-diagonal factor hk and value hv: FINE_FINE and
// FINE_CRSE give T and the gathered ghost, CRSE_FINE the coarse-side T, 1 and
// the fine-side sum, physical faces 0 or 2T and 0); cells then read their
// neighbours from the tile.  Every value is combined in smooth_cell_fast's
// order with the same operations, so the result is bit-identical.  The tile
// (both colours, black cells unchanged) is written back whole.
template <typename T, int ND, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_rbgs_tile(Topo t, Coef<T> c, BlockList L, int color,
                                                              T *__restrict__ phi, const T *__restrict__ rhs,
                                                              const int *guard) {
  extern __shared__ __align__(16) unsigned char rbgs_smem[];
  pdl_enter();
  if (guard && *guard) return;
  const int nb = t.nb, ncell = t.ncell, nhalf = ncell >> 1;
  const int nface = ND == 3 ? nb * nb : nb;  // cells on one block face
  T *tile = reinterpret_cast<T *>(rbgs_smem);
  T *hc = tile + ncell;
  T *hk = hc + 2 * ND * nface;
  T *hv = hk + 2 * ND * nface;
  for (int p = blockIdx.x; p < L.n; p += gridDim.x) {
    const int *hxe = L.hx ? L.hx + (long)p * kHX : nullptr;
    const int b = hxe ? hxe[kHXBlock] : L.blocks[p];
    if (block_off(L, b)) continue;  // uniform over the CTA
    const uint16_t ft = hxe ? (uint16_t)(hxe[kHXInfo] & 0xffff) : L.ftypes[p];
    const long cb = (long)b * ncell;
    const long fb = (long)b * t.nfb;
    if ((ncell & 3) == 0 && sizeof(T) == 4) {
      const float4 *src = reinterpret_cast<const float4 *>(phi + cb);
      float4 *dst = reinterpret_cast<float4 *>(tile);
      for (int i = threadIdx.x; i < (ncell >> 2); i += blockDim.x) dst[i] = src[i];
    } else {
      for (int i = threadIdx.x; i < ncell; i += blockDim.x) tile[i] = phi[cb + i];
    }
    // boundary contributions of the cells of this colour
    for (int e = threadIdx.x; e < 2 * ND * nface; e += blockDim.x) {
      const int f = e / nface, m = e - f * nface;
      const int d = f >> 1, s = f & 1;
      int ijk[3];
      ijk[d] = s ? nb - 1 : 0;
      const int q0 = d == 0 ? 1 : 0, q1 = d == 2 ? 1 : 2;
      ijk[q0] = m % nb;
      if (ND == 3) ijk[q1] = m / nb;
      else if (d != 2) ijk[2] = 0;
      if (ND == 2) ijk[2] = 0;
      if (((ijk[0] + ijk[1] + ijk[2]) & 1) != color) continue;
      int fx;
      if (d == 0)
        fx = ijk[0] + s + (nb + 1) * (ijk[1] + nb * ijk[2]);
      else if (d == 1)
        fx = ijk[0] + nb * (ijk[1] + s + (nb + 1) * ijk[2]);
      else
        fx = encode(ijk, nb) + s * nb * nb;
      const int ty = face_type_of(ft, f);
      const T *u = uniform_of(c, b);
      T vc = 0, vk = 0, vv = 0;
      if (ty == 0) {
        vc = vk = u ? u[d] : c.tff[d][fb + fx];
        vv = same_level_ghost<T, false>(t, b, f, ijk, phi, hxe);
      } else if (ty == 1) {
        if (t.bc_type[b * 6 + f] != kBCNeumann) vc = (u ? u[d] : c.tff[d][fb + fx]) * (T)2.0;
      } else if (ty == 2) {
        vc = vk = cf_coef(c, t, b, d, fx, (T)1.5);
        vv = fine_crse_ghost<T, ND, false>(t, b, f, ijk, phi, hxe);
      } else {
        vc = cf_coef(c, t, b, d, fx, (T)0.75);
        vk = (T)1;
        vv = crse_fine_sum<T, ND, false>(t, c, b, f, ijk, phi, hxe);
      }
      hc[e] = vc;
      hk[e] = vk;
      hv[e] = vv;
    }
    __syncthreads();
    const T dv = geom(c, b, 6);
    const T *u = uniform_of(c, b);  // constant coefficients: no face or vf loads
    // a cell's global operands (face coefficients, rhs and vf or the FP64
    // factors) are gathered before any update: a thread with two cells has
    // both cells' loads in flight together (the shared-memory tile written
    // by the updates may alias the operand pointers for the compiler)
    struct Ops {
      int ijk[3], ci;
      T coef[2 * ND], r, v;
      double sa, ia;
    };
    auto gather = [&](int h, Ops &o) {
      color_cell_fast<ND>(h, t, color, o.ijk);
      o.ci = t.lnb >= 0 ? o.ijk[0] + ((o.ijk[1] + (o.ijk[2] << t.lnb)) << t.lnb) : encode(o.ijk, nb);
#pragma unroll
      for (int f = 0; f < 2 * ND; f++) {
        const int d = f >> 1, s = f & 1;
        const bool bnd = s ? o.ijk[d] == nb - 1 : o.ijk[d] == 0;
        int fx;
        if (d == 0)
          fx = o.ijk[0] + s + (nb + 1) * (o.ijk[1] + nb * o.ijk[2]);
        else if (d == 1)
          fx = o.ijk[0] + nb * (o.ijk[1] + s + (nb + 1) * o.ijk[2]);
        else
          fx = o.ci + s * nb * nb;
        o.coef[f] = bnd ? (T)0 : (u ? u[d] : c.tff[d][fb + fx]);
      }
      o.r = rhs[cb + o.ci];
      if (sizeof(T) == 8 && L.sa) {
        bool inner = true;
#pragma unroll
        for (int q = 0; q < ND; q++) inner = inner && o.ijk[q] > 0 && o.ijk[q] < nb - 1;
        if (u && inner) {
          o.sa = u[6];
          o.ia = u[7];
        } else {
          const long fo = (long)p * ncell + o.ci;
          o.sa = L.sa[fo];
          o.ia = L.ia[fo];
        }
        o.v = 0;
      } else {
        o.v = u ? (T)1 : c.vf[cb + o.ci];
        o.sa = o.ia = 0.0;
      }
    };
    auto update = [&](const Ops &o) {
      T diag = c.alpha * dv;
      T off = 0;
#pragma unroll
      for (int f = 0; f < 2 * ND; f++) {
        const int d = f >> 1, s = f & 1;
        const bool bnd = s ? o.ijk[d] == nb - 1 : o.ijk[d] == 0;
        if (!bnd) {
          const int stride = d == 0 ? 1 : (d == 1 ? nb : nb * nb);
          diag += o.coef[f];
          off = fma_t(o.coef[f], tile[o.ci + (s ? stride : -stride)], off);
        } else {
          const int q0 = d == 0 ? 1 : 0, q1 = d == 2 ? 1 : 2;
          const int m = o.ijk[q0] + (ND == 3 ? nb * o.ijk[q1] : 0);
          const int e = f * nface + m;
          diag += hc[e];
          off = fma_t(hk[e], hv[e], off);
        }
      }
      T unew = 0;
      if (sizeof(T) == 8 && L.sa) {
        unew = fma_t(o.r, (T)o.sa, off * (T)o.ia);
        if (o.ia != 0) unew = relax(c.omega, unew, tile[o.ci]);
      } else {
        if (o.v > 0 && diag > 0) unew = relax(c.omega, fast_div(fma_t(o.r * dv, o.v, off), diag), tile[o.ci]);
      }
      tile[o.ci] = unew;
    };
    for (int h = threadIdx.x; h < nhalf; h += 2 * blockDim.x) {
      const int h2 = h + blockDim.x;
      Ops o1, o2;
      gather(h, o1);
      if (h2 < nhalf) gather(h2, o2);
      update(o1);
      if (h2 < nhalf) update(o2);
    }
    __syncthreads();
    if ((ncell & 3) == 0 && sizeof(T) == 4) {
      const float4 *src = reinterpret_cast<const float4 *>(tile);
      float4 *dst = reinterpret_cast<float4 *>(phi + cb);
      for (int i = threadIdx.x; i < (ncell >> 2); i += blockDim.x) dst[i] = src[i];
    } else {
      for (int i = threadIdx.x; i < ncell; i += blockDim.x) phi[cb + i] = tile[i];
    }
    __syncthreads();
  }
}

// ---- Block-hybrid Gauss-Seidel: one pass over every block of a list (all
// sublevels of a tower at once).  Each CTA loads its block's tile from src,
// takes every value outside the block from src too (frozen for the pass:
// Jacobi between blocks), runs nsweep red-black sweeps on the tile in shared
// memory and writes the tile to dst.  src is not written during the pass, so
// the result does not depend on the order in which CTAs run: the pass is one
// fixed linear map, like the sweeps it replaces, but it moves a block's data
// once for nsweep sweeps and needs one launch per pass instead of one per
// colour, level parity and sweep.  The boundary faces are evaluated as in
// smooth_cell_fast (same-level, coarse/fine and physical faces).
template <typename T, int ND, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) k_bhgs(Topo t, Coef<T> c, BlockList L, int nsweep,
                                                         const T *__restrict__ src, T *__restrict__ dst,
                                                         const T *__restrict__ rhs, const int *guard) {
  extern __shared__ __align__(16) unsigned char bhgs_smem[];
  pdl_enter();
  if (guard && *guard) return;
  const int nb = t.nb, ncell = t.ncell, nhalf = ncell >> 1;
  const int nface = ND == 3 ? nb * nb : nb;  // cells on one block face
  T *tile = reinterpret_cast<T *>(bhgs_smem);
  T *hc = tile + ncell;            // diagonal part of every boundary face of the block
  T *ho = hc + 2 * ND * nface;     // its off-diagonal part (frozen neighbour values)
  for (int p = blockIdx.x; p < L.n; p += gridDim.x) {
    const int *hxe = L.hx ? L.hx + (long)p * kHX : nullptr;
    const int b = hxe ? hxe[kHXBlock] : L.blocks[p];
    if (block_off(L, b)) continue;  // uniform over the CTA
    const uint16_t ft = hxe ? (uint16_t)(hxe[kHXInfo] & 0xffff) : L.ftypes[p];
    const long cb = (long)b * ncell;
    const long fb = (long)b * t.nfb;
    if ((ncell & 3) == 0 && sizeof(T) == 4) {
      const float4 *s4 = reinterpret_cast<const float4 *>(src + cb);
      float4 *d4 = reinterpret_cast<float4 *>(tile);
      for (int i = threadIdx.x; i < (ncell >> 2); i += blockDim.x) d4[i] = s4[i];
    } else {
      for (int i = threadIdx.x; i < ncell; i += blockDim.x) tile[i] = src[cb + i];
    }
    for (int e = threadIdx.x; e < 2 * ND * nface; e += blockDim.x) {
      const int f = e / nface, m = e - f * nface;
      const int d = f >> 1, s = f & 1;
      int ijk[3] = {0, 0, 0};
      ijk[d] = s ? nb - 1 : 0;
      const int q0 = d == 0 ? 1 : 0, q1 = d == 2 ? 1 : 2;
      ijk[q0] = m % nb;
      if (ND == 3) ijk[q1] = m / nb;
      int fx;
      if (d == 0)
        fx = ijk[0] + s + (nb + 1) * (ijk[1] + nb * ijk[2]);
      else if (d == 1)
        fx = ijk[0] + nb * (ijk[1] + s + (nb + 1) * ijk[2]);
      else
        fx = encode(ijk, nb) + s * nb * nb;
      const int ty = face_type_of(ft, f);
      const T *u = uniform_of(c, b);
      T vc = 0, vo = 0;
      if (ty == 0) {
        vc = u ? u[d] : c.tff[d][fb + fx];
        vo = vc * same_level_ghost<T, false>(t, b, f, ijk, src, hxe);
      } else if (ty == 1) {
        if (t.bc_type[b * 6 + f] != kBCNeumann) vc = (u ? u[d] : c.tff[d][fb + fx]) * (T)2.0;
      } else if (ty == 2) {
        vc = cf_coef(c, t, b, d, fx, (T)1.5);
        vo = vc * fine_crse_ghost<T, ND, false>(t, b, f, ijk, src, hxe);
      } else {
        vc = cf_coef(c, t, b, d, fx, (T)0.75);
        vo = crse_fine_sum<T, ND, false>(t, c, b, f, ijk, src, hxe);
      }
      hc[e] = vc;
      ho[e] = vo;
    }
    __syncthreads();
    const T dv = geom(c, b, 6);
    const T *u = uniform_of(c, b);  // constant coefficients: no face or vf loads
    for (int sw = 0; sw < nsweep; sw++) {
      for (int color = 0; color < 2; color++) {
        for (int h = threadIdx.x; h < nhalf; h += blockDim.x) {
          int ijk[3];
          color_cell_fast<ND>(h, t, color, ijk);
          const int ci = t.lnb >= 0 ? ijk[0] + ((ijk[1] + (ijk[2] << t.lnb)) << t.lnb) : encode(ijk, nb);
          T diag = c.alpha * dv;
          T off = 0;
#pragma unroll
          for (int f = 0; f < 2 * ND; f++) {
            const int d = f >> 1, s = f & 1;
            const bool bnd = s ? ijk[d] == nb - 1 : ijk[d] == 0;
            if (!bnd) {
              int fx;
              if (d == 0)
                fx = ijk[0] + s + (nb + 1) * (ijk[1] + nb * ijk[2]);
              else if (d == 1)
                fx = ijk[0] + nb * (ijk[1] + s + (nb + 1) * ijk[2]);
              else
                fx = ci + s * nb * nb;
              const T coef = u ? u[d] : c.tff[d][fb + fx];
              const int stride = d == 0 ? 1 : (d == 1 ? nb : nb * nb);
              diag += coef;
              off = fma_t(coef, tile[ci + (s ? stride : -stride)], off);
            } else {
              const int qa = d == 0 ? 1 : 0, qb = d == 2 ? 1 : 2;
              const int e = f * nface + ijk[qa] + (ND == 3 ? nb * ijk[qb] : 0);
              diag += hc[e];
              off += ho[e];
            }
          }
          T unew = 0;
          if (sizeof(T) == 8 && L.sa) {
            bool inner = true;
#pragma unroll
            for (int q = 0; q < ND; q++) inner = inner && ijk[q] > 0 && ijk[q] < nb - 1;
            const long fo = (long)p * ncell + ci;
            const bool ui = u && inner;
            const T iav = ui ? u[7] : (T)L.ia[fo];  // 0 in a solid cell
            unew = fma_t(rhs[cb + ci], ui ? u[6] : (T)L.sa[fo], off * iav);
            if (iav != (T)0) unew = relax(c.omega, unew, tile[ci]);
          } else {
            const T vfv = u ? (T)1 : c.vf[cb + ci];
            if (vfv > 0 && diag > 0) unew = relax(c.omega, fast_div(fma_t(rhs[cb + ci] * dv, vfv, off), diag), tile[ci]);
          }
          tile[ci] = unew;
        }
        __syncthreads();
      }
    }
    if ((ncell & 3) == 0 && sizeof(T) == 4) {
      const float4 *s4 = reinterpret_cast<const float4 *>(tile);
      float4 *d4 = reinterpret_cast<float4 *>(dst + cb);
      for (int i = threadIdx.x; i < (ncell >> 2); i += blockDim.x) d4[i] = s4[i];
    } else {
      for (int i = threadIdx.x; i < ncell; i += blockDim.x) dst[cb + i] = tile[i];
    }
    __syncthreads();
  }
}

// dst = src over the blocks of a list
template <typename T>
__global__ void __launch_bounds__(kThreads) k_copy_blocks(BlockList L, int ncell, const T *__restrict__ src,
                                                          T *__restrict__ dst, const int *guard) {
  pdl_enter();
  if (guard && *guard) return;
  const long total = (long)L.n * ncell;
  for (long it = blockIdx.x * (long)blockDim.x + threadIdx.x; it < total; it += (long)gridDim.x * blockDim.x) {
    const int p = (int)(it / ncell);
    if (block_off(L, L.blocks[p])) continue;
    const long q = (long)L.blocks[p] * ncell + (it - (long)p * ncell);
    dst[q] = src[q];
  }
}

// ---- the same sweep with the block's phi tile and face coefficients staged
// by TMA bulk copies (cp.async.bulk, completion on an mbarrier): in the
// compact layout both are contiguous per block.  The boundary contributions
// are gathered while the copies are in flight; the update then reads tile
// and coefficients from shared memory.  The wait is bounded: a CTA that
// times out raises the solver's error word (Topo::err), waits (bounded) for
// its own copies and leaves the block unchanged.

__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *mbar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *mbar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(mbar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, unsigned bytes, unsigned long long *mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(mbar))
      : "memory");
}
// bounded wait for phase `parity` of the mbarrier; true when it completed
__device__ __forceinline__ bool mbar_wait(unsigned long long *mbar, unsigned parity, long limit) {
  for (long i = 0; i < limit; i++) {
    unsigned done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(mbar)), "r"(parity)
        : "memory");
    if (done) return true;
    if (i > 64) __nanosleep(64);
  }
  return false;
}

template <typename T, int ND>
__global__ void __launch_bounds__(kThreads, 2) k_rbgs_bulk(Topo t, Coef<T> c, BlockList L, int color,
                                                          T *__restrict__ phi, const T *__restrict__ rhs,
                                                          const int *guard) {
  extern __shared__ __align__(128) unsigned char rbgs_bulk_smem[];
  pdl_enter();
  if (guard && *guard) return;
  const int nb = t.nb, ncell = t.ncell, nhalf = ncell >> 1, nfb = t.nfb;
  const int nface = ND == 3 ? nb * nb : nb;
  unsigned long long *mbar = reinterpret_cast<unsigned long long *>(rbgs_bulk_smem);
  T *tile = reinterpret_cast<T *>(rbgs_bulk_smem + 16);
  T *tf[3];
  for (int d = 0; d < 3; d++) tf[d] = tile + ncell + d * nfb;
  T *hc = tile + ncell + ND * nfb;
  T *hk = hc + 2 * ND * nface;
  T *hv = hk + 2 * ND * nface;
  const int p = blockIdx.x;
  const int *hxe = L.hx ? L.hx + (long)p * kHX : nullptr;
  const int b = hxe ? hxe[kHXBlock] : L.blocks[p];
  const uint16_t ft = hxe ? (uint16_t)(hxe[kHXInfo] & 0xffff) : L.ftypes[p];
  const long cb = (long)b * ncell, fb = (long)b * nfb;
  const unsigned tile_bytes = (unsigned)(ncell * sizeof(T)), face_bytes = (unsigned)(nfb * sizeof(T));
  if (threadIdx.x == 0) mbar_init(mbar, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(mbar, tile_bytes + ND * face_bytes);
    bulk_copy(tile, phi + cb, tile_bytes, mbar);
    for (int d = 0; d < ND; d++) bulk_copy(tf[d], c.tff[d] + fb, face_bytes, mbar);
  }
  // boundary contributions of the cells of this colour, from global memory
  for (int e = threadIdx.x; e < 2 * ND * nface; e += blockDim.x) {
    const int f = e / nface, m = e - f * nface;
    const int d = f >> 1, s = f & 1;
    int ijk[3] = {0, 0, 0};
    ijk[d] = s ? nb - 1 : 0;
    const int q0 = d == 0 ? 1 : 0, q1 = d == 2 ? 1 : 2;
    ijk[q0] = m % nb;
    if (ND == 3) ijk[q1] = m / nb;
    if (((ijk[0] + ijk[1] + ijk[2]) & 1) != color) continue;
    int fx;
    if (d == 0)
      fx = ijk[0] + s + (nb + 1) * (ijk[1] + nb * ijk[2]);
    else if (d == 1)
      fx = ijk[0] + nb * (ijk[1] + s + (nb + 1) * ijk[2]);
    else
      fx = encode(ijk, nb) + s * nb * nb;
    const int ty = face_type_of(ft, f);
    T vc = 0, vk = 0, vv = 0;
    if (ty == 0) {
      vc = vk = c.tff[d][fb + fx];
      vv = same_level_ghost<T, false>(t, b, f, ijk, phi, hxe);
    } else if (ty == 1) {
      if (t.bc_type[b * 6 + f] != kBCNeumann) vc = c.tff[d][fb + fx] * (T)2.0;
    } else if (ty == 2) {
      vc = vk = cf_coef(c, t, b, d, fx, (T)1.5);
      vv = fine_crse_ghost<T, ND, false>(t, b, f, ijk, phi, hxe);
    } else {
      vc = cf_coef(c, t, b, d, fx, (T)0.75);
      vk = (T)1;
      vv = crse_fine_sum<T, ND, false>(t, c, b, f, ijk, phi, hxe);
    }
    hc[e] = vc;
    hk[e] = vk;
    hv[e] = vv;
  }
  const long kWait = 1l << 22;  // about 0.3 s with the back-off: never reached unless the copy engine failed
  const bool ok = mbar_wait(mbar, 0, kWait);
  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0) {
      // the error word makes the solve report a CUDA error; should this
      // bounded drain time out too, copies may still land in shared memory
      // the CTA released, so nothing the device computes after the flag is
      // set is trusted (the host reports the failure after the solve)
      if (t.err) atomicExch(t.err, 1);
      mbar_wait(mbar, 0, kWait);  // let the copies into this CTA's shared memory land before it exits
    }
    return;
  }
  const T dv = geom(c, b, 6);
  for (int h = threadIdx.x; h < nhalf; h += blockDim.x) {
    int ijk[3];
    color_cell_fast<ND>(h, t, color, ijk);
    const int ci = t.lnb >= 0 ? ijk[0] + ((ijk[1] + (ijk[2] << t.lnb)) << t.lnb) : encode(ijk, nb);
    T diag = c.alpha * dv;
    T off = 0;
#pragma unroll
    for (int f = 0; f < 2 * ND; f++) {
      const int d = f >> 1, s = f & 1;
      const bool bnd = s ? ijk[d] == nb - 1 : ijk[d] == 0;
      if (!bnd) {
        int fx;
        if (d == 0)
          fx = ijk[0] + s + (nb + 1) * (ijk[1] + nb * ijk[2]);
        else if (d == 1)
          fx = ijk[0] + nb * (ijk[1] + s + (nb + 1) * ijk[2]);
        else
          fx = ci + s * nb * nb;
        const T coef = tf[d][fx];
        const int stride = d == 0 ? 1 : (d == 1 ? nb : nb * nb);
        diag += coef;
        off = fma_t(coef, tile[ci + (s ? stride : -stride)], off);
      } else {
        const int q0 = d == 0 ? 1 : 0, q1 = d == 2 ? 1 : 2;
        const int m = ijk[q0] + (ND == 3 ? nb * ijk[q1] : 0);
        const int e = f * nface + m;
        diag += hc[e];
        off = fma_t(hk[e], hv[e], off);
      }
    }
    T unew = 0;
    if (sizeof(T) == 8 && L.sa) {
      const long fo = (long)p * ncell + ci;
      unew = fma_t(rhs[cb + ci], (T)L.sa[fo], off * (T)L.ia[fo]);
      if (L.ia[fo] != 0.0) unew = relax(c.omega, unew, tile[ci]);
    } else {
      const T vfv = c.vf[cb + ci];
      if (vfv > 0 && diag > 0) unew = relax(c.omega, fast_div(fma_t(rhs[cb + ci] * dv, vfv, off), diag), tile[ci]);
    }
    tile[ci] = unew;
  }
  __syncthreads();
  if ((ncell & 3) == 0 && sizeof(T) == 4) {
    const float4 *src = reinterpret_cast<const float4 *>(tile);
    float4 *dst = reinterpret_cast<float4 *>(phi + cb);
    for (int i = threadIdx.x; i < (ncell >> 2); i += blockDim.x) dst[i] = src[i];
  } else {
    for (int i = threadIdx.x; i < ncell; i += blockDim.x) phi[cb + i] = tile[i];
  }
}

// ---- persistent, double-buffered: one CTA per SM walks blocks p = blockIdx.x,
// blockIdx.x + gridDim.x, ...; while it gathers the boundary contributions of
// block i and updates it from shared memory, the copy engine streams block
// i+1's tile, face coefficients, rhs and vf into the other buffer.
constexpr int kStreamThreads = 512;

template <typename T, int ND>
__global__ void __launch_bounds__(kStreamThreads, 1) k_rbgs_stream(Topo t, Coef<T> c, BlockList L, int color,
                                                                   T *__restrict__ phi, const T *__restrict__ rhs,
                                                                   const int *guard) {
  extern __shared__ __align__(128) unsigned char rbgs_stream_smem[];
  pdl_enter();
  if (guard && *guard) return;
  const int nb = t.nb, ncell = t.ncell, nhalf = ncell >> 1, nfb = t.nfb;
  const int nface = ND == 3 ? nb * nb : nb;
  const size_t buf_elems = (size_t)3 * ncell + (size_t)ND * nfb;  // tile, rhs, vf, faces
  unsigned long long *mbar = reinterpret_cast<unsigned long long *>(rbgs_stream_smem);  // [2]
  T *buf0 = reinterpret_cast<T *>(rbgs_stream_smem + 16);
  T *hc = buf0 + 2 * buf_elems;
  T *hk = hc + 2 * ND * nface;
  T *hv = hk + 2 * ND * nface;
  const unsigned tile_bytes = (unsigned)(ncell * sizeof(T)), face_bytes = (unsigned)(nfb * sizeof(T));
  const unsigned tx = 3 * tile_bytes + ND * face_bytes;
  auto issue = [&](int pp, int j) {  // thread 0: copies of list entry pp into buffer j
    const int bb = L.blocks[pp];
    T *bt = buf0 + j * buf_elems;
    // buffer j was last read and written through the generic proxy (the
    // sweep and the copy-out, ordered before this point by __syncthreads);
    // the bulk copies write it through the async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&mbar[j], tx);
    bulk_copy(bt, phi + (long)bb * ncell, tile_bytes, &mbar[j]);
    bulk_copy(bt + ncell, rhs + (long)bb * ncell, tile_bytes, &mbar[j]);
    bulk_copy(bt + 2 * ncell, c.vf + (long)bb * ncell, tile_bytes, &mbar[j]);
    for (int d = 0; d < ND; d++) bulk_copy(bt + 3 * ncell + d * nfb, c.tff[d] + (long)bb * nfb, face_bytes, &mbar[j]);
  };
  if (threadIdx.x == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
  }
  __syncthreads();
  if (blockIdx.x >= L.n) return;
  if (threadIdx.x == 0) issue(blockIdx.x, 0);
  const long kWait = 1l << 22;
  unsigned phase[2] = {0u, 0u};
  int k = 0;
  for (int p = blockIdx.x; p < L.n; p += gridDim.x, k++) {
    const int j = k & 1;
    if (threadIdx.x == 0 && p + (int)gridDim.x < L.n) issue(p + gridDim.x, j ^ 1);
    const int *hxe = L.hx ? L.hx + (long)p * kHX : nullptr;
    const int b = hxe ? hxe[kHXBlock] : L.blocks[p];
    const uint16_t ft = hxe ? (uint16_t)(hxe[kHXInfo] & 0xffff) : L.ftypes[p];
    const long cb = (long)b * ncell, fb = (long)b * nfb;
    for (int e = threadIdx.x; e < 2 * ND * nface; e += blockDim.x) {
      const int f = e / nface, m = e - f * nface;
      const int d = f >> 1, s = f & 1;
      int ijk[3] = {0, 0, 0};
      ijk[d] = s ? nb - 1 : 0;
      const int q0 = d == 0 ? 1 : 0, q1 = d == 2 ? 1 : 2;
      ijk[q0] = m % nb;
      if (ND == 3) ijk[q1] = m / nb;
      if (((ijk[0] + ijk[1] + ijk[2]) & 1) != color) continue;
      int fx;
      if (d == 0)
        fx = ijk[0] + s + (nb + 1) * (ijk[1] + nb * ijk[2]);
      else if (d == 1)
        fx = ijk[0] + nb * (ijk[1] + s + (nb + 1) * ijk[2]);
      else
        fx = encode(ijk, nb) + s * nb * nb;
      const int ty = face_type_of(ft, f);
      T vc = 0, vk = 0, vv = 0;
      if (ty == 0) {
        vc = vk = c.tff[d][fb + fx];
        vv = same_level_ghost<T, false>(t, b, f, ijk, phi, hxe);
      } else if (ty == 1) {
        if (t.bc_type[b * 6 + f] != kBCNeumann) vc = c.tff[d][fb + fx] * (T)2.0;
      } else if (ty == 2) {
        vc = vk = cf_coef(c, t, b, d, fx, (T)1.5);
        vv = fine_crse_ghost<T, ND, false>(t, b, f, ijk, phi, hxe);
      } else {
        vc = cf_coef(c, t, b, d, fx, (T)0.75);
        vk = (T)1;
        vv = crse_fine_sum<T, ND, false>(t, c, b, f, ijk, phi, hxe);
      }
      hc[e] = vc;
      hk[e] = vk;
      hv[e] = vv;
    }
    const bool ok = mbar_wait(&mbar[j], phase[j], kWait);
    phase[j] ^= 1u;
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        // the error word makes the solve report a CUDA error; should the
        // bounded drain below also time out, copies may still be landing in
        // shared memory this CTA released, so nothing the device computes
        // after the flag is set is trusted (the host reports the failure)
        if (t.err) atomicExch(t.err, 1);
        // let this CTA's copies land before it exits
        mbar_wait(&mbar[j], phase[j] ^ 1u, kWait);
        if (p + (int)gridDim.x < L.n) mbar_wait(&mbar[j ^ 1], phase[j ^ 1], kWait);
      }
      return;
    }
    T *tile = buf0 + j * buf_elems;
    const T *rh = tile + ncell, *vfs = tile + 2 * ncell, *tf0 = tile + 3 * ncell;
    const T dv = geom(c, b, 6);
    for (int h = threadIdx.x; h < nhalf; h += blockDim.x) {
      int ijk[3];
      color_cell_fast<ND>(h, t, color, ijk);
      const int ci = t.lnb >= 0 ? ijk[0] + ((ijk[1] + (ijk[2] << t.lnb)) << t.lnb) : encode(ijk, nb);
      T diag = c.alpha * dv;
      T off = 0;
#pragma unroll
      for (int f = 0; f < 2 * ND; f++) {
        const int d = f >> 1, s = f & 1;
        const bool bnd = s ? ijk[d] == nb - 1 : ijk[d] == 0;
        if (!bnd) {
          int fx;
          if (d == 0)
            fx = ijk[0] + s + (nb + 1) * (ijk[1] + nb * ijk[2]);
          else if (d == 1)
            fx = ijk[0] + nb * (ijk[1] + s + (nb + 1) * ijk[2]);
          else
            fx = ci + s * nb * nb;
          const T coef = tf0[d * nfb + fx];
          const int stride = d == 0 ? 1 : (d == 1 ? nb : nb * nb);
          diag += coef;
          off = fma_t(coef, tile[ci + (s ? stride : -stride)], off);
        } else {
          const int q0 = d == 0 ? 1 : 0, q1 = d == 2 ? 1 : 2;
          const int m = ijk[q0] + (ND == 3 ? nb * ijk[q1] : 0);
          const int e = f * nface + m;
          diag += hc[e];
          off = fma_t(hk[e], hv[e], off);
        }
      }
      T unew = 0;
      if (sizeof(T) == 8 && L.sa) {
        const long fo = (long)p * ncell + ci;
        unew = fma_t(rh[ci], (T)L.sa[fo], off * (T)L.ia[fo]);
        if (L.ia[fo] != 0.0) unew = relax(c.omega, unew, tile[ci]);
      } else {
        const T vfv = vfs[ci];
        if (vfv > 0 && diag > 0) unew = relax(c.omega, fast_div(fma_t(rh[ci] * dv, vfv, off), diag), tile[ci]);
      }
      tile[ci] = unew;
    }
    __syncthreads();
    if ((ncell & 3) == 0 && sizeof(T) == 4) {
      const float4 *src = reinterpret_cast<const float4 *>(tile);
      float4 *dst = reinterpret_cast<float4 *>(phi + cb);
      for (int i = threadIdx.x; i < (ncell >> 2); i += blockDim.x) dst[i] = src[i];
    } else {
      for (int i = threadIdx.x; i < ncell; i += blockDim.x) phi[cb + i] = tile[i];
    }
    __syncthreads();  // buffer j and the boundary arrays are free again
  }
}

template <typename T, int ND>
static size_t rbgs_stream_smem(const Topo &t) {
  const int nface = ND == 3 ? t.nb * t.nb : t.nb;
  return 16 + sizeof(T) * (2 * ((size_t)3 * t.ncell + (size_t)ND * t.nfb) + 3 * 2 * ND * (size_t)nface);
}

template <typename T, int ND>
static void rbgs_stream_go(const Topo &t, const Coef<T> &c, const BlockList &L, int color, T *phi, const T *rhs,
                           const int *guard, cudaStream_t s, bool pdl) {
  const size_t smem = rbgs_stream_smem<T, ND>(t);
  int dev = 0, nsm = 152;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    nsm = 152;
  }
  ensure_max_smem((const void *)k_rbgs_stream<T, ND>, 227 * 1024);
  launch_k(pdl, k_rbgs_stream<T, ND>, std::min(L.n, nsm), kStreamThreads, smem, s, t, c, L, color, phi, rhs,
           guard);
}

template <typename T, int ND>
static size_t rbgs_bulk_smem(const Topo &t) {
  const int nface = ND == 3 ? t.nb * t.nb : t.nb;
  return 16 + sizeof(T) * ((size_t)t.ncell + (size_t)ND * t.nfb + 3 * 2 * ND * (size_t)nface);
}

template <typename T, int ND>
static void rbgs_bulk_go(const Topo &t, const Coef<T> &c, const BlockList &L, int color, T *phi, const T *rhs,
                         const int *guard, cudaStream_t s, bool pdl) {
  const size_t smem = rbgs_bulk_smem<T, ND>(t);
  ensure_max_smem((const void *)k_rbgs_bulk<T, ND>, 200 * 1024);
  const int threads = std::min(kThreads, ((t.ncell >> 1) + 31) / 32 * 32);
  launch_k(pdl, k_rbgs_bulk<T, ND>, L.n, threads, smem, s, t, c, L, color, phi, rhs, guard);
}

int rbgs_bulk_error(int *err, cudaStream_t s, bool clear) {
  if (!err) return 0;
  int v = 0;
  if (cudaMemcpyAsync(&v, err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return -1;
  if (clear && v) {
    if (cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) return -1;
  }
  return v;
}

// ---- prolongation of a level fused with the first (red) sweep that follows
// it: one CTA per block of the level; the block's tile is filled with its
// prolonged values (masked injection from the parent, as k_prolong), the
// red cells' same-level neighbours outside the block are prolonged on the
// fly from their own parents, coarse neighbours (FINE_CRSE) are read as they
// are; the red cells are then updated with the tiled sweep's arithmetic and
// the whole tile is written.  Same values as k_prolong + k_rbgs_tile.

template <typename T, int ND>
__global__ void __launch_bounds__(kThreads, 4) k_prolong_red(Topo t, Coef<T> c, BlockList L, T *__restrict__ phi,
                                                            const T *__restrict__ rhs, const int *guard,
                                                            BlockList X) {
  extern __shared__ __align__(16) unsigned char pr_smem[];
  pdl_enter();
  if (guard && *guard) return;
  const int nb = t.nb, ncell = t.ncell, nhalf = ncell >> 1;
  const int nface = ND == 3 ? nb * nb : nb;
  T *tile = reinterpret_cast<T *>(pr_smem);
  T *hc = tile + ncell;
  T *hk = hc + 2 * ND * nface;
  T *hv = hk + 2 * ND * nface;
  for (int p = blockIdx.x; p < L.n + X.n; p += gridDim.x) {
    if (p >= L.n) {
      // the red sweep of a block of X: blocks two or more levels coarser,
      // which neither read nor are read by the level being prolonged
      const int px = p - L.n;
      const long fo = (long)px * ncell;
      const int *e = X.hx + (long)px * kHX;
      if (block_off(X, e[kHXBlock])) continue;
      for (int h = threadIdx.x; h < nhalf; h += blockDim.x) {
        int ijk[3];
        color_cell_fast<ND>(h, t, 0, ijk);
        smooth_cell_fast<T, ND>(t, c, e[kHXBlock], (uint16_t)(e[kHXInfo] & 0xffff), ijk, phi, rhs,
                                X.sa ? X.sa + fo : nullptr, X.ia ? X.ia + fo : nullptr, e);
      }
      continue;
    }
    const int *hxe = L.hx ? L.hx + (long)p * kHX : nullptr;
    const int b = hxe ? hxe[kHXBlock] : L.blocks[p];
    if (block_off(L, b)) continue;  // uniform over the CTA
    const uint16_t ft = hxe ? (uint16_t)(hxe[kHXInfo] & 0xffff) : L.ftypes[p];
    const long cb = (long)b * ncell;
    const long fb = (long)b * t.nfb;
    const T *u = uniform_of(c, b);  // constant coefficients: no face or vf loads
    for (int i = threadIdx.x; i < ncell; i += blockDim.x) {
      int ijk[3];
      decode<ND>(i, nb, ijk);
      tile[i] = prolonged_value<T, ND>(t, c, b, ijk, phi, hxe ? hxe[kHXPar + 6] : -1, u != nullptr);
    }
    for (int e = threadIdx.x; e < 2 * ND * nface; e += blockDim.x) {
      const int f = e / nface, m = e - f * nface;
      const int d = f >> 1, s = f & 1;
      int ijk[3] = {0, 0, 0};
      ijk[d] = s ? nb - 1 : 0;
      const int q0 = d == 0 ? 1 : 0, q1 = d == 2 ? 1 : 2;
      ijk[q0] = m % nb;
      if (ND == 3) ijk[q1] = m / nb;
      if ((ijk[0] + ijk[1] + ijk[2]) & 1) continue;  // red cells only
      int fx;
      if (d == 0)
        fx = ijk[0] + s + (nb + 1) * (ijk[1] + nb * ijk[2]);
      else if (d == 1)
        fx = ijk[0] + nb * (ijk[1] + s + (nb + 1) * ijk[2]);
      else
        fx = encode(ijk, nb) + s * nb * nb;
      const int ty = face_type_of(ft, f);
      T vc = 0, vk = 0, vv = 0;
      if (ty == 0) {
        const int n = hxe ? hxe[f] : t.neighbor[b * 6 + f];
        int ni[3] = {ijk[0], ijk[1], ijk[2]};
        ni[d] = s ? 0 : nb - 1;
        vc = vk = u ? u[d] : c.tff[d][fb + fx];
        vv = prolonged_value<T, ND>(t, c, n, ni, phi, hxe ? hxe[kHXPar + f] : -1);
      } else if (ty == 1) {
        if (t.bc_type[b * 6 + f] != kBCNeumann) vc = (u ? u[d] : c.tff[d][fb + fx]) * (T)2.0;
      } else if (ty == 2) {
        vc = vk = cf_coef(c, t, b, d, fx, (T)1.5);
        vv = fine_crse_ghost<T, ND, false>(t, b, f, ijk, phi, hxe);
      } else {  // not at the finest level of a tower
        vc = cf_coef(c, t, b, d, fx, (T)0.75);
        vk = (T)1;
        vv = crse_fine_sum<T, ND, false>(t, c, b, f, ijk, phi, hxe);
      }
      hc[e] = vc;
      hk[e] = vk;
      hv[e] = vv;
    }
    __syncthreads();
    const T dv = geom(c, b, 6);
    for (int h = threadIdx.x; h < nhalf; h += blockDim.x) {
      int ijk[3];
      color_cell_fast<ND>(h, t, 0, ijk);
      const int ci = t.lnb >= 0 ? ijk[0] + ((ijk[1] + (ijk[2] << t.lnb)) << t.lnb) : encode(ijk, nb);
      T diag = c.alpha * dv;
      T off = 0;
#pragma unroll
      for (int f = 0; f < 2 * ND; f++) {
        const int d = f >> 1, s = f & 1;
        const bool bnd = s ? ijk[d] == nb - 1 : ijk[d] == 0;
        if (!bnd) {
          int fx;
          if (d == 0)
            fx = ijk[0] + s + (nb + 1) * (ijk[1] + nb * ijk[2]);
          else if (d == 1)
            fx = ijk[0] + nb * (ijk[1] + s + (nb + 1) * ijk[2]);
          else
            fx = ci + s * nb * nb;
          const T coef = u ? u[d] : c.tff[d][fb + fx];
          const int stride = d == 0 ? 1 : (d == 1 ? nb : nb * nb);
          diag += coef;
          off = fma_t(coef, tile[ci + (s ? stride : -stride)], off);
        } else {
          const int q0 = d == 0 ? 1 : 0, q1 = d == 2 ? 1 : 2;
          const int m = ijk[q0] + (ND == 3 ? nb * ijk[q1] : 0);
          const int e = f * nface + m;
          diag += hc[e];
          off = fma_t(hk[e], hv[e], off);
        }
      }
      T unew = 0;
      if (sizeof(T) == 8 && L.sa) {
        bool inner = true;
#pragma unroll
        for (int q = 0; q < ND; q++) inner = inner && ijk[q] > 0 && ijk[q] < nb - 1;
        const long fo = (long)p * ncell + ci;
        const bool ui = u && inner;
        const T iav = ui ? u[7] : (T)L.ia[fo];  // 0 in a solid cell
        unew = fma_t(rhs[cb + ci], ui ? u[6] : (T)L.sa[fo], off * iav);
        if (iav != (T)0) unew = relax(c.omega, unew, tile[ci]);
      } else {
        const T vfv = u ? (T)1 : c.vf[cb + ci];
        if (vfv > 0 && diag > 0) unew = relax(c.omega, fast_div(fma_t(rhs[cb + ci] * dv, vfv, off), diag), tile[ci]);
      }
      tile[ci] = unew;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < ncell; i += blockDim.x) phi[cb + i] = tile[i];
    __syncthreads();
  }
}

template <typename T>
void launch_prolong_red(const Topo &t, const Coef<T> &c, const BlockList &L, T *phi, const T *rhs,
                        const int *guard, cudaStream_t s, bool pdl, const BlockList &X, int form) {
  if (L.n == 0) return;
  if (X.n > 0 && !X.hx) return;  // the extra sweep reads its blocks through halo descriptors
  if constexpr (sizeof(T) == 4) {
    if (form == 1 && t.ndim == 2 && t.nb == 16) {
      const int g = std::min((L.n + X.n + 7) / 8, 152 * 64);
      launch_k(pdl, k_prolong_red_warp16<5>, g, kThreads, 0, s, t, c, L, phi, rhs, guard, X);
      return;
    }
  }
  const int nface = t.ndim == 3 ? t.nb * t.nb : t.nb;
  const size_t smem = sizeof(T) * ((size_t)t.ncell + 3 * 2 * t.ndim * (size_t)nface);
  ensure_max_smem(t.ndim == 2 ? (const void *)k_prolong_red<T, 2> : (const void *)k_prolong_red<T, 3>, 200 * 1024);
  const int threads = std::min(kThreads, ((t.ncell >> 1) + 31) / 32 * 32);
  const int grid = std::min(L.n + X.n, 152 * 64);
  if (t.ndim == 2)
    launch_k(pdl, k_prolong_red<T, 2>, grid, threads, smem, s, t, c, L, phi, rhs, guard, X);
  else
    launch_k(pdl, k_prolong_red<T, 3>, grid, threads, smem, s, t, c, L, phi, rhs, guard, X);
}

template <typename T, int ND>
static size_t rbgs_tile_smem(const Topo &t) {
  const int nface = ND == 3 ? t.nb * t.nb : t.nb;
  return sizeof(T) * ((size_t)t.ncell + 3 * 2 * ND * (size_t)nface);
}

template <typename T, int ND, int MINB>
static void rbgs_tile_go(const Topo &t, const Coef<T> &c, const BlockList &L, int color, T *phi, const T *rhs,
                         const int *guard, cudaStream_t s, bool pdl) {
  const size_t smem = rbgs_tile_smem<T, ND>(t);
  ensure_max_smem((const void *)k_rbgs_tile<T, ND, MINB>, 200 * 1024);
  const int threads = std::min(kThreads, ((t.ncell >> 1) + 31) / 32 * 32);
  const int grid = std::min(L.n, 152 * 64);
  launch_k(pdl, k_rbgs_tile<T, ND, MINB>, grid, threads, smem, s, t, c, L, color, phi, rhs, guard);
}

// variant v: launch bounds (256 threads, kRbgsMinBlocks[v] CTAs per SM), i.e.
// a register cap of 65536 / (256 * min CTAs); same arithmetic in every variant
template <typename T, int ND, int MINB>
static void rbgs_go(const Topo &t, const Coef<T> &c, const BlockList &L, int color, T *phi, const T *rhs,
                    const int *guard, cudaStream_t s, bool pdl, dim3 grid, int threads) {
  launch_k(pdl, k_rbgs<T, ND, MINB>, grid, threads, 0, s, t, c, L, color, phi, rhs, guard);
}

// variant 10: CPT = 2 cells per thread (k_rbgs_ilp), cap 64; variants 11, 12:
// one warp per 16x16 block in 2D FP32 (k_rbgs_warp16, caps 64 and 48);
// variant 13: the same with every load issued before the first branch
// (k_rbgs_warp16_flat, cap 64: at 48 registers it spills and loses,
// 20.8 vs 16.9 us on the batch workload's first 64 problems); elsewhere
// variant 3
template <typename T, int ND, int MINB, int CPT>
static void rbgs_ilp_go(const Topo &t, const Coef<T> &c, const BlockList &L, int color, T *phi, const T *rhs,
                        const int *guard, cudaStream_t s, bool pdl, dim3 grid, int threads) {
  grid.y = std::min((L.n + CPT - 1) / CPT, 65535);
  launch_k(pdl, k_rbgs_ilp<T, ND, MINB, CPT>, grid, threads, 0, s, t, c, L, color, phi, rhs, guard);
}

template <typename T, int ND>
static void rbgs_nd(int variant, const Topo &t, const Coef<T> &c, const BlockList &L, int color, T *phi,
                    const T *rhs, const int *guard, cudaStream_t s, bool pdl, dim3 grid, int threads) {
  switch (variant) {
    case 10: rbgs_ilp_go<T, ND, 4, 2>(t, c, L, color, phi, rhs, guard, s, pdl, grid, threads); return;
    case 11:
    case 12:
    case 13:
      if constexpr (ND == 2 && sizeof(T) == 4) {
        if (t.nb == 16) {
          const int g = std::min((L.n + 7) / 8, 152 * 64);
          if (variant == 11)
            launch_k(pdl, k_rbgs_warp16<4>, g, kThreads, 0, s, t, c, L, color, phi, rhs, guard);
          else if (variant == 12 || !L.hx)
            launch_k(pdl, k_rbgs_warp16<5>, g, kThreads, 0, s, t, c, L, color, phi, rhs, guard);
          else
            launch_k(pdl, k_rbgs_warp16_flat<4>, g, kThreads, 0, s, t, c, L, color, phi, rhs, guard);
          return;
        }
      }
      rbgs_go<T, ND, 6>(t, c, L, color, phi, rhs, guard, s, pdl, grid, threads);
      return;
    default: break;
  }
  switch (variant) {
    case 0: rbgs_go<T, ND, 2>(t, c, L, color, phi, rhs, guard, s, pdl, grid, threads); break;
    case 1: rbgs_go<T, ND, 3>(t, c, L, color, phi, rhs, guard, s, pdl, grid, threads); break;
    case 2: rbgs_go<T, ND, 4>(t, c, L, color, phi, rhs, guard, s, pdl, grid, threads); break;
    case 3: rbgs_go<T, ND, 6>(t, c, L, color, phi, rhs, guard, s, pdl, grid, threads); break;
    case 4: rbgs_go<T, ND, 8>(t, c, L, color, phi, rhs, guard, s, pdl, grid, threads); break;
    case 5: rbgs_tile_go<T, ND, 2>(t, c, L, color, phi, rhs, guard, s, pdl); break;
    case 6: rbgs_tile_go<T, ND, 4>(t, c, L, color, phi, rhs, guard, s, pdl); break;
    case 7: rbgs_tile_go<T, ND, 6>(t, c, L, color, phi, rhs, guard, s, pdl); break;
    case 8: rbgs_bulk_go<T, ND>(t, c, L, color, phi, rhs, guard, s, pdl); break;
    default: rbgs_stream_go<T, ND>(t, c, L, color, phi, rhs, guard, s, pdl); break;
  }
}

template <typename T>
void launch_rbgs(const Topo &t, const Coef<T> &c, const BlockList &L, int color, T *phi, const T *rhs,
                 const int *guard, cudaStream_t s, bool pdl, int variant) {
  const int nhalf = t.ncell / 2;
  if (L.n == 0 || nhalf == 0) return;
  // the tiled variants need the tile and halo in shared memory (<= 200 KiB);
  // the bulk-copy variant also needs 16-byte multiples for the tile and the
  // face rows of a block (and L.n CTAs in one grid dimension)
  const size_t tile = t.ndim == 2 ? rbgs_tile_smem<T, 2>(t) : rbgs_tile_smem<T, 3>(t);
  if (variant >= 5 && variant <= 9 && tile > 200 * 1024) variant = 3;
  const bool aligned = (t.ncell * sizeof(T)) % 16 == 0 && (t.nfb * sizeof(T)) % 16 == 0;
  if (L.stc && (variant == 8 || variant == 9)) variant = 7;  // the bulk-copy variants know no per-problem states
  if (variant == 8) {
    const size_t bulk = t.ndim == 2 ? rbgs_bulk_smem<T, 2>(t) : rbgs_bulk_smem<T, 3>(t);
    if (bulk > 200 * 1024 || !aligned) variant = 7;
  }
  if (variant == 9) {
    const size_t st = t.ndim == 2 ? rbgs_stream_smem<T, 2>(t) : rbgs_stream_smem<T, 3>(t);
    if (st > 227 * 1024 || !aligned) variant = 7;
  }
  const int threads = std::min(kThreads, (nhalf + 31) / 32 * 32);
  const dim3 grid((nhalf + threads - 1) / threads, std::min(L.n, 65535));
  if (t.ndim == 2)
    rbgs_nd<T, 2>(variant, t, c, L, color, phi, rhs, guard, s, pdl, grid, threads);
  else
    rbgs_nd<T, 3>(variant, t, c, L, color, phi, rhs, guard, s, pdl, grid, threads);
}

template <typename T>
void launch_bhgs(const Topo &t, const Coef<T> &c, const BlockList &L, int nsweep, const T *src, T *dst,
                 const T *rhs, const int *guard, cudaStream_t s, bool pdl) {
  const int nhalf = t.ncell / 2;
  if (L.n == 0 || nhalf == 0) return;
  const int nface = t.ndim == 3 ? t.nb * t.nb : t.nb;
  const size_t smem = sizeof(T) * ((size_t)t.ncell + 2 * 2 * t.ndim * (size_t)nface);
  const int threads = std::min(kThreads, (nhalf + 31) / 32 * 32);
  const int grid = std::min(L.n, 152 * 64);
  if (t.ndim == 2) {
    ensure_max_smem((const void *)k_bhgs<T, 2, 2>, 200 * 1024);
    launch_k(pdl, k_bhgs<T, 2, 2>, grid, threads, smem, s, t, c, L, nsweep, src, dst, rhs, guard);
  } else {
    ensure_max_smem((const void *)k_bhgs<T, 3, 2>, 200 * 1024);
    launch_k(pdl, k_bhgs<T, 3, 2>, grid, threads, smem, s, t, c, L, nsweep, src, dst, rhs, guard);
  }
}

template <typename T>
void launch_copy_blocks(const BlockList &L, int ncell, const T *src, T *dst, const int *guard, cudaStream_t s,
                        bool pdl) {
  const long work = (long)L.n * ncell;
  if (work == 0) return;
  launch_k(pdl, k_copy_blocks<T>, grid_for(work), kThreads, 0, s, L, ncell, src, dst, guard);
}

template <typename T>
void launch_smooth(const Topo &t, const Coef<T> &c, const BlockList &L, int color, T *phi, const T *rhs,
                   const int *guard, cudaStream_t s, bool pdl) {
  const long work = (long)L.n * (t.ncell / 2);
  if (work == 0) return;
  if (t.ndim == 2)
    launch_k(pdl, k_smooth<T, 2>, grid_for(work), kThreads, 0, s, t, c, L, color, phi, rhs, guard);
  else
    launch_k(pdl, k_smooth<T, 3>, grid_for(work), kThreads, 0, s, t, c, L, color, phi, rhs, guard);
}

template <typename T>
void launch_restrict(const Topo &t, const Coef<T> &c, const BlockList &L, T *phi, const int *guard,
                     cudaStream_t s, bool pdl) {
  const long work = (long)L.n * t.ncell;
  if (work == 0) return;
  if (t.ndim == 2)
    launch_k(pdl, k_restrict<T, 2>, grid_for(work), kThreads, 0, s, t, c, L, phi, guard);
  else
    launch_k(pdl, k_restrict<T, 3>, grid_for(work), kThreads, 0, s, t, c, L, phi, guard);
}

template <typename T>
void launch_prolong(const Topo &t, const Coef<T> &c, const BlockList &L, T *phi, const int *guard,
                    cudaStream_t s, bool pdl) {
  const long work = (long)L.n * t.ncell;
  if (work == 0) return;
  if (t.ndim == 2)
    launch_k(pdl, k_prolong<T, 2>, grid_for(work), kThreads, 0, s, t, c, L, phi, guard);
  else
    launch_k(pdl, k_prolong<T, 3>, grid_for(work), kThreads, 0, s, t, c, L, phi, guard);
}

void launch_flux(const Topo &t, const Coef<double> &c, const BlockList &L, int dir, const double *phi, double *flux,
                 cudaStream_t s) {
  const long work = (long)L.n * t.nfb;
  if (work == 0) return;
  if (t.ndim == 2)
    k_flux<2><<<grid_for(work), kThreads, 0, s>>>(t, c, L, dir, phi, flux);
  else
    k_flux<3><<<grid_for(work), kThreads, 0, s>>>(t, c, L, dir, phi, flux);
}

void launch_fix_bc(const Topo &t, const Coef<double> &c, const BlockList &L, const double *phig, int ng, double *rhs,
                   cudaStream_t s) {
  const long work = (long)L.n * t.ncell;
  if (work == 0) return;
  if (t.ndim == 2)
    k_fix_bc<2><<<grid_for(work), kThreads, 0, s>>>(t, c, L, phig, ng, rhs);
  else
    k_fix_bc<3><<<grid_for(work), kThreads, 0, s>>>(t, c, L, phig, ng, rhs);
}

#define SAYAKA_INST(T)                                                                                          \
  template void launch_face_coef<T>(const Topo &, const double *, const T *[3], const T *[3], double, T *[3],  \
                                    cudaStream_t);                                                              \
  template void launch_apply<T>(const Topo &, const Coef<T> &, const BlockList &, const T *, T *, const T *,   \
                                const int *, cudaStream_t, bool);                                               \
  template void launch_smooth<T>(const Topo &, const Coef<T> &, const BlockList &, int, T *, const T *,        \
                                 const int *, cudaStream_t, bool);                                              \
  template void launch_rbgs<T>(const Topo &, const Coef<T> &, const BlockList &, int, T *, const T *,          \
                               const int *, cudaStream_t, bool, int);                                           \
  template void launch_restrict<T>(const Topo &, const Coef<T> &, const BlockList &, T *, const int *,         \
                                   cudaStream_t, bool);                                                         \
  template void launch_prolong<T>(const Topo &, const Coef<T> &, const BlockList &, T *, const int *,          \
                                  cudaStream_t, bool);                                                          \
  template void launch_prolong_red<T>(const Topo &, const Coef<T> &, const BlockList &, T *, const T *,        \
                                      const int *, cudaStream_t, bool, const BlockList &, int);                 \
  template void launch_bhgs<T>(const Topo &, const Coef<T> &, const BlockList &, int, const T *, T *,          \
                               const T *, const int *, cudaStream_t, bool);                                     \
  template void launch_copy_blocks<T>(const BlockList &, int, const T *, T *, const int *, cudaStream_t, bool);
SAYAKA_INST(double)
SAYAKA_INST(float)
#undef SAYAKA_INST

}  // namespace sayaka_gb300
