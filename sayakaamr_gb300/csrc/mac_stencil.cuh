// Device-side stencil helpers shared by every kernel that evaluates the MAC
// operator, the red-black smoother or the inter-level transfers: index
// arithmetic of the compact block layout and the gathers that replace the
// reference's ghost-cell fills and coarse/fine flux registers (the mapping to
// the reference is described in mac_kernels.cu).
//
// Template flag CG: loads of fields that other CTAs write inside the same
// cooperative kernel go through L2 (ld.global.cg) instead of L1.
#pragma once

#include <cstdint>

#include <cuda_fp16.h>

#include "mac_device.h"
#include "mac_fp.cuh"

namespace sayaka_gb300 {
namespace stencil {

template <bool CG, typename T>
__device__ __forceinline__ T ld(const T *p) {
  if (CG) return __ldcg(p);
  return *p;
}

__device__ __forceinline__ int face_type_of(uint16_t ft, int f) { return (ft >> (2 * f)) & 3; }

template <int ND>
__device__ __forceinline__ void decode(int c, int nb, int ijk[3]) {
  ijk[0] = c % nb;
  ijk[1] = ND >= 2 ? (c / nb) % nb : 0;
  ijk[2] = ND == 3 ? c / (nb * nb) : 0;
}

__device__ __forceinline__ int encode(const int ijk[3], int nb) { return ijk[0] + nb * (ijk[1] + nb * ijk[2]); }

// decode with shifts when nb is a power of two
template <int ND>
__device__ __forceinline__ void decode_fast(int c, const Topo &t, int ijk[3]) {
  if (t.lnb >= 0) {
    const int m = t.nb - 1;
    ijk[0] = c & m;
    ijk[1] = ND >= 2 ? (c >> t.lnb) & m : 0;
    ijk[2] = ND == 3 ? c >> (2 * t.lnb) : 0;
  } else {
    decode<ND>(c, t.nb, ijk);
  }
}

// flat (list entry, cell) index -> list entry p and cell ci (32-bit)
template <int ND>
__device__ __forceinline__ void split_cell(int it, const Topo &t, int &p, int &ci) {
  if (t.lnb >= 0) {
    p = it >> (ND * t.lnb);
    ci = it & (t.ncell - 1);
  } else {
    p = it / t.ncell;
    ci = it - p * t.ncell;
  }
}

// face index of the face on side s of cell ijk in direction d (face-centred
// valid box of the reference, first dimension fastest)
__device__ __forceinline__ int face_index(int d, const int ijk[3], int s, int nb) {
  int f[3] = {ijk[0], ijk[1], ijk[2]};
  f[d] += s;
  const int e0 = nb + (d == 0), e1 = nb + (d == 1);
  return f[0] + e0 * (f[1] + e1 * f[2]);
}

template <typename T>
__device__ __forceinline__ T geom(const Coef<T> &c, int b, int q) { return c.geom[b * 8 + q]; }

// the record of block b when it is a constant-coefficient block (Coef::ut),
// else null
// (the flag is 0 or 1: tested as bits, so that no FP64 compare is issued)
template <typename T>
__device__ __forceinline__ const T *uniform_of(const Coef<T> &c, int b) {
  if (!c.ut) return nullptr;
  const T *u = c.ut + (long)b * kUni;
  if constexpr (sizeof(T) == 8)
    return __double_as_longlong(u[3]) != 0 ? u : nullptr;
  else
    return __float_as_uint(u[3]) != 0u ? u : nullptr;
}

// coefficient of a coarse/fine face: ((beta*ds)/(dx*h))*B*a
// (src/SayakaMacOperator.cpp:1155-1161 and :1258-1266)
template <typename T>
__device__ __forceinline__ T cf_coef(const Coef<T> &c, const Topo &t, int b, int d, int fidx, T h) {
  T v = c.beta * geom(c, b, 3 + d) / (geom(c, b, d) * h);
  v = v * c.bcoef[d][(long)b * t.nfb + fidx];
  v = v * c.afrac[d][(long)b * t.nfb + fidx];
  return v;
}

// CRSE_FINE face: sum of the fine-side contributions T_f * phi_f over the
// fine faces covering coarse face (d, s) of cell ijk of block b, in the
// reference's RESTRICT_SUM order (lower transverse dimension fastest)
template <typename T, int ND, bool CG = false, typename TX = T>
__device__ __forceinline__ T crse_fine_sum(const Topo &t, const Coef<T> &c, int b, int f, const int ijk[3],
                                           const TX *__restrict__ x, const int *__restrict__ hx = nullptr) {
  const int nb = t.nb, half = nb >> 1;
  const int d = f >> 1, s = f & 1;
  int cidx = (1 - s) << d, k = 0;
  int base[3] = {0, 0, 0};
  int tq[2] = {0, 0}, nt = 0;
  for (int q = 0; q < ND; q++) {
    if (q == d) continue;
    const int sq = ijk[q] >= half ? 1 : 0;
    cidx |= sq << q;
    k |= sq << nt;
    base[q] = 2 * (ijk[q] - sq * half);
    tq[nt++] = q;
  }
  const int F = hx ? hx[kHXKids + f * 4 + k] : t.child[t.neighbor[b * 6 + f] * 8 + cidx];
  int fi[3];
  fi[d] = s == 1 ? 0 : nb - 1;
  const int fside = s == 1 ? 0 : 1;  // the fine block's face toward b
  const T h15 = (T)1.5;
  T val = 0;
  const int n1 = ND == 3 ? 2 : 1;
  for (int a1 = 0; a1 < n1; a1++) {
    for (int a0 = 0; a0 < 2; a0++) {
      fi[tq[0]] = base[tq[0]] + a0;
      if (ND == 3) fi[tq[1]] = base[tq[1]] + a1;
      if (ND == 2) fi[2] = 0;
      const int fx = face_index(d, fi, fside, nb);
      const T tf = cf_coef(c, t, F, d, fx, h15);
      val += tf * fpint::cvt<T>(ld<CG>(&x[(long)F * t.ncell + encode(fi, nb)]));
    }
  }
  return val;
}

// value a FINE_CRSE ghost cell holds: the coarse leaf's boundary cell
// (injection through the parent's ghost layer)
template <typename T, int ND, bool CG = false>
__device__ __forceinline__ T fine_crse_ghost(const Topo &t, int b, int f, const int ijk[3], const T *__restrict__ x,
                                             const int *__restrict__ hx = nullptr) {
  const int nb = t.nb, half = nb >> 1;
  const int d = f >> 1, s = f & 1;
  const int C = hx ? hx[f] : t.fc_neigh[b * 6 + f];
  const int wc = hx ? hx[kHXInfo] >> 16 : t.which_child[b];
  int ci[3] = {0, 0, 0};
  for (int q = 0; q < ND; q++) {
    if (q == d)
      ci[q] = s == 1 ? 0 : nb - 1;
    else
      ci[q] = ((wc >> q) & 1) * half + (ijk[q] >> 1);
  }
  return ld<CG>(&x[(long)C * t.ncell + encode(ci, nb)]);
}

// mirrored boundary cell of the same-level neighbour
template <typename T, bool CG = false>
__device__ __forceinline__ T same_level_ghost(const Topo &t, int b, int f, const int ijk[3], const T *__restrict__ x,
                                              const int *__restrict__ hx = nullptr) {
  const int d = f >> 1, s = f & 1;
  const int n = hx ? hx[f] : t.neighbor[b * 6 + f];
  int ni[3] = {ijk[0], ijk[1], ijk[2]};
  ni[d] = s == 1 ? 0 : t.nb - 1;
  return ld<CG>(&x[(long)n * t.ncell + encode(ni, t.nb)]);
}

// operator value of cell ci of block b: (phi_c*sum T - sum T*phi_nb)/dv/vf,
// 0 on cells with vf = 0 (src/SayakaMacOperator.cpp:1325-1459)
template <typename T, int ND, bool CG = false>
__device__ __forceinline__ T apply_cell(const Topo &t, const Coef<T> &c, int b, uint16_t ft, int ci,
                                        const T *__restrict__ x) {
  const int nb = t.nb;
  int ijk[3];
  decode<ND>(ci, nb, ijk);
  const long cb = (long)b * t.ncell;
  const T dv = geom(c, b, 6);
  const T phic = ld<CG>(&x[cb + ci]);
  T diag = c.alpha * dv;
  T off = 0;
#pragma unroll
  for (int f = 0; f < 2 * ND; f++) {
    const int d = f >> 1, s = f & 1;
    const bool bnd = s ? ijk[d] == nb - 1 : ijk[d] == 0;
    const int fx = face_index(d, ijk, s, nb);
    T coef, val;
    if (!bnd) {
      coef = c.tff[d][(long)b * t.nfb + fx];
      const int stride = d == 0 ? 1 : (d == 1 ? nb : nb * nb);
      val = coef * ld<CG>(&x[cb + ci + (s ? stride : -stride)]);
    } else {
      const int ty = face_type_of(ft, f);
      if (ty == 0) {  // FINE_FINE
        coef = c.tff[d][(long)b * t.nfb + fx];
        val = coef * same_level_ghost<T, CG>(t, b, f, ijk, x);
      } else if (ty == 1) {  // FINE_BC
        if (t.bc_type[b * 6 + f] == kBCNeumann) {
          coef = 0;
          val = 0;
        } else {
          coef = c.tff[d][(long)b * t.nfb + fx];
          val = -coef * phic;
        }
      } else if (ty == 2) {  // FINE_CRSE
        coef = cf_coef(c, t, b, d, fx, (T)1.5);
        val = coef * fine_crse_ghost<T, ND, CG>(t, b, f, ijk, x);
      } else {  // CRSE_FINE
        coef = cf_coef(c, t, b, d, fx, (T)0.75);
        val = crse_fine_sum<T, ND, CG>(t, c, b, f, ijk, x);
      }
    }
    diag += coef;
    off += val;
  }
  const T lphi = (phic * diag - off) / dv;
  const T vfv = c.vf[cb + ci];
  return vfv > 0 ? lphi / vfv : (T)0;
}

// one red-black Gauss-Seidel update of cell ijk of block b (tower face types
// ft): unew = (rhs*dv*vf + sum T*phi_nb) / sum T, 0 where vf = 0
// (src/SayakaMacOperator.cpp:1191-1323)
template <typename T, int ND, bool CG = false>
__device__ __forceinline__ void smooth_cell(const Topo &t, const Coef<T> &c, int b, uint16_t ft, const int ijk[3],
                                            T *__restrict__ phi, const T *__restrict__ rhs) {
  const int nb = t.nb;
  const int ci = encode(ijk, nb);
  const long cb = (long)b * t.ncell;
  const T dv = geom(c, b, 6);
  T diag = c.alpha * dv;
  T off = 0;
#pragma unroll
  for (int f = 0; f < 2 * ND; f++) {
    const int d = f >> 1, s = f & 1;
    const bool bnd = s ? ijk[d] == nb - 1 : ijk[d] == 0;
    const int fx = face_index(d, ijk, s, nb);
    T coef, val;
    if (!bnd) {
      coef = c.tff[d][(long)b * t.nfb + fx];
      const int stride = d == 0 ? 1 : (d == 1 ? nb : nb * nb);
      val = coef * ld<CG>(&phi[cb + ci + (s ? stride : -stride)]);
    } else {
      const int ty = face_type_of(ft, f);
      if (ty == 0) {
        coef = c.tff[d][(long)b * t.nfb + fx];
        val = coef * same_level_ghost<T, CG>(t, b, f, ijk, phi);
      } else if (ty == 1) {
        if (t.bc_type[b * 6 + f] == kBCNeumann)
          coef = 0;
        else
          coef = c.tff[d][(long)b * t.nfb + fx] * (T)2.0;
        val = 0;
      } else if (ty == 2) {
        coef = cf_coef(c, t, b, d, fx, (T)1.5);
        val = coef * fine_crse_ghost<T, ND, CG>(t, b, f, ijk, phi);
      } else {
        coef = cf_coef(c, t, b, d, fx, (T)0.75);
        val = crse_fine_sum<T, ND, CG>(t, c, b, f, ijk, phi);
      }
    }
    diag += coef;
    off += val;
  }
  const T vfv = c.vf[cb + ci];
  T unew = 0;
  if (vfv > 0) unew = (ld<CG>(&rhs[cb + ci]) * dv * vfv + off) / diag;
  phi[cb + ci] = unew;
}

__device__ __forceinline__ float fast_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double fast_div(double a, double b) { return a / b; }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }

// the relaxed red-black update of a fluid cell, u_old + omega (u_gs - u_old)
// (successive over-relaxation for omega > 1); omega 1 returns u_gs itself,
// the plain Gauss-Seidel update with the same bits.  omega is a launch
// argument, so the test is uniform over the grid.
template <typename T>
__device__ __forceinline__ T relax(T omega, T unew, T old) {
  return omega == (T)1 ? unew : fma_t(omega, unew - old, old);
}

// red-black update of the device solve's V-cycle: the smoother of
// smooth_cell with 32-bit shift indexing, FMA accumulation and a fast
// division.  Same face coefficients and gathers, different rounding; every
// V-cycle variant of the device solve uses it, so they agree bit for bit.
// With FP64 factors (sa, ia of the block's list entry, see BlockList) the
// diagonal is not summed and unew = rhs*sa + off*ia: no FP64 division.
template <typename T, int ND, bool CG = false>
__device__ __forceinline__ void smooth_cell_fast(const Topo &t, const Coef<T> &c, int b, uint16_t ft,
                                                 const int ijk[3], T *__restrict__ phi, const T *__restrict__ rhs,
                                                 const double *sa = nullptr, const double *ia = nullptr,
                                                 const int *__restrict__ hx = nullptr) {
  const int nb = t.nb;
  const int ci = t.lnb >= 0 ? ijk[0] + ((ijk[1] + (ijk[2] << t.lnb)) << t.lnb) : encode(ijk, nb);
  const long cb = (long)b * t.ncell;
  const long fb = (long)b * t.nfb;
  const T dv = geom(c, b, 6);
  const T *u = uniform_of(c, b);  // constant coefficients: no face or vf loads
  T diag = c.alpha * dv;
  T off = 0;
  bool inner = true;
#pragma unroll
  for (int f = 0; f < 2 * ND; f++) {
    const int d = f >> 1, s = f & 1;
    const bool bnd = s ? ijk[d] == nb - 1 : ijk[d] == 0;
    inner = inner && !bnd;
    // face index (first dimension fastest, nb+1 faces along d)
    int fx;
    if (d == 0)
      fx = ijk[0] + s + (nb + 1) * (ijk[1] + nb * ijk[2]);
    else if (d == 1)
      fx = ijk[0] + nb * (ijk[1] + s + (nb + 1) * ijk[2]);
    else
      fx = ci + s * nb * nb;
    if (!bnd) {
      const T coef = u ? u[d] : c.tff[d][fb + fx];
      const int stride = d == 0 ? 1 : (d == 1 ? nb : nb * nb);
      diag += coef;
      off = fma_t(coef, ld<CG>(&phi[cb + ci + (s ? stride : -stride)]), off);
    } else {
      const int ty = face_type_of(ft, f);
      if (ty == 0) {
        const T coef = u ? u[d] : c.tff[d][fb + fx];
        diag += coef;
        off = fma_t(coef, same_level_ghost<T, CG>(t, b, f, ijk, phi, hx), off);
      } else if (ty == 1) {
        if (t.bc_type[b * 6 + f] != kBCNeumann) diag += (u ? u[d] : c.tff[d][fb + fx]) * (T)2.0;
      } else if (ty == 2) {
        const T coef = cf_coef(c, t, b, d, fx, (T)1.5);
        diag += coef;
        off = fma_t(coef, fine_crse_ghost<T, ND, CG>(t, b, f, ijk, phi, hx), off);
      } else {
        diag += cf_coef(c, t, b, d, fx, (T)0.75);
        off += crse_fine_sum<T, ND, CG>(t, c, b, f, ijk, phi, hx);
      }
    }
  }
  if (sizeof(T) == 8 && sa) {
    const bool ui = u && inner;  // interior cell of a constant-coefficient block
    const T iav = ui ? u[7] : (T)ia[ci];  // 0 in a solid cell
    T unew = fma_t(ld<CG>(&rhs[cb + ci]), ui ? u[6] : (T)sa[ci], off * iav);
    if (c.omega != (T)1 && iav != (T)0) unew = relax(c.omega, unew, ld<CG>(&phi[cb + ci]));
    phi[cb + ci] = unew;
    return;
  }
  const T vfv = u ? (T)1 : c.vf[cb + ci];
  T unew = 0;
  if (vfv > 0 && diag > 0) {
    unew = fast_div(fma_t(ld<CG>(&rhs[cb + ci]) * dv, vfv, off), diag);
    if (c.omega != (T)1) unew = relax(c.omega, unew, ld<CG>(&phi[cb + ci]));
  }
  phi[cb + ci] = unew;
}

// smooth_cell_fast in two halves, for threads that update several cells:
// smooth_gather loads one cell's operands into registers, per face its part
// of the diagonal (dp), the off-diagonal factor (kc) and value (v) -- the
// tiled sweep's form; smooth_update then combines them in the same order
// with the same operations (kc = 1 for a CRSE_FINE face, 0 for a physical
// one: fma(1, v, off) = off + v, fma(0, 0, off) = off), so the result is the
// same as smooth_cell_fast's.  A thread gathers all its cells before
// updating any, so that their global loads are in flight together (none of
// them reads a cell that the launch writes).
template <typename T, int ND>
struct SmoothOps {
  long q;
  T dv, r, vf;
  T dp[2 * ND], kc[2 * ND], v[2 * ND];
  double sa, ia;
  bool fac;
};
template <typename T, int ND>
__device__ __forceinline__ void smooth_gather(const Topo &t, const Coef<T> &c, int b, uint16_t ft, const int ijk[3],
                                              const T *__restrict__ phi, const T *__restrict__ rhs,
                                              const double *sa, const double *ia, const int *__restrict__ hx,
                                              SmoothOps<T, ND> &o) {
  const int nb = t.nb;
  const int ci = t.lnb >= 0 ? ijk[0] + ((ijk[1] + (ijk[2] << t.lnb)) << t.lnb) : encode(ijk, nb);
  const long cb = (long)b * t.ncell;
  const long fb = (long)b * t.nfb;
  const T *u = uniform_of(c, b);
  o.q = cb + ci;
  o.dv = geom(c, b, 6);
  bool inner = true;
#pragma unroll
  for (int f = 0; f < 2 * ND; f++) {
    const int d = f >> 1, s = f & 1;
    const bool bnd = s ? ijk[d] == nb - 1 : ijk[d] == 0;
    inner = inner && !bnd;
    int fx;
    if (d == 0)
      fx = ijk[0] + s + (nb + 1) * (ijk[1] + nb * ijk[2]);
    else if (d == 1)
      fx = ijk[0] + nb * (ijk[1] + s + (nb + 1) * ijk[2]);
    else
      fx = ci + s * nb * nb;
    if (!bnd) {
      const int stride = d == 0 ? 1 : (d == 1 ? nb : nb * nb);
      o.dp[f] = o.kc[f] = u ? u[d] : c.tff[d][fb + fx];
      o.v[f] = phi[cb + ci + (s ? stride : -stride)];
      continue;
    }
    const int ty = face_type_of(ft, f);
    if (ty == 0) {
      o.dp[f] = o.kc[f] = u ? u[d] : c.tff[d][fb + fx];
      o.v[f] = same_level_ghost<T, false>(t, b, f, ijk, phi, hx);
    } else if (ty == 1) {
      o.dp[f] = t.bc_type[b * 6 + f] != kBCNeumann ? (u ? u[d] : c.tff[d][fb + fx]) * (T)2.0 : (T)0;
      o.kc[f] = (T)0;
      o.v[f] = (T)0;
    } else if (ty == 2) {
      o.dp[f] = o.kc[f] = cf_coef(c, t, b, d, fx, (T)1.5);
      o.v[f] = fine_crse_ghost<T, ND, false>(t, b, f, ijk, phi, hx);
    } else {
      o.dp[f] = cf_coef(c, t, b, d, fx, (T)0.75);
      o.kc[f] = (T)1;
      o.v[f] = crse_fine_sum<T, ND, false>(t, c, b, f, ijk, phi, hx);
    }
  }
  o.r = rhs[cb + ci];
  o.fac = sizeof(T) == 8 && sa;
  if (o.fac) {
    const bool ui = u && inner;
    o.sa = ui ? (double)u[6] : sa[ci];
    o.ia = ui ? (double)u[7] : ia[ci];
    o.vf = (T)0;
  } else {
    o.vf = u ? (T)1 : c.vf[cb + ci];
    o.sa = o.ia = 0.0;
  }
}
template <typename T, int ND>
__device__ __forceinline__ void smooth_update(const Coef<T> &c, const SmoothOps<T, ND> &o, T *__restrict__ phi) {
  T diag = c.alpha * o.dv;
  T off = 0;
#pragma unroll
  for (int f = 0; f < 2 * ND; f++) {
    diag += o.dp[f];
    off = fma_t(o.kc[f], o.v[f], off);
  }
  if (o.fac) {
    T unew = fma_t(o.r, (T)o.sa, off * (T)o.ia);
    if (c.omega != (T)1 && o.ia != 0.0) unew = relax(c.omega, unew, phi[o.q]);
    phi[o.q] = unew;
    return;
  }
  T unew = 0;
  if (o.vf > 0 && diag > 0) {
    unew = fast_div(fma_t(o.r * o.dv, o.vf, off), diag);
    if (c.omega != (T)1) unew = relax(c.omega, unew, phi[o.q]);
  }
  phi[o.q] = unew;
}

// colour cell with shifts when nb is a power of two
template <int ND>
__device__ __forceinline__ void color_cell_fast(int h, const Topo &t, int color, int ijk[3]) {
  if (t.lnb < 1) {
    const int hrow = t.nb >> 1;
    const int row = h / hrow;
    ijk[1] = ND >= 2 ? row % t.nb : 0;
    ijk[2] = ND == 3 ? row / t.nb : 0;
    ijk[0] = 2 * (h - row * hrow) + ((color + ijk[1] + ijk[2]) & 1);
    return;
  }
  const int row = h >> (t.lnb - 1);
  ijk[1] = ND >= 2 ? row & (t.nb - 1) : 0;
  ijk[2] = ND == 3 ? row >> t.lnb : 0;
  ijk[0] = 2 * (h & ((t.nb >> 1) - 1)) + ((color + ijk[1] + ijk[2]) & 1);
}

// cell (block-local index ijk) of colour `color` for the h-th half-cell of a block
template <int ND>
__device__ __forceinline__ void color_cell(int h, int nb, int color, int ijk[3]) {
  const int hrow = nb >> 1;
  const int row = h / hrow;
  ijk[1] = ND >= 2 ? row % nb : 0;
  ijk[2] = ND == 3 ? row / nb : 0;
  ijk[0] = 2 * (h - row * hrow) + ((color + ijk[1] + ijk[2]) & 1);
}

// volume-weighted restriction of one coarse cell of non-leaf block b:
// avg(fine*vf_fine)/vf_coarse (src/SayakaMacIB.cpp:157-232,
// src/SayakaInterpPatch.cpp:398-444)
template <typename T, int ND, bool CG = false>
__device__ __forceinline__ void restrict_cell(const Topo &t, const Coef<T> &c, int b, int ci, T *__restrict__ phi,
                                              const int *__restrict__ kids = nullptr) {
  const int nb = t.nb, ncell = t.ncell, half = nb >> 1;
  const T wgt = (T)1.0 / (T)(1 << ND);
  int ijk[3];
  decode<ND>(ci, nb, ijk);
  int cidx = 0, fb[3] = {0, 0, 0};
  for (int q = 0; q < ND; q++) {
    const int sq = ijk[q] >= half ? 1 : 0;
    cidx |= sq << q;
    fb[q] = 2 * (ijk[q] - sq * half);
  }
  const int F = kids ? kids[cidx] : t.child[b * 8 + cidx];
  const long fbase = (long)F * ncell;
  T sum = 0;
  for (int kk = 0; kk < (ND == 3 ? 2 : 1); kk++)
    for (int jj = 0; jj < 2; jj++)
      for (int ii = 0; ii < 2; ii++) {
        const int fi[3] = {fb[0] + ii, fb[1] + jj, ND == 3 ? fb[2] + kk : 0};
        const long q = fbase + encode(fi, nb);
        const T wv = ld<CG>(&phi[q]) * c.vf[q];
        sum += wv;
      }
  const T vfc = c.vf[(long)b * ncell + ci];
  const T avg = sum * wgt;
  phi[(long)b * ncell + ci] = vfc > 0 ? avg / vfc : (T)0;
}

// masked injection of one fine cell of block b from its parent
// (src/SayakaMacIB.cpp:234-283)
template <typename T, int ND, bool CG = false>
__device__ __forceinline__ void prolong_cell(const Topo &t, const Coef<T> &c, int b, int ci, T *__restrict__ phi,
                                             int pw = -1) {
  const int nb = t.nb, ncell = t.ncell, half = nb >> 1;
  int ijk[3];
  decode<ND>(ci, nb, ijk);
  const int P = pw >= 0 ? pw >> 3 : t.parent[b], wc = pw >= 0 ? pw & 7 : t.which_child[b];
  int pc[3] = {0, 0, 0};
  for (int q = 0; q < ND; q++) pc[q] = ((wc >> q) & 1) * half + (ijk[q] >> 1);
  const T v = ld<CG>(&phi[(long)P * ncell + encode(pc, nb)]);
  const long q = (long)b * ncell + ci;
  phi[q] = c.vf[q] > 0 ? v : (T)0;
}

// rows [row0, row0 + 8) of one component of the bottom solve:
// corr = Binv_c * resid_c, one warp per row; rv: shared memory for the
// component's residual (max_n doubles); every thread of the CTA calls it
// a component's residual (rows r0 .. r0+m, whole blocks of ncell rows) into
// shared memory: eight block ids loaded at once, then their cells, so that
// the loads are in flight together instead of one dependent pair per cell
template <typename T, bool CG, typename R>
__device__ __forceinline__ void bottom_gather(const BottomDev &bd, int r0, int m, const T *resid, R *out) {
  const int nc = bd.ncell, nblk = m / nc;
  const int *bl = bd.blocks + r0 / nc;
  for (int p0 = 0; p0 < nblk; p0 += 8) {
    int bb[8];
#pragma unroll
    for (int u = 0; u < 8; u++) bb[u] = p0 + u < nblk ? bl[p0 + u] : -1;
    for (int ci = threadIdx.x; ci < nc; ci += blockDim.x) {
      T v[8];
#pragma unroll
      for (int u = 0; u < 8; u++) v[u] = bb[u] >= 0 ? ld<CG>(&resid[(long)bb[u] * nc + ci]) : (T)0;
#pragma unroll
      for (int u = 0; u < 8; u++)
        if (bb[u] >= 0) out[(p0 + u) * nc + ci] = (R)v[u];
    }
  }
}

template <typename T, bool CG = false>
__device__ __forceinline__ void bottom_tile(const BottomDev &bd, int tile, const T *resid, T *corr, double *rv) {
  const int c = bd.tile_comp[tile], r0 = bd.comp_row0[c], m = bd.comp_n[c], nc = bd.ncell;
  // a finished problem of a forest (per-problem states): nothing to solve
  if (bd.stc && bd.stc[bd.comp[bd.blocks[r0 / nc]]].done) return;
  if (sizeof(T) == 4 && bd.binv16) {  // FP16 rows with FP32 scales, FP32 accumulation
    float *rf = reinterpret_cast<float *>(rv);
    bottom_gather<T, CG>(bd, r0, m, resid, rf);
    __syncthreads();
    const int lane = threadIdx.x & 31, row = bd.tile_row0[tile] + (threadIdx.x >> 5);
    if ((threadIdx.x >> 5) < kBottomTileRows && row < m) {
      // rows start on 16-byte boundaries: m and the component offsets are
      // multiples of the block size (at least 64 cells)
      const uint4 *a8 = reinterpret_cast<const uint4 *>(bd.binv16 + bd.comp_off[c] + (long long)row * m);
      const float4 *r4 = reinterpret_cast<const float4 *>(rf);
      const int q8 = m >> 3;
      float s0 = 0.f, s1 = 0.f;
      auto dot8 = [&](const uint4 u, int j, float &acc) {
        const float2 f0 = __half22float2(*reinterpret_cast<const __half2 *>(&u.x));
        const float2 f1 = __half22float2(*reinterpret_cast<const __half2 *>(&u.y));
        const float2 f2 = __half22float2(*reinterpret_cast<const __half2 *>(&u.z));
        const float2 f3 = __half22float2(*reinterpret_cast<const __half2 *>(&u.w));
        const float4 x0 = r4[2 * j], x1 = r4[2 * j + 1];
        acc = fmaf(f0.x, x0.x, acc);
        acc = fmaf(f0.y, x0.y, acc);
        acc = fmaf(f1.x, x0.z, acc);
        acc = fmaf(f1.y, x0.w, acc);
        acc = fmaf(f2.x, x1.x, acc);
        acc = fmaf(f2.y, x1.y, acc);
        acc = fmaf(f3.x, x1.z, acc);
        acc = fmaf(f3.y, x1.w, acc);
      };
      int j = lane;
      for (; j + 96 < q8; j += 128) {
        const uint4 u0 = a8[j], u1 = a8[j + 32], u2 = a8[j + 64], u3 = a8[j + 96];
        dot8(u0, j, s0);
        dot8(u1, j + 32, s1);
        dot8(u2, j + 64, s0);
        dot8(u3, j + 96, s1);
      }
      for (; j < q8; j += 32) dot8(a8[j], j, s0);
      float s = s0 + s1;
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      const int g = r0 + row;
      if (lane == 0) corr[(long)bd.blocks[g / nc] * nc + g % nc] = (T)(s * bd.rscale[g]);
    }
    __syncthreads();
    return;
  }
  if (sizeof(T) == 4 && bd.binv32) {  // FP32 inverse, FP32 accumulation
    float *rf = reinterpret_cast<float *>(rv);
    bottom_gather<T, CG>(bd, r0, m, resid, rf);
    __syncthreads();
    const int lane = threadIdx.x & 31, row = bd.tile_row0[tile] + (threadIdx.x >> 5);
    if ((threadIdx.x >> 5) < kBottomTileRows && row < m) {
      const float4 *a4 = reinterpret_cast<const float4 *>(bd.binv32 + bd.comp_off[c] + (long long)row * m);
      const float4 *r4 = reinterpret_cast<const float4 *>(rf);
      float s = 0.f;
      if ((m & 3) == 0 && ((bd.comp_off[c] + (long long)row * m) & 3) == 0) {
        // four independent float4 loads in flight per lane
        const int q4 = m >> 2;
        float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
        int j = lane;
        for (; j + 96 < q4; j += 128) {
          const float4 a0 = a4[j], a1 = a4[j + 32], a2 = a4[j + 64], a3 = a4[j + 96];
          const float4 x0 = r4[j], x1 = r4[j + 32], x2 = r4[j + 64], x3 = r4[j + 96];
          s0 = fmaf(a0.w, x0.w, fmaf(a0.z, x0.z, fmaf(a0.y, x0.y, fmaf(a0.x, x0.x, s0))));
          s1 = fmaf(a1.w, x1.w, fmaf(a1.z, x1.z, fmaf(a1.y, x1.y, fmaf(a1.x, x1.x, s1))));
          s2 = fmaf(a2.w, x2.w, fmaf(a2.z, x2.z, fmaf(a2.y, x2.y, fmaf(a2.x, x2.x, s2))));
          s3 = fmaf(a3.w, x3.w, fmaf(a3.z, x3.z, fmaf(a3.y, x3.y, fmaf(a3.x, x3.x, s3))));
        }
        for (; j < q4; j += 32) {
          const float4 a0 = a4[j], x0 = r4[j];
          s0 = fmaf(a0.w, x0.w, fmaf(a0.z, x0.z, fmaf(a0.y, x0.y, fmaf(a0.x, x0.x, s0))));
        }
        s = (s0 + s1) + (s2 + s3);
      } else {
        const float *a = bd.binv32 + bd.comp_off[c] + (long long)row * m;
        for (int j = lane; j < m; j += 32) s = fmaf(a[j], rf[j], s);
      }
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      const int g = r0 + row;
      if (lane == 0) corr[(long)bd.blocks[g / nc] * nc + g % nc] = (T)s;
    }
    __syncthreads();
    return;
  }
  bottom_gather<T, CG>(bd, r0, m, resid, rv);
  __syncthreads();
  const int lane = threadIdx.x & 31, row = bd.tile_row0[tile] + (threadIdx.x >> 5);
  if ((threadIdx.x >> 5) < kBottomTileRows && row < m) {
    const double *a = bd.binv + bd.comp_off[c] + (long long)row * m;
    // four independent loads in flight per lane, four partial sums
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int j = lane;
    for (; j + 96 < m; j += 128) {
      const double a0 = a[j], a1 = a[j + 32], a2 = a[j + 64], a3 = a[j + 96];
      s0 += a0 * rv[j];
      s1 += a1 * rv[j + 32];
      s2 += a2 * rv[j + 64];
      s3 += a3 * rv[j + 96];
    }
    for (; j < m; j += 32) s0 += a[j] * rv[j];
    double s = (s0 + s1) + (s2 + s3);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const int g = r0 + row;
    if (lane == 0) corr[(long)bd.blocks[g / nc] * nc + g % nc] = (T)s;
  }
  __syncthreads();
}

}  // namespace stencil
}  // namespace sayaka_gb300
