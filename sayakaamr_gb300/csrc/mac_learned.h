// Learned block correction for the device solve's V-cycle (2D).
//
// A small convolutional network per block refines the V-cycle's result:
//   z  = V(r)                              (FP32 V-cycle)
//   r1 = r - A z                           (FP32 operator on the tower)
//   z += s * sa * P(net(r1 / s, log10(B) / 3, vf))
// with s = max |r1| over the block, sa = dv*vf/diag the Jacobi factor of the
// cell, and P the projection onto the block-local part (the least-squares
// fit by {1, x, y} over the block removed; the V-cycle keeps the smooth
// part).  net: 3x3 convolutions 3 -> 32 -> 32 -> 1 with ReLU, zero padding
// at the block edge.  Training minimises the residual the correction leaves
// under the block-local operator, over post-V-cycle residuals r1 that come
// from the plain solver's own iterates; the weights are trained on the GPU by
// the FP32 forward/backward kernels of mac_learned.cu (Adam), and inference
// runs the 32 -> 32 layer on tensor cores in BF16 with FP32 accumulation.
#pragma once

#include <cstdint>
#include <vector>

#include "mac_device.h"

namespace sayaka_gb300 {

namespace learned {

constexpr int kC = 32;   // hidden channels
constexpr int kCin = 3;  // residual, log B, vf
// FP32 parameter vector: w1[32][3][9], b1[32], w2[32][32][9], b2[32], w3[32][9], b3
constexpr int kOW1 = 0;
constexpr int kOB1 = kOW1 + kC * kCin * 9;
constexpr int kOW2 = kOB1 + kC;
constexpr int kOB2 = kOW2 + kC * kC * 9;
constexpr int kOW3 = kOB2 + kC;
constexpr int kOB3 = kOW3 + kC * 9;
constexpr int kNParam = kOB3 + 1;

}  // namespace learned

// training set and network state, owned by MacGpu
struct LearnedState {
  int nb = 0;               // block edge (8 or 16)
  float *w = nullptr;       // FP32 master weights [kNParam]
  float *g = nullptr;       // gradient accumulator
  float *m = nullptr, *v = nullptr;  // Adam moments
  uint16_t *w2bf = nullptr; // BF16 copy of w2 in the tensor-core layout [tap][out][in]
  float *loss = nullptr;    // device loss accumulator
  int step = 0;
  // training set: nsamp blocks of features [3][ncell] and the block-local
  // operator data aux = [sa][dv*vf][x-face T][y-face T]
  float *feat = nullptr, *aux = nullptr;
  int nsamp = 0, cap = 0;
  // inference scratch on the finest tower
  float *r1 = nullptr;      // r - A z (FP32, all blocks)
  float *scale = nullptr;   // per list entry
  bool trained = false;
};

// error word of the tcgen05 inference (a tensor-core wait timed out):
// 1 if raised since the last clear, -1 on a CUDA error
int nn_tc_error(bool clear);

}  // namespace sayaka_gb300
