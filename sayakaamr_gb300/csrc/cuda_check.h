// Error-check helpers for MacGpu member functions: a failing CUDA call
// records its message through fail() and returns from the caller.
#pragma once

#include <string>

#define CK(x)                                                 \
  do {                                                        \
    cudaError_t e_ = (x);                                     \
    if (e_ != cudaSuccess) {                                  \
      fail(std::string(#x) + ": " + cudaGetErrorString(e_)); \
      return;                                                 \
    }                                                         \
  } while (0)
#define CKR(x, r)                                             \
  do {                                                        \
    cudaError_t e_ = (x);                                     \
    if (e_ != cudaSuccess) {                                  \
      fail(std::string(#x) + ": " + cudaGetErrorString(e_)); \
      return r;                                               \
    }                                                         \
  } while (0)
#define CK_(x) CK(x)
#define CKR_(x, r) CKR(x, r)
