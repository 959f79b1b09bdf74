// Shared device helpers for the bundle-adjustment kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "camera_model.h"

namespace ba {

constexpr unsigned kFull = 0xffffffffu;

// Device error bits, OR-ed into Workspace::err.
enum : uint32_t {
  ERR_BARRIER_TIMEOUT = 1u,  // a group barrier gave up waiting
  ERR_BAD_INDEX = 2u,        // camera / point / group index out of range
  ERR_UNSORTED = 4u,         // observations not sorted by point
  ERR_MODEL_MIX = 8u,        // observation links a camera and a point of different models
  ERR_STRUCTURE = 16u,       // internal index check failed (write skipped)
  ERR_NONFINITE = 32u,       // NaN / Inf in a measurement, prior or initial state; sigma <= 0
};

// Default spin limit of every device-side wait: ~2 s at the maximum SM clock
// (ba_options.wait_limit_cycles overrides it).
constexpr long long kSpinCycles = 4000000000LL;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// Deterministic block sum of N values per thread (fixed tree: lanes by
// butterfly, then warps in index order).  Result valid in thread 0.
// `scratch` holds N * 32 doubles.
template <int N, typename T>
__device__ __forceinline__ void block_sum(T (&v)[N], T* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = warp_sum(v[i]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < N; ++i) scratch[i * 32 + warp] = v[i];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < N; ++i) {
      T s = (T)0;
      for (int w = 0; w < nw; ++w) s += scratch[i * 32 + w];
      v[i] = s;
    }
  }
  __syncthreads();
}

// Symmetric 3x3 stored as 6 upper entries: 00 01 02 11 12 22.
__device__ __forceinline__ void sym3_full(const double* s, double* A) {
  A[0] = s[0]; A[1] = s[1]; A[2] = s[2];
  A[3] = s[1]; A[4] = s[3]; A[5] = s[4];
  A[6] = s[2]; A[7] = s[4]; A[8] = s[5];
}

// 3x3 inverse via the adjugate; false iff the determinant is exactly zero.
__device__ __forceinline__ bool inv3(const double* A, double* Ai) {
  const double c00 = A[4] * A[8] - A[5] * A[7];
  const double c01 = A[5] * A[6] - A[3] * A[8];
  const double c02 = A[3] * A[7] - A[4] * A[6];
  const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
  if (det == 0.0) return false;
  const double id = __drcp_rn(det);  // IEEE 1 / det
  Ai[0] = c00 * id;
  Ai[1] = (A[2] * A[7] - A[1] * A[8]) * id;
  Ai[2] = (A[1] * A[5] - A[2] * A[4]) * id;
  Ai[3] = c01 * id;
  Ai[4] = (A[0] * A[8] - A[2] * A[6]) * id;
  Ai[5] = (A[2] * A[3] - A[0] * A[5]) * id;
  Ai[6] = c02 * id;
  Ai[7] = (A[1] * A[6] - A[0] * A[7]) * id;
  Ai[8] = (A[0] * A[4] - A[1] * A[3]) * id;
  return true;
}

// 6x6 inverse, LU with partial pivoting (row-major); false on a zero pivot.
__device__ __forceinline__ bool inv6(const double* A, double* Ai) {
  double a[36];
  int perm[6];
#pragma unroll
  for (int i = 0; i < 36; ++i) a[i] = A[i];
#pragma unroll
  for (int i = 0; i < 6; ++i) perm[i] = i;
  for (int k = 0; k < 6; ++k) {
    int piv = k;
    double best = fabs(a[6 * k + k]);
    for (int i = k + 1; i < 6; ++i) {
      const double v = fabs(a[6 * i + k]);
      if (v > best) best = v, piv = i;
    }
    if (best == 0.0) return false;
    if (piv != k) {
      for (int j = 0; j < 6; ++j) {
        const double t = a[6 * k + j];
        a[6 * k + j] = a[6 * piv + j];
        a[6 * piv + j] = t;
      }
      const int t = perm[k];
      perm[k] = perm[piv];
      perm[piv] = t;
    }
    const double inv = 1.0 / a[6 * k + k];
    for (int i = k + 1; i < 6; ++i) {
      const double l = a[6 * i + k] * inv;
      a[6 * i + k] = l;
      for (int j = k + 1; j < 6; ++j) a[6 * i + j] -= l * a[6 * k + j];
    }
  }
  for (int j = 0; j < 6; ++j) {
    double x[6];
    for (int i = 0; i < 6; ++i) x[i] = (perm[i] == j) ? 1.0 : 0.0;
    for (int i = 0; i < 6; ++i)
      for (int k = 0; k < i; ++k) x[i] -= a[6 * i + k] * x[k];
    for (int i = 5; i >= 0; --i) {
      for (int k = i + 1; k < 6; ++k) x[i] -= a[6 * i + k] * x[k];
      x[i] /= a[6 * i + i];
    }
    for (int i = 0; i < 6; ++i) Ai[6 * i + j] = x[i];
  }
  return true;
}

}  // namespace ba
