// Epipolar geometry ahead of bundle adjustment, on the device:
//
//  * fundamental-matrix RANSAC of every photo pair's putative matches
//    (ransac_fundamental, geometry.rs:248-300, called per pair at
//    sparse.rs:290 with threshold 1.5 px, 600 iterations, seed i*7919 + j);
//  * the pair check of the third round (pair_fits, sparse.rs:620-645): the
//    median Sampson error of a pair's matches under the current poses.
//
// RANSAC is split into its data-parallel parts.  Hypothesis samples depend
// on one xorshift stream per pair (each draw depends on the previous), so a
// thread per pair writes all of its pair's samples first.  Then a thread per
// hypothesis fits the normalised 8-point F (the null vector of its 8x9
// system, rank 2 by removing the smallest singular value); each warp counts
// four hypotheses' inliers over the pair's correspondences (FP32 with an
// error bound, FP64 near the threshold: the decisions are the FP64 ones); a
// CTA per pair takes the first hypothesis with the most inliers and refits on
// its inliers (normal matrix, smallest eigenvector).  Geometry in FP64, as
// the reference.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ba_gb300.h"
#include "context.cuh"
#include "primitives.cuh"

namespace ba {
namespace {

constexpr double kF64Max = 1.7976931348623157e308;
constexpr int kFitThreads = 64;
constexpr int kCountThreads = 256;
constexpr int kHypPerCountCta = 32;  // 4 hypotheses per warp
constexpr int kRefitThreads = 128;
constexpr int64_t kMaxChunkHyp = int64_t(1) << 22;

// ---- shared device math -------------------------------------------------------

// normalise (geometry.rs:161-183) of side `side` (0: first photo, 1: second)
// of the eight correspondences idx[0..8): centroid as a running sum of p/8,
// mean distance to it, scale sqrt(2)/d.  Division by 8 is the exact
// multiplication by 0.125.  Writes the similarity T (row-major) and the
// centroid/scale (mx, my, s) used to map points on the fly.
__device__ void ep_normalise8(const double* uv, const uint32_t* idx, int side, double* T,
                              double& mx, double& my, double& s) {
  mx = 0.0, my = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const double* p = uv + 4 * (size_t)idx[i] + 2 * side;
    mx = mx + p[0] * 0.125;
    my = my + p[1] * 0.125;
  }
  double d = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const double* p = uv + 4 * (size_t)idx[i] + 2 * side;
    const double dx = p[0] - mx, dy = p[1] - my;
    d += sqrt(dx * dx + dy * dy);
  }
  d *= 0.125;
  s = d > 1e-12 ? 1.4142135623730951 / d : 1.0;
  T[0] = s, T[1] = 0.0, T[2] = -s * mx;
  T[3] = 0.0, T[4] = s, T[5] = -s * my;
  T[6] = 0.0, T[7] = 0.0, T[8] = 1.0;
}

__device__ __forceinline__ void mul3(const double* A, const double* B, double* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}

// sampson (geometry.rs:233-246).
__device__ __forceinline__ double ep_sampson(const double* F, double ax, double ay, double bx,
                                             double by) {
  const double f0 = F[0] * ax + F[1] * ay + F[2];
  const double f1 = F[3] * ax + F[4] * ay + F[5];
  const double f2 = F[6] * ax + F[7] * ay + F[8];
  const double g0 = F[0] * bx + F[3] * by + F[6];
  const double g1 = F[1] * bx + F[4] * by + F[7];
  const double e = bx * f0 + by * f1 + f2;
  const double d = f0 * f0 + f1 * f1 + g0 * g0 + g1 * g1;
  return d < 1e-18 ? kF64Max : e * e / d;
}

// ---- RANSAC -------------------------------------------------------------------

struct RansacArgs {
  int64_t p0, np;  // pairs [p0, p0 + np) of this chunk
  const uint32_t* match_ptr;
  const double* uv;
  const uint64_t* seed;
  int iters;
  double t2;
  uint32_t* samples;  // [np * iters * 8]
  double* F;          // [np * iters * 9]
  uint8_t* valid;     // [np * iters]
  int32_t* count;     // [np * iters]
  uint32_t* scratch;  // [n_matches] inlier index lists
  uint8_t* inlier;    // [n_matches]
  int32_t* n_inl;     // [n_pairs]
  int32_t* best;      // [n_pairs]
  uint8_t* refit;     // [n_pairs]
  uint32_t* err;
};

__global__ void ransac_sample_kernel(RansacArgs A) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= A.np) return;
  const int64_t p = A.p0 + q;
  const uint32_t n = A.match_ptr[p + 1] - A.match_ptr[p];
  if (n < 12) return;
  uint64_t s = A.seed[p] | 1;
  uint32_t* out = A.samples + (size_t)q * A.iters * 8;
  // s % n without a 64-bit division: with M = floor((2^64 - 1) / n),
  // umulhi(s, M) is floor(s / n) or one less, so one correction is exact.
  const uint64_t M = ~0ull / n;
  for (int it = 0; it < A.iters; ++it) {
    // The eight indices stay in registers: every access below has a
    // compile-time index (fills and duplicate checks are predicated).
    uint32_t idx[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int k = 0;
    // Bounded: with n >= 12 the xorshift stream yields eight distinct
    // residues within a few dozen draws; the cap only guards the loop.
    for (int draws = 0; k < 8; ++draws) {
      if (draws == (1 << 20)) {
        atomicOr(A.err, ERR_STRUCTURE);
#pragma unroll
        for (int j = 0; j < 8; ++j) idx[j] = j;
        break;
      }
      s ^= s << 13;
      s ^= s >> 7;
      s ^= s << 17;
      uint64_t r = s - __umul64hi(s, M) * n;
      if (r >= n) r -= n;
      const uint32_t c = (uint32_t)r;
      bool dup = false;
#pragma unroll
      for (int j = 0; j < 8; ++j) dup |= (j < k) & (idx[j] == c);
      if (!dup) {
#pragma unroll
        for (int j = 0; j < 8; ++j)
          if (j == k) idx[j] = c;
        ++k;
      }
    }
    uint4* o4 = reinterpret_cast<uint4*>(out + 8 * it);
    o4[0] = make_uint4(idx[0], idx[1], idx[2], idx[3]);
    o4[1] = make_uint4(idx[4], idx[5], idx[6], idx[7]);
  }
}

// Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations (registers).
__device__ void jacobi3(double (&A)[3][3], double (&V)[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) V[i][j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    const double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
    const double diag = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
    if (off <= 1e-34 * diag || off == 0.0) break;
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int q = p + 1; q < 3; ++q) {
        if (A[p][q] == 0.0) continue;
        const double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - sn * akq;
          A[k][q] = sn * akp + c * akq;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - sn * aqk;
          A[q][k] = sn * apk + c * aqk;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - sn * vkq;
          V[k][q] = sn * vkp + c * vkq;
        }
      }
  }
}

// Eigenvector of the smallest eigenvalue of the symmetric positive
// semi-definite N x N matrix M (row-major, overwritten) by inverse iteration
// on its pivoted Cholesky factor, from the start vector x (overwritten with
// the unit result).  A pivot below 1e-30 trace(M) is raised to that floor, so
// an exactly singular M yields a null vector.  Single thread.  The reference
// takes this eigenvector from nalgebra's symmetric_eigen (geometry.rs:209-215)
// and the rank-2 step's right singular vector from its SVD (:216-221); any
// accurate method gives it up to sign and rounding when the smallest
// eigenvalue is simple.
template <int N>
__device__ void smallest_eigvec(double* M, double* x) {
  int perm[N];
  double tr = 0.0;
  for (int i = 0; i < N; ++i) perm[i] = i, tr += M[(N + 1) * i];
  const double floor_d = 1e-30 * tr + 1e-300;
  double rdiag[N];
  for (int k = 0; k < N; ++k) {
    int pk = k;
    for (int i = k + 1; i < N; ++i)
      if (M[(N + 1) * i] > M[(N + 1) * pk]) pk = i;
    if (pk != k) {  // symmetric swap of rows/columns k and pk
      for (int j = 0; j < N; ++j) {
        const double t = M[N * k + j];
        M[N * k + j] = M[N * pk + j], M[N * pk + j] = t;
      }
      for (int j = 0; j < N; ++j) {
        const double t = M[N * j + k];
        M[N * j + k] = M[N * j + pk], M[N * j + pk] = t;
      }
      const int t = perm[k];
      perm[k] = perm[pk], perm[pk] = t;
    }
    const double lkk = sqrt(fmax(M[(N + 1) * k], floor_d));
    const double rk = 1.0 / lkk;
    M[(N + 1) * k] = lkk, rdiag[k] = rk;
    for (int i = k + 1; i < N; ++i) M[N * i + k] *= rk;
    for (int i = k + 1; i < N; ++i)
      for (int j = k + 1; j <= i; ++j) {
        M[N * i + j] -= M[N * i + k] * M[N * j + k];
        M[N * j + i] = M[N * i + j];
      }
  }
  // L in the lower triangle: P^T M P = L L^T.
  double nx = 0.0;
  for (int i = 0; i < N; ++i) nx += x[i] * x[i];
  if (!(nx > 1e-300) || !(nx < 1e300)) {  // zero or non-finite start: a generic one
    nx = 0.0;
    for (int i = 0; i < N; ++i) x[i] = 1.0 - 0.0625 * i, nx += x[i] * x[i];
  }
  nx = 1.0 / sqrt(nx);
  for (int i = 0; i < N; ++i) x[i] *= nx;
  for (int it = 0; it < 60; ++it) {
    double y[N];
    for (int i = 0; i < N; ++i) y[i] = x[perm[i]];
    for (int i = 0; i < N; ++i) {  // L z = P^T x
      double a = y[i];
      for (int j = 0; j < i; ++j) a -= M[N * i + j] * y[j];
      y[i] = a * rdiag[i];
    }
    for (int i = N - 1; i >= 0; --i) {  // L^T w = z
      double a = y[i];
      for (int j = i + 1; j < N; ++j) a -= M[N * j + i] * y[j];
      y[i] = a * rdiag[i];
    }
    double z[N], nn = 0.0;
    for (int i = 0; i < N; ++i) z[perm[i]] = y[i];
    for (int i = 0; i < N; ++i) nn += z[i] * z[i];
    nn = 1.0 / sqrt(nn);
    double dot = 0.0;
    for (int i = 0; i < N; ++i) z[i] *= nn, dot += z[i] * x[i];
    const double sg = dot < 0.0 ? -1.0 : 1.0;
    double diff = 0.0;
    for (int i = 0; i < N; ++i) diff = fmax(diff, fabs(sg * z[i] - x[i])), x[i] = sg * z[i];
    if (diff <= 1e-15) break;
  }
}

// Rank 2, denormalisation and unit norm of the 8-point solution f
// (geometry.rs:216-229), as ep_fundamental does after its eigenvector.
__device__ bool ep_finish(const double* fm, const double* ta, const double* tb, double* F) {
  // Right singular vector of fm's smallest singular value: the eigenvector
  // of fm^T fm's smallest eigenvalue.
  double ftf[3][3], W[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      ftf[r][c] = fm[r] * fm[c] + fm[3 + r] * fm[3 + c] + fm[6 + r] * fm[6 + c];
  jacobi3(ftf, W);
  int j = 0;
  if (ftf[1][1] < ftf[j][j]) j = 1;
  if (ftf[2][2] < ftf[j][j]) j = 2;
  const double v0 = j == 0 ? W[0][0] : j == 1 ? W[0][1] : W[0][2];
  const double v1 = j == 0 ? W[1][0] : j == 1 ? W[1][1] : W[1][2];
  const double v2 = j == 0 ? W[2][0] : j == 1 ? W[2][1] : W[2][2];
  double f2[9];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const double fv = fm[3 * r] * v0 + fm[3 * r + 1] * v1 + fm[3 * r + 2] * v2;
    f2[3 * r] = fm[3 * r] - fv * v0;
    f2[3 * r + 1] = fm[3 * r + 1] - fv * v1;
    f2[3 * r + 2] = fm[3 * r + 2] - fv * v2;
  }
  double tbt[9], tmp[9], full[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) tbt[3 * r + c] = tb[3 * c + r];
  mul3(tbt, f2, tmp);
  mul3(tmp, ta, full);
  double nrm = 0.0;
#pragma unroll
  for (int i = 0; i < 9; ++i) nrm += full[i] * full[i];
  nrm = sqrt(nrm);
  if (!(nrm > 1e-15)) return false;
#pragma unroll
  for (int i = 0; i < 9; ++i) F[i] = full[i] / nrm;
  return true;
}

// The 8-point hypothesis (geometry.rs:186-230 on eight correspondences).
// Its normal matrix M = A^T A has the null vector of the 8x9 system A as the
// eigenvector of its zero eigenvalue, which is the one the reference takes;
// here that null vector comes from A directly, by Gaussian elimination with
// full pivoting (about 500 operations instead of a 9x9 eigen-decomposition).
// The two agree to rounding for any sample of rank 8; for a rank-deficient
// sample both return some vector of the null space.  A lives in shared
// memory, element (r, c) at As[(9 r + c) * stride].
__device__ bool ep_fundamental8(const double* uv, const uint32_t* idx, double* As, int stride,
                                double* F) {
  double ta[9], tb[9], ax, ay, as, bx, by, bs;
  ep_normalise8(uv, idx, 0, ta, ax, ay, as);
  ep_normalise8(uv, idx, 1, tb, bx, by, bs);
#define AS(r, c) As[(9 * (r) + (c)) * stride]
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const double* u = uv + 4 * (size_t)idx[i];
    const double p0 = (u[0] - ax) * as, p1 = (u[1] - ay) * as;
    const double q0 = (u[2] - bx) * bs, q1 = (u[3] - by) * bs;
    AS(i, 0) = q0 * p0, AS(i, 1) = q0 * p1, AS(i, 2) = q0;
    AS(i, 3) = q1 * p0, AS(i, 4) = q1 * p1, AS(i, 5) = q1;
    AS(i, 6) = p0, AS(i, 7) = p1, AS(i, 8) = 1.0;
  }
  uint64_t perm = 0;  // 4 bits per column: original index of column k
#pragma unroll
  for (int c = 0; c < 9; ++c) perm |= (uint64_t)c << (4 * c);
  int rank = 8;
  for (int k = 0; k < 8; ++k) {
    // Pivot choice on FP32 magnitudes (the choice only steers stability);
    // a zero pivot is tested exactly.
    int pr = k, pc = k;
    float best = -1.0f;
    for (int r = k; r < 8; ++r)
      for (int c = k; c < 9; ++c) {
        const float v = fabsf((float)AS(r, c));
        if (v > best) best = v, pr = r, pc = c;
      }
    if (AS(pr, pc) == 0.0) {
      rank = k;
      break;
    }
    if (pr != k)
      for (int c = 0; c < 9; ++c) {
        const double t = AS(k, c);
        AS(k, c) = AS(pr, c), AS(pr, c) = t;
      }
    if (pc != k) {
      for (int r = 0; r < 8; ++r) {
        const double t = AS(r, k);
        AS(r, k) = AS(r, pc), AS(r, pc) = t;
      }
      const uint64_t a = (perm >> (4 * k)) & 15, b = (perm >> (4 * pc)) & 15;
      perm &= ~((uint64_t)15 << (4 * k)) & ~((uint64_t)15 << (4 * pc));
      perm |= (b << (4 * k)) | (a << (4 * pc));
    }
    const double rpiv = 1.0 / AS(k, k);
    for (int r = k + 1; r < 8; ++r) {
      const double m = AS(r, k) * rpiv;
      for (int c = k + 1; c < 9; ++c) AS(r, c) -= m * AS(k, c);
    }
  }
  // Null vector: the free (last unpivoted) unknown is 1, the rest follow by
  // back-substitution through the upper-triangular rows 0..rank-1.
  double x[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) x[c] = c == rank ? 1.0 : 0.0;
  for (int k = rank - 1; k >= 0; --k) {
    double acc = 0.0;
    for (int c = k + 1; c < 9; ++c) acc += AS(k, c) * (c == rank ? 1.0 : (c < rank ? x[c] : 0.0));
    x[k] = -acc / AS(k, k);
  }
#undef AS
  double fm[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) fm[c] = 0.0;
  for (int c = 0; c < 9; ++c) {
    const int o = (int)((perm >> (4 * c)) & 15);
#pragma unroll
    for (int t = 0; t < 9; ++t)
      if (t == o) fm[t] = x[c];
  }
  double nn = 0.0;
#pragma unroll
  for (int c = 0; c < 9; ++c) nn += fm[c] * fm[c];
  nn = sqrt(nn);
#pragma unroll
  for (int c = 0; c < 9; ++c) fm[c] /= nn;
  return ep_finish(fm, ta, tb, F);
}

__global__ void __launch_bounds__(kFitThreads) ransac_fit_kernel(RansacArgs A) {
  __shared__ double As[72 * kFitThreads];
  const int64_t h = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= A.np * A.iters) return;
  const int64_t p = A.p0 + h / A.iters;
  const uint32_t b = A.match_ptr[p], n = A.match_ptr[p + 1] - b;
  A.valid[h] = 0;
  if (n < 12) return;
  uint32_t idx[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) idx[j] = A.samples[8 * h + j];
  double F[9];
  if (!ep_fundamental8(A.uv + 4 * (size_t)b, idx, As + threadIdx.x, kFitThreads, F)) return;
#pragma unroll
  for (int j = 0; j < 9; ++j) A.F[9 * h + j] = F[j];
  A.valid[h] = 1;
}

// Inlier test of one correspondence against one hypothesis, decided in FP32
// with a rounding-error bound and in FP64 (ep_sampson, as the reference) only
// when the FP32 value is too close to the threshold to be sure.  With
// u = 2^-24, each FP32 value x_hat of the test carries a bound dx on
// |x_hat - x| (x exact from the FP64 inputs): inputs rounded to FP32 and a
// three-term FMA dot product stay within 8u of the sum of the terms'
// magnitudes, and e = b^T F a, d = |(F a)_xy|^2 + |(F^T b)_xy|^2 propagate
// those.  "Surely in" means e^2 < t^2 d (1 - 32u) for every e, d in their
// intervals; "surely out" the converse; the FP64 evaluation's own error
// (about 2^-50 relative) is far inside those margins, so the decisions
// equal the FP64 ones.
struct Hyp32 {
  float f[9];
};

// 1: surely an inlier, 0: surely not, -1: evaluate in FP64.
__device__ __forceinline__ int inlier_fp32(const Hyp32& H, float4 c, float t2) {
  constexpr float u = 5.9604645e-8f;  // 2^-24
  const float* f = H.f;
  const float ax = c.x, ay = c.y, bx = c.z, by = c.w;
  const float f0 = fmaf(f[0], ax, fmaf(f[1], ay, f[2]));
  const float f1 = fmaf(f[3], ax, fmaf(f[4], ay, f[5]));
  const float f2 = fmaf(f[6], ax, fmaf(f[7], ay, f[8]));
  const float g0 = fmaf(f[0], bx, fmaf(f[3], by, f[6]));
  const float g1 = fmaf(f[1], bx, fmaf(f[4], by, f[7]));
  const float af = fabsf(ax), ag = fabsf(ay), bf = fabsf(bx), bg = fabsf(by);
  const float d0 = 8.0f * u * fmaf(fabsf(f[0]), af, fmaf(fabsf(f[1]), ag, fabsf(f[2])));
  const float d1 = 8.0f * u * fmaf(fabsf(f[3]), af, fmaf(fabsf(f[4]), ag, fabsf(f[5])));
  const float d2 = 8.0f * u * fmaf(fabsf(f[6]), af, fmaf(fabsf(f[7]), ag, fabsf(f[8])));
  const float e0 = 8.0f * u * fmaf(fabsf(f[0]), bf, fmaf(fabsf(f[3]), bg, fabsf(f[6])));
  const float e1 = 8.0f * u * fmaf(fabsf(f[1]), bf, fmaf(fabsf(f[4]), bg, fabsf(f[7])));
  const float e = fmaf(bx, f0, fmaf(by, f1, f2));
  const float de = fmaf(bf, d0, fmaf(bg, d1, d2)) +
                   8.0f * u * fmaf(bf, fabsf(f0), fmaf(bg, fabsf(f1), fabsf(f2)));
  const float d = fmaf(f0, f0, fmaf(f1, f1, fmaf(g0, g0, g1 * g1)));
  const float dd = fmaf(d0, fmaf(2.0f, fabsf(f0), d0),
                        fmaf(d1, fmaf(2.0f, fabsf(f1), d1),
                             fmaf(e0, fmaf(2.0f, fabsf(g0), e0), e1 * fmaf(2.0f, fabsf(g1), e1)))) +
                   8.0f * u * d;
  const float ae = fabsf(e);
  const float lo = d - dd, hi = d + dd;
  if (lo > 2e-18f) {
    const float in_l = (ae + de) * (ae + de), in_r = t2 * lo * (1.0f - 32.0f * u);
    if (in_l < in_r) return 1;
    const float out_e = ae - de;
    if (out_e > 0.0f && out_e * out_e > t2 * hi * (1.0f + 32.0f * u)) return 0;
  } else if (hi < 5e-19f && hi >= 0.0f) {
    return 0;  // the FP64 d is below 1e-18: f64::MAX, never an inlier
  }
  return -1;
}

constexpr int kCountTile = 1024;

// First-tier bounds of one hypothesis over one tile of correspondences, from
// the tile's largest coordinate magnitudes (ax, ay, bx, by): every |f_k| is
// at most S_k, so the error bounds of inlier_fp32 become constants de, dd
// (plus the 8u d term of d's own rounding).
struct TileBound {
  float de, dd;
};

__device__ __forceinline__ TileBound tile_bound(const Hyp32& H, float4 m) {
  constexpr float u = 5.9604645e-8f;
  const float* f = H.f;
  const float S0 = fmaf(fabsf(f[0]), m.x, fmaf(fabsf(f[1]), m.y, fabsf(f[2])));
  const float S1 = fmaf(fabsf(f[3]), m.x, fmaf(fabsf(f[4]), m.y, fabsf(f[5])));
  const float S2 = fmaf(fabsf(f[6]), m.x, fmaf(fabsf(f[7]), m.y, fabsf(f[8])));
  const float T0 = fmaf(fabsf(f[0]), m.z, fmaf(fabsf(f[3]), m.w, fabsf(f[6])));
  const float T1 = fmaf(fabsf(f[1]), m.z, fmaf(fabsf(f[4]), m.w, fabsf(f[7])));
  const float d0 = 8.0f * u * S0, d1 = 8.0f * u * S1, d2 = 8.0f * u * S2;
  const float e0 = 8.0f * u * T0, e1 = 8.0f * u * T1;
  TileBound B;
  // |f_hat| <= S + d; bounds rounded up by the 2x in the factors.
  B.de = 2.0f * (fmaf(m.z, d0, fmaf(m.w, d1, d2)) +
                 8.0f * u * fmaf(m.z, S0 + d0, fmaf(m.w, S1 + d1, S2 + d2)));
  B.dd = 2.0f * (d0 * (2.0f * (S0 + d0) + d0) + d1 * (2.0f * (S1 + d1) + d1) +
                 e0 * (2.0f * (T0 + e0) + e0) + e1 * (2.0f * (T1 + e1) + e1));
  return B;
}

// 1 / 0 surely in / out by the tile's constant bounds, -1 undecided.
__device__ __forceinline__ int inlier_tile(const Hyp32& H, const TileBound& B, float4 c,
                                           float t2) {
  constexpr float u = 5.9604645e-8f;
  const float* f = H.f;
  const float f0 = fmaf(f[0], c.x, fmaf(f[1], c.y, f[2]));
  const float f1 = fmaf(f[3], c.x, fmaf(f[4], c.y, f[5]));
  const float f2 = fmaf(f[6], c.x, fmaf(f[7], c.y, f[8]));
  const float g0 = fmaf(f[0], c.z, fmaf(f[3], c.w, f[6]));
  const float g1 = fmaf(f[1], c.z, fmaf(f[4], c.w, f[7]));
  const float ae = fabsf(fmaf(c.z, f0, fmaf(c.w, f1, f2)));
  const float d = fmaf(f0, f0, fmaf(f1, f1, fmaf(g0, g0, g1 * g1)));
  const float dd = fmaf(8.0f * u, d, B.dd);
  const float lo = d - dd;
  if (lo > 2e-18f) {
    const float a = ae + B.de;
    if (a * a < t2 * lo * (1.0f - 32.0f * u)) return 1;
    const float o = ae - B.de;
    if (o > 0.0f && o * o > t2 * (d + dd) * (1.0f + 32.0f * u)) return 0;
  }
  return -1;
}

// CTA per (pair, 32 hypotheses); each warp tests four hypotheses against
// every correspondence of the pair, the pair's FP32 coordinates staged
// through shared memory a tile at a time.  Tests are decided by the tile's
// constant bounds, else by the correspondence's own bounds, else in FP64.
__global__ void __launch_bounds__(kCountThreads) ransac_count_kernel(RansacArgs A,
                                                                     const float4* uv32) {
  __shared__ float4 tile[kCountTile];
  __shared__ float4 wmax[kCountThreads / 32];
  const int blocks_per_pair = (A.iters + kHypPerCountCta - 1) / kHypPerCountCta;
  const int64_t q = blockIdx.x / blocks_per_pair;
  const int hb = (int)(blockIdx.x % blocks_per_pair) * kHypPerCountCta;
  const int64_t p = A.p0 + q;
  const uint32_t b = A.match_ptr[p], n = A.match_ptr[p + 1] - b;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int kPerWarp = kHypPerCountCta / (kCountThreads / 32);
  const float t2 = (float)A.t2;
  Hyp32 H[kPerWarp];
  bool ok[kPerWarp];
  int cnt[kPerWarp];
#pragma unroll
  for (int j = 0; j < kPerWarp; ++j) {
    const int it = hb + warp * kPerWarp + j;
    const int64_t h = q * A.iters + it;
    ok[j] = n >= 12 && it < A.iters && A.valid[h];
    cnt[j] = 0;
#pragma unroll
    for (int k = 0; k < 9; ++k) H[j].f[k] = ok[j] ? (float)A.F[9 * h + k] : 0.0f;
  }
  if (n < 12) {
    if (lane < kPerWarp && hb + warp * kPerWarp + lane < A.iters)
      A.count[q * A.iters + hb + warp * kPerWarp + lane] = 0;
    return;
  }
  for (uint32_t t0 = 0; t0 < n; t0 += kCountTile) {
    const uint32_t tn = min((uint32_t)kCountTile, n - t0);
    __syncthreads();
    float4 m = make_float4(0.f, 0.f, 0.f, 0.f);
    for (uint32_t i = threadIdx.x; i < tn; i += kCountThreads) {
      const float4 c = uv32[b + t0 + i];
      tile[i] = c;
      m.x = fmaxf(m.x, fabsf(c.x)), m.y = fmaxf(m.y, fabsf(c.y));
      m.z = fmaxf(m.z, fabsf(c.z)), m.w = fmaxf(m.w, fabsf(c.w));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      m.x = fmaxf(m.x, __shfl_xor_sync(kFull, m.x, o));
      m.y = fmaxf(m.y, __shfl_xor_sync(kFull, m.y, o));
      m.z = fmaxf(m.z, __shfl_xor_sync(kFull, m.z, o));
      m.w = fmaxf(m.w, __shfl_xor_sync(kFull, m.w, o));
    }
    if (lane == 0) wmax[warp] = m;
    __syncthreads();
#pragma unroll
    for (int w = 0; w < kCountThreads / 32; ++w) {
      const float4 v = wmax[w];
      m.x = fmaxf(m.x, v.x), m.y = fmaxf(m.y, v.y), m.z = fmaxf(m.z, v.z), m.w = fmaxf(m.w, v.w);
    }
    TileBound TB[kPerWarp];
#pragma unroll
    for (int j = 0; j < kPerWarp; ++j) TB[j] = tile_bound(H[j], m);
    for (uint32_t i = lane; i < tn; i += 32) {
      const float4 c = tile[i];
#pragma unroll
      for (int j = 0; j < kPerWarp; ++j) {
        if (!ok[j]) continue;
        int r = inlier_tile(H[j], TB[j], c, t2);
        if (r < 0) r = inlier_fp32(H[j], c, t2);
        if (r < 0) {
          const int64_t h = q * A.iters + hb + warp * kPerWarp + j;
          const double* u64 = A.uv + 4 * ((size_t)b + t0 + i);
          r = ep_sampson(A.F + 9 * h, u64[0], u64[1], u64[2], u64[3]) < A.t2;
        }
        cnt[j] += r;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < kPerWarp; ++j) {
    int v = cnt[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    const int it = hb + warp * kPerWarp + j;
    if (lane == 0 && it < A.iters) A.count[q * A.iters + it] = ok[j] ? v : 0;
  }
}

__global__ void uv_f32_kernel(int64_t n, const double* uv, float4* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* u = uv + 4 * i;
  out[i] = make_float4((float)u[0], (float)u[1], (float)u[2], (float)u[3]);
}

__device__ __forceinline__ uint64_t cta_max_u64(uint64_t v, uint64_t* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, (uint64_t)__shfl_xor_sync(kFull, v, o));
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < kRefitThreads / 32 ? red[lane] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, (uint64_t)__shfl_xor_sync(kFull, v, o));
    if (lane == 0) red[kRefitThreads / 32] = v;
  }
  __syncthreads();
  const uint64_t r = red[kRefitThreads / 32];
  __syncthreads();
  return r;
}

__device__ __forceinline__ int cta_sum_int(int v, int* wsum) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = v;
  __syncthreads();
  int t = 0;
  for (int w = 0; w < kRefitThreads / 32; ++w) t += wsum[w];
  __syncthreads();
  return t;
}

// Inlier flags of F for the CTA's pair into `flag`, and the inlier indices
// in correspondence order into `list`; returns the count.
__device__ int mark_inliers(const double* F, const double* uv, uint32_t n, double t2,
                            uint8_t* flag, uint32_t* list, int* wsum) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ int base_s;
  if (threadIdx.x == 0) base_s = 0;
  __syncthreads();
  for (uint32_t i0 = 0; i0 < n; i0 += kRefitThreads) {
    const uint32_t i = i0 + threadIdx.x;
    bool in = false;
    if (i < n) {
      const double* u = uv + 4 * (size_t)i;
      in = ep_sampson(F, u[0], u[1], u[2], u[3]) < t2;
      flag[i] = in;
    }
    const unsigned m = __ballot_sync(kFull, in);
    if (lane == 0) wsum[warp] = __popc(m);
    __syncthreads();
    int off = base_s;
    for (int w = 0; w < warp; ++w) off += wsum[w];
    if (in) list[off + __popc(m & ((1u << lane) - 1u))] = i;
    __syncthreads();
    if (threadIdx.x == 0)
      for (int w = 0; w < kRefitThreads / 32; ++w) base_s += wsum[w];
    __syncthreads();
  }
  return base_s;
}

__device__ __forceinline__ double cta_sum_d(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
#pragma unroll
  for (int w = 0; w < kRefitThreads / 32; ++w) t += red[w];
  __syncthreads();
  return t;
}

// CTA per pair: the best hypothesis (the first with the most inliers), its
// inliers, and one refit on them (geometry.rs:286-298), kept when it has at
// least as many inliers.  The refit's centroid, mean distance and normal
// matrix are CTA reductions in a fixed order; its eigenvector comes from
// smallest_eigvec9.
__global__ void __launch_bounds__(kRefitThreads) ransac_select_kernel(RansacArgs A) {
  __shared__ uint64_t red[kRefitThreads / 32 + 1];
  __shared__ int wsum[kRefitThreads / 32];
  __shared__ double dred[kRefitThreads / 32];
  __shared__ double msum[kRefitThreads / 32][45];
  __shared__ double Ms[81];
  __shared__ double Fs[9];
  __shared__ int ok_s;
  const int64_t q = blockIdx.x, p = A.p0 + q;
  const uint32_t b = A.match_ptr[p], n = A.match_ptr[p + 1] - b;
  uint8_t* flag = A.inlier + b;
  for (uint32_t i = threadIdx.x; i < n; i += kRefitThreads) flag[i] = 0;
  if (threadIdx.x == 0) A.n_inl[p] = 0, A.best[p] = -1, A.refit[p] = 0;
  if (n < 12) return;
  uint64_t key = 0;
  for (int it = threadIdx.x; it < A.iters; it += kRefitThreads) {
    const int c = A.count[q * A.iters + it];
    if (c > 0) key = max(key, ((uint64_t)c << 32) | (uint32_t)(0x7fffffff - it));
  }
  key = cta_max_u64(key, red);
  if (key == 0) return;
  const int hbest = 0x7fffffff - (int)(uint32_t)key;
  if (threadIdx.x < 9) Fs[threadIdx.x] = A.F[9 * (q * A.iters + hbest) + threadIdx.x];
  __syncthreads();
  const double* U = A.uv + 4 * (size_t)b;
  uint32_t* list = A.scratch + b;
  const int nb = mark_inliers(Fs, U, n, A.t2, flag, list, wsum);
  if (threadIdx.x == 0) A.best[p] = hbest, A.n_inl[p] = nb;
  if (nb < 8) return;
  // normalise (geometry.rs:161-183) of both sides over the inliers.
  const double nn = (double)nb;
  double sa = 0.0, sb = 0.0, sc = 0.0, sd = 0.0;
  for (int i = threadIdx.x; i < nb; i += kRefitThreads) {
    const double* u = U + 4 * (size_t)list[i];
    sa += u[0] / nn, sb += u[1] / nn, sc += u[2] / nn, sd += u[3] / nn;
  }
  const double max_ = cta_sum_d(sa, dred), may = cta_sum_d(sb, dred);
  const double mbx = cta_sum_d(sc, dred), mby = cta_sum_d(sd, dred);
  double da = 0.0, db = 0.0;
  for (int i = threadIdx.x; i < nb; i += kRefitThreads) {
    const double* u = U + 4 * (size_t)list[i];
    const double x0 = u[0] - max_, y0 = u[1] - may, x1 = u[2] - mbx, y1 = u[3] - mby;
    da += sqrt(x0 * x0 + y0 * y0), db += sqrt(x1 * x1 + y1 * y1);
  }
  const double dA = cta_sum_d(da, dred) / nn, dB = cta_sum_d(db, dred) / nn;
  const double sA = dA > 1e-12 ? 1.4142135623730951 / dA : 1.0;
  const double sB = dB > 1e-12 ? 1.4142135623730951 / dB : 1.0;
  // Normal matrix, upper triangle (45 entries) per thread, then in order.
  double acc[45];
#pragma unroll
  for (int k = 0; k < 45; ++k) acc[k] = 0.0;
  for (int i = threadIdx.x; i < nb; i += kRefitThreads) {
    const double* u = U + 4 * (size_t)list[i];
    const double p0 = (u[0] - max_) * sA, p1 = (u[1] - may) * sA;
    const double q0 = (u[2] - mbx) * sB, q1 = (u[3] - mby) * sB;
    const double row[9] = {q0 * p0, q0 * p1, q0, q1 * p0, q1 * p1, q1, p0, p1, 1.0};
    int k = 0;
#pragma unroll
    for (int r = 0; r < 9; ++r)
#pragma unroll
      for (int c = r; c < 9; ++c) acc[k++] += row[r] * row[c];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 45; ++k) {
    double v = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    if (lane == 0) msum[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 45) {
    double t = 0.0;
    for (int w = 0; w < kRefitThreads / 32; ++w) t += msum[w][threadIdx.x];
    int r = 0, k = threadIdx.x;
    while (k >= 9 - r) k -= 9 - r, ++r;
    const int c = r + k;
    Ms[9 * r + c] = t, Ms[9 * c + r] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double fm[9], F[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) fm[i] = 1.0 - 0.0625 * i;
    smallest_eigvec<9>(Ms, fm);
    const double ta[9] = {sA, 0.0, -sA * max_, 0.0, sA, -sA * may, 0.0, 0.0, 1.0};
    const double tb[9] = {sB, 0.0, -sB * mbx, 0.0, sB, -sB * mby, 0.0, 0.0, 1.0};
    ok_s = ep_finish(fm, ta, tb, F);
    if (ok_s)
      for (int j = 0; j < 9; ++j) Fs[j] = F[j];
  }
  __syncthreads();
  if (!ok_s) return;
  int cnt = 0;
  for (uint32_t i = threadIdx.x; i < n; i += kRefitThreads) {
    const double* u = U + 4 * (size_t)i;
    cnt += ep_sampson(Fs, u[0], u[1], u[2], u[3]) < A.t2;
  }
  const int nr = cta_sum_int(cnt, wsum);
  if (nr < nb) return;
  mark_inliers(Fs, U, n, A.t2, flag, list, wsum);
  if (threadIdx.x == 0) A.n_inl[p] = nr, A.refit[p] = 1;
}

// ---- pair_fits ----------------------------------------------------------------

__device__ __forceinline__ void undistort(const double* K, const double* u, double* p) {
  const double qx = (u[0] - K[1]) / K[0], qy = (u[1] - K[2]) / K[0];
  double px = qx, py = qy;
  for (int i = 0; i < 8; ++i) {
    const double r2 = px * px + py * py;
    const double d = 1.0 + K[3] * r2 + K[4] * r2 * r2;
    px = qx / d;
    py = qy / d;
  }
  p[0] = px, p[1] = py;
}

__device__ __forceinline__ uint64_t total_order_key(double z) {
  const uint64_t b = (uint64_t)__double_as_longlong(z);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_total_order_key(uint64_t k) {
  const uint64_t b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}

struct FitsArgs {
  int64_t n_pairs;
  const uint32_t* pair_cam;
  const uint32_t* match_ptr;
  const double* uv;
  const double* rot;
  const double* center;
  const double* intr;
  const uint32_t* cam_group;
  uint64_t* key;  // [n_matches] total-order key of the error
  uint32_t* pair; // [n_matches]
};

// CTA per pair: E = [t]x R_b R_a^T, t = R_b (C_a - C_b) (sparse.rs:629-631),
// then every match's error sqrt(sampson) * f_a on undistorted coordinates.
__global__ void pair_err_kernel(FitsArgs A) {
  __shared__ double E[9];
  const int64_t p = blockIdx.x;
  const uint32_t ca = A.pair_cam[2 * p], cb = A.pair_cam[2 * p + 1];
  const double* Ka = A.intr + 5 * (size_t)A.cam_group[ca];
  const double* Kb = A.intr + 5 * (size_t)A.cam_group[cb];
  if (threadIdx.x == 0) {
    const double* Ra = A.rot + 9 * (size_t)ca;
    const double* Rb = A.rot + 9 * (size_t)cb;
    double RaT[9], R[9], S[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) RaT[3 * r + c] = Ra[3 * c + r];
    mul3(Rb, RaT, R);
    const double d0 = A.center[3 * ca] - A.center[3 * cb];
    const double d1 = A.center[3 * ca + 1] - A.center[3 * cb + 1];
    const double d2 = A.center[3 * ca + 2] - A.center[3 * cb + 2];
    double t[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) t[r] = Rb[3 * r] * d0 + Rb[3 * r + 1] * d1 + Rb[3 * r + 2] * d2;
    S[0] = 0.0, S[1] = -t[2], S[2] = t[1];
    S[3] = t[2], S[4] = 0.0, S[5] = -t[0];
    S[6] = -t[1], S[7] = t[0], S[8] = 0.0;
    double Et[9];
    mul3(S, R, Et);
    for (int j = 0; j < 9; ++j) E[j] = Et[j];
  }
  __syncthreads();
  double Er[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) Er[j] = E[j];
  for (uint32_t i = A.match_ptr[p] + threadIdx.x; i < A.match_ptr[p + 1]; i += blockDim.x) {
    double x1[2], x2[2];
    undistort(Ka, A.uv + 4 * (size_t)i, x1);
    undistort(Kb, A.uv + 4 * (size_t)i + 2, x2);
    const double err = sqrt(ep_sampson(Er, x1[0], x1[1], x2[0], x2[1])) * Ka[0];
    A.key[i] = total_order_key(err);
    A.pair[i] = (uint32_t)p;
  }
}

__global__ void pair_swap_kernel(int64_t n, const uint64_t* key, const uint32_t* pair,
                                 uint64_t* okey, uint64_t* oval) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  okey[i] = pair[i];
  oval[i] = key[i];
}

__global__ void pair_median_kernel(int64_t n_pairs, const uint32_t* match_ptr,
                                   const uint64_t* sorted, double* median) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_pairs) return;
  const uint32_t b = match_ptr[p], n = match_ptr[p + 1] - b;
  median[p] = n ? from_total_order_key(sorted[b + n / 2]) : kF64Max;
}

// ---- input checks ---------------------------------------------------------------

__global__ void check_pairs_kernel(int64_t n_pairs, int64_t n_matches, const uint32_t* match_ptr,
                                   const uint32_t* pair_cam, int64_t nc, const uint32_t* cam_group,
                                   int64_t ng, uint32_t* err) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p > n_pairs) return;
  if (p == 0 && match_ptr[0] != 0) atomicOr(err, ERR_BAD_INDEX);
  if (p == n_pairs) {
    if (match_ptr[p] != (uint64_t)n_matches) atomicOr(err, ERR_BAD_INDEX);
    return;
  }
  if (match_ptr[p + 1] < match_ptr[p]) atomicOr(err, ERR_BAD_INDEX);
  if (pair_cam) {
    const uint32_t a = pair_cam[2 * p], c = pair_cam[2 * p + 1];
    if (a >= (uint64_t)nc || c >= (uint64_t)nc) {
      atomicOr(err, ERR_BAD_INDEX);
    } else if (cam_group && (cam_group[a] >= (uint64_t)ng || cam_group[c] >= (uint64_t)ng)) {
      atomicOr(err, ERR_BAD_INDEX);
    }
  }
}

__global__ void default_seed_kernel(int64_t n_pairs, const uint32_t* pair_cam, uint64_t* seed) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n_pairs) seed[p] = (uint64_t)pair_cam[2 * p] * 7919u + pair_cam[2 * p + 1];
}

template <typename T>
void upload_n(DevBuf<T>& d, const T* h, int64_t n, cudaStream_t s) {
  d.alloc(std::max<int64_t>(n, 1), s);
  if (n > 0) check(cudaMemcpyAsync(d.p, h, n * sizeof(T), cudaMemcpyDefault, s), "copy in");
}

template <typename T>
void download_n(T* h, const DevBuf<T>& d, int64_t n, cudaStream_t s) {
  if (h && n > 0) check(cudaMemcpyAsync(h, d.p, n * sizeof(T), cudaMemcpyDefault, s), "copy out");
}

struct PairsIn {
  int64_t np = 0, nm = 0;
  DevBuf<uint32_t> match_ptr, pair_cam, err;
  DevBuf<double> uv;

  void load(const ba_pair_matches* m, bool need_cams, int64_t nc, const uint32_t* cam_group_dev,
            int64_t ng, cudaStream_t s) {
    if (!m) throw BadInput("null pair matches");
    np = m->n_pairs, nm = m->n_matches;
    if (np < 0 || nm < 0) throw BadInput("negative size");
    if (nm > 0xfffffff0LL || np > 0x7ffffff0LL) throw BadInput("too many pairs or matches");
    if (!m->match_ptr) throw BadInput("null match_ptr");
    if (nm > 0 && !m->uv) throw BadInput("null uv");
    if (need_cams && np > 0 && !m->pair_cam) throw BadInput("null pair_cam");
    upload_n(match_ptr, m->match_ptr, np + 1, s);
    upload_n(uv, m->uv, 4 * nm, s);
    if (m->pair_cam) upload_n(pair_cam, m->pair_cam, 2 * np, s);
    err.alloc(1, s);
    err.zero();
    BA_LAUNCH(check_pairs_kernel<<<grid_for(np + 1, 256), 256, 0, s>>>(
        np, nm, match_ptr, m->pair_cam ? pair_cam.p : nullptr, nc, cam_group_dev, ng, err));
    uint32_t e = 0;
    check(cudaMemcpyAsync(&e, err.p, 4, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaStreamSynchronize(s), "pair check");
    if (e) throw BadInput("match_ptr not increasing from 0 to n_matches, or a camera or group index out of range");
  }
};

int bit_width(uint64_t v) {
  int b = 0;
  while (v) ++b, v >>= 1;
  return b;
}

}  // namespace
}  // namespace ba

using namespace ba;

extern "C" ba_status ba_ransac_fundamental(const ba_pair_matches* m, double thresh_px,
                                           int32_t iters, void* stream, uint8_t* inlier,
                                           int32_t* n_inliers, int32_t* best_hypothesis,
                                           uint8_t* refit) {
  return guarded([&] {
    if (!(thresh_px >= 0.0) || !std::isfinite(thresh_px)) throw BadInput("thresh_px must be finite and >= 0");
    if (iters < 0 || iters > (1 << 20)) throw BadInput("iters must be in 0..2^20");
    cudaStream_t s = (cudaStream_t)stream;
    PairsIn P;
    P.load(m, m && !m->seed, (int64_t)1 << 32, nullptr, 0, s);
    const int64_t np = P.np, nm = P.nm;
    DevBuf<uint64_t> seed;
    if (m->seed) {
      upload_n(seed, m->seed, np, s);
    } else {
      seed.alloc(std::max<int64_t>(np, 1), s);
      if (np > 0) BA_LAUNCH(default_seed_kernel<<<grid_for(np, 256), 256, 0, s>>>(np, P.pair_cam, seed));
    }
    DevBuf<uint8_t> d_inl(std::max<int64_t>(nm, 1), s), d_refit(std::max<int64_t>(np, 1), s);
    DevBuf<int32_t> d_n(std::max<int64_t>(np, 1), s), d_best(std::max<int64_t>(np, 1), s);
    DevBuf<uint32_t> scratch(std::max<int64_t>(nm, 1), s);
    const int64_t chunk = iters > 0 ? std::max<int64_t>(1, kMaxChunkHyp / iters) : np;
    const int64_t cp = std::min<int64_t>(std::max<int64_t>(np, 1), chunk);
    const int64_t ch = std::max<int64_t>(cp * iters, 1);
    DevBuf<uint32_t> samples(8 * ch, s);
    DevBuf<double> F(9 * ch, s);
    DevBuf<uint8_t> valid(ch, s);
    DevBuf<int32_t> count(ch, s);
    DevBuf<float4> uv32(std::max<int64_t>(nm, 1), s);
    if (nm > 0) BA_LAUNCH(uv_f32_kernel<<<grid_for(nm, 256), 256, 0, s>>>(nm, P.uv, uv32));
    for (int64_t p0 = 0; p0 < np; p0 += cp) {
      const int64_t n = std::min(cp, np - p0);
      RansacArgs A{p0, n, P.match_ptr, P.uv, seed, iters, thresh_px * thresh_px, samples, F,
                   valid, count, scratch, d_inl, d_n, d_best, d_refit, P.err};
      if (iters > 0) {
        BA_LAUNCH(ransac_sample_kernel<<<grid_for(n, 128), 128, 0, s>>>(A));
        BA_LAUNCH(ransac_fit_kernel<<<grid_for(n * iters, kFitThreads), kFitThreads, 0, s>>>(A));
        const int64_t bpp = (iters + kHypPerCountCta - 1) / kHypPerCountCta;
        BA_LAUNCH(ransac_count_kernel<<<(unsigned)(n * bpp), kCountThreads, 0, s>>>(A, uv32));
      }
      BA_LAUNCH(ransac_select_kernel<<<(unsigned)n, kRefitThreads, 0, s>>>(A));
    }
    uint32_t e = 0;
    check(cudaMemcpyAsync(&e, P.err.p, 4, cudaMemcpyDeviceToHost, s), "d2h");
    download_n(inlier, d_inl, nm, s), download_n(n_inliers, d_n, np, s);
    download_n(best_hypothesis, d_best, np, s), download_n(refit, d_refit, np, s);
    check(cudaStreamSynchronize(s), "ransac");
    if (e) throw std::runtime_error("RANSAC sampling found no eight distinct correspondences");
  });
}

extern "C" ba_status ba_pair_fits(const ba_pair_matches* m, const double* rot, const double* center,
                                  const double* intr, const uint32_t* cam_group, int64_t n_cams,
                                  int64_t n_groups, void* stream, double* median_px) {
  return guarded([&] {
    if (n_cams < 0 || n_groups < 0) throw BadInput("negative size");
    if ((n_cams > 0 && (!rot || !center || !cam_group)) || (n_groups > 0 && !intr))
      throw BadInput("null camera array");
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf<double> d_rot, d_center, d_intr;
    DevBuf<uint32_t> d_group;
    upload_n(d_rot, rot, 9 * n_cams, s), upload_n(d_center, center, 3 * n_cams, s);
    upload_n(d_intr, intr, 5 * n_groups, s), upload_n(d_group, cam_group, n_cams, s);
    PairsIn P;
    P.load(m, true, n_cams, d_group, n_groups, s);
    const int64_t np = P.np, nm = P.nm;
    DevBuf<uint64_t> key(std::max<int64_t>(nm, 1), s), ktmp(std::max<int64_t>(nm, 1), s);
    DevBuf<uint32_t> pair(std::max<int64_t>(nm, 1), s), ptmp(std::max<int64_t>(nm, 1), s);
    DevBuf<double> med(std::max<int64_t>(np, 1), s);
    if (np > 0) {
      FitsArgs A{np, P.pair_cam, P.match_ptr, P.uv, d_rot, d_center, d_intr, d_group, key, pair};
      if (np > 0x7fffffff) throw BadInput("too many pairs");
      BA_LAUNCH(pair_err_kernel<<<(unsigned)np, 128, 0, s>>>(A));
      if (nm > 0) {
        radix_sort_u64_u32(key, pair, ktmp, ptmp, nm, 64, s);
        DevBuf<uint64_t> ck(nm, s), cv(nm, s);
        BA_LAUNCH(pair_swap_kernel<<<grid_for(nm, 256), 256, 0, s>>>(nm, key, pair, ck, cv));
        radix_sort_u64_u64(ck, cv, ktmp, key, nm, bit_width((uint64_t)np), s);
        BA_LAUNCH(pair_median_kernel<<<grid_for(np, 256), 256, 0, s>>>(np, P.match_ptr, cv, med));
      } else {
        BA_LAUNCH(pair_median_kernel<<<grid_for(np, 256), 256, 0, s>>>(np, P.match_ptr, key, med));
      }
    }
    download_n(median_px, med, np, s);
    check(cudaStreamSynchronize(s), "pair fits");
  });
}
