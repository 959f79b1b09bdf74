// Two-level preconditioner of the mixed form's reduced camera system: block
// Jacobi plus a coarse correction over groups of cameras,
//   M^-1 r = B^-1 r + W E^-1 W^T r,   E = W^T S W,
// where each group of consecutive cameras contributes the seven similarity
// motions of that group (translation 3, rotation about the group centroid 3,
// scale about it 1) as columns of W.  These are the motions the reduced
// system hardly resists (the gauge of the whole block, held only by the GPS
// priors, and its low-frequency bending across groups), which is where
// block-Jacobi PCG spends its iterations.  The FP64 form keeps the
// reference's block-Jacobi PCG (ba.rs:155-196); this is the mixed form's own
// solver.
//
// In camera block coordinates (rotation as the left perturbation of the
// world->camera R, then the centre), a world rotation phi about the centroid
// C0 moves camera c by omega = -R_c phi, dC = phi x (C_c - C0); a translation
// t by dC = t; a scale s by dC = s (C_c - C0).  Lens rows take no part.
//
// E is assembled per group of rows in a fixed order, Jacobi-scaled (its
// condition then is about 1e4 on the surveys measured, from about 1e8) and
// inverted in FP32 by Gauss-Jordan in one CTA's shared memory; the inverse
// is symmetrised and applied in FP32 inside the cluster PCG kernel.
#pragma once

#include "ba_common.cuh"
#include "lm_kernels.cuh"

namespace ba {

constexpr int kCoarseModes = 7;
constexpr int kCoarseMaxGroups = 27;                    // per model
constexpr int kCoarseMaxDim = kCoarseModes * kCoarseMaxGroups;  // 189
constexpr int kCoarseW = 6 * kCoarseModes;              // W values per row

struct CoarseArgs {
  int32_t ngroups;           // all models
  const int32_t* grp_row0;   // [ngroups] first block row
  const int32_t* grp_row1;   // [ngroups] end block row
  const int32_t* grp_model;  // [ngroups]
  const int32_t* model_g0;   // [nm + 1] first group of each model
  const int64_t* model_eoff; // [nm] offset of the model's E (D x D floats)
  const int32_t* row_grp;    // [nb] group of each block row (-1: lens row)
  const int32_t* active;
  float* W;                  // [nb * 42] row-major 6 x 7
  double* W64;               // the same values in FP64 (for the coarse matrix)
  float* E;                  // per model D x D, D = 7 * groups of the model
  float* Einv;               // same layout
};

// W of every camera row of every group: a warp per group, the centroid as a
// warp sum in a fixed order, then a lane per row.
static __global__ void coarse_basis_kernel(Prob P, StateView st, CoarseArgs A) {
  const int g = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (g >= A.ngroups || !A.active[A.grp_model[g]]) return;
  const int r0 = A.grp_row0[g], r1 = A.grp_row1[g];
  double c0 = 0.0, c1 = 0.0, c2 = 0.0;
  for (int r = r0 + lane; r < r1; r += 32) {
    const double* C = st.center + 3 * (size_t)P.blk_id[r];
    c0 += C[0], c1 += C[1], c2 += C[2];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    c0 += __shfl_xor_sync(kFull, c0, o);
    c1 += __shfl_xor_sync(kFull, c1, o);
    c2 += __shfl_xor_sync(kFull, c2, o);
  }
  const double inv = 1.0 / (double)(r1 - r0);
  c0 *= inv, c1 *= inv, c2 *= inv;
  for (int r = r0 + lane; r < r1; r += 32) {
    const uint32_t cam = P.blk_id[r];
    const double* R = st.rot + 9 * (size_t)cam;
    const double* C = st.center + 3 * (size_t)cam;
    const float d0 = (float)(C[0] - c0), d1 = (float)(C[1] - c1), d2 = (float)(C[2] - c2);
    float w[6][kCoarseModes] = {};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      w[3 + k][k] = 1.0f;  // translation
#pragma unroll
      for (int i = 0; i < 3; ++i) w[i][3 + k] = -(float)R[3 * i + k];  // rotation: -R e_k
    }
    // rotation: e_k x d
    w[4][3] = -d2, w[5][3] = d1;
    w[3][4] = d2, w[5][4] = -d0;
    w[3][5] = -d1, w[4][5] = d0;
    w[3][6] = d0, w[4][6] = d1, w[5][6] = d2;  // scale
    float* out = A.W + (size_t)r * kCoarseW;
    double* out64 = A.W64 + (size_t)r * kCoarseW;
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < kCoarseModes; ++j) {
        out[kCoarseModes * i + j] = w[i][j];
        out64[kCoarseModes * i + j] = (double)w[i][j];
      }
  }
}

// E = W^T S W in two passes, both in a fixed order.  (1) A warp per (camera
// row r, group g of r's model): P[r][g] = W_r^T (sum over r's blocks in g's
// columns of S_rc W_c), 7 x 7, zero when r has no block there.  (2) A thread
// per entry of E: the sum of P over the rows of the entry's row group, in row
// order.  S: the FP64 values of the reduced matrix before its rounding to
// FP32 (full symmetric BSR); the sums are FP64 and E is rounded to FP32 once.
// The group motions nearly annihilate S (its weakest directions are the
// similarity motions held only by the GPS priors), so W^T S W is a small
// difference of large terms: from FP32 S it would be rounding noise.
constexpr int kCoarseMatThreads = 256;

static __global__ void __launch_bounds__(kCoarseMatThreads)
    coarse_rowgroup_kernel(StructView SV, const double* S, CoarseArgs A, int64_t npairs,
                           const int32_t* pair_row, const int32_t* pair_grp, double* Pbuf) {
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= npairs) return;
  const int32_t r = pair_row[wid], g = pair_grp[wid];
  double* P = Pbuf + (size_t)wid * 49;
  if (!A.active[A.grp_model[g]]) return;
  // Blocks of row r whose columns lie in rows [c0, c1) of group g.
  const int32_t c0 = A.grp_row0[g], c1 = A.grp_row1[g];
  uint32_t lo = SV.row_ptr[r], hi = SV.row_ptr[r + 1];
  {
    uint32_t a0 = lo, a1 = hi;
    while (a0 < a1) {
      const uint32_t mid = (a0 + a1) >> 1;
      if ((int32_t)SV.col_idx[mid] < c0) a0 = mid + 1; else a1 = mid;
    }
    lo = a0;
    a1 = hi;
    while (a0 < a1) {
      const uint32_t mid = (a0 + a1) >> 1;
      if ((int32_t)SV.col_idx[mid] < c1) a0 = mid + 1; else a1 = mid;
    }
    hi = a0;
  }
  // T = sum_k S_k W_col(k) (6 x 7): lane = 7 q + j handles column j of the
  // blocks lo + q, lo + q + 4, ... (q < 4); the four partials are summed in
  // order q = 0..3.
  const int q = lane / 7, j = lane - 7 * (lane / 7);
  double t[6] = {0, 0, 0, 0, 0, 0};
  if (q < 4)
    for (uint32_t k = lo + q; k < hi; k += 4) {
      const double* blk = S + (size_t)k * 36;
      const double* Wc = A.W64 + (size_t)SV.col_idx[k] * kCoarseW;
      double wc[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) wc[i] = Wc[kCoarseModes * i + j];
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        double v = t[i];
#pragma unroll
        for (int c = 0; c < 6; ++c) v += blk[6 * i + c] * wc[c];
        t[i] = v;
      }
    }
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const double v1 = __shfl_down_sync(kFull, t[i], 7), v2 = __shfl_down_sync(kFull, t[i], 14),
                 v3 = __shfl_down_sync(kFull, t[i], 21);
    t[i] = ((t[i] + v1) + v2) + v3;  // lanes 0..6: column j summed over q
  }
  // P = W_r^T T: the 49 entries over the 32 lanes in two rounds (an FP64
  // warp instruction costs the same for one active lane as for 32); lane b
  // holds column b of T.
  const double* Wr = A.W64 + (size_t)r * kCoarseW;
#pragma unroll
  for (int rd = 0; rd < 2; ++rd) {
    const int o = lane + 32 * rd;
    const int oo = o < kCoarseModes * kCoarseModes ? o : 0;
    const int a = oo / kCoarseModes, b = oo - kCoarseModes * (oo / kCoarseModes);
    double v = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) v += Wr[kCoarseModes * i + a] * __shfl_sync(kFull, t[i], b);
    if (o < kCoarseModes * kCoarseModes) P[o] = v;
  }
}

// E entry (7 g1 + a, 7 g2 + b) of model m = sum over rows r of group g1 of
// P[r][g2][a][b]; pairs are listed row-major by (row, group of the model).
static __global__ void coarse_sum_kernel(CoarseArgs A, const int64_t* row_pair0,
                                         const double* Pbuf) {
  const int g1 = blockIdx.x;
  const int m = A.grp_model[g1];
  if (!A.active[m]) return;
  const int gm0 = A.model_g0[m];
  const int G = A.model_g0[m + 1] - gm0;
  const int D = kCoarseModes * G;
  float* Em = A.E + A.model_eoff[m];
  // blockIdx.y splits the group's 7 x D entries over gridDim.y CTAs.
  for (int t = blockIdx.y * blockDim.x + threadIdx.x; t < kCoarseModes * D;
       t += gridDim.y * blockDim.x) {
    const int a = t / D, col = t - (t / D) * D;
    const int g2 = col / kCoarseModes, bcol = col - kCoarseModes * g2;
    double v = 0.0;
    for (int32_t r = A.grp_row0[g1]; r < A.grp_row1[g1]; ++r)
      v += Pbuf[(size_t)(row_pair0[r] + g2) * 49 + a * kCoarseModes + bcol];
    Em[(size_t)(kCoarseModes * (g1 - gm0) + a) * D + col] = (float)v;
  }
}

// E^-1 per model (CTA per model): Jacobi scaling, then in-place block
// Gauss-Jordan without pivoting (E is symmetric positive definite), four
// pivots per step.  The 16 x 32 threads each hold a TR x TC tile of the
// matrix in registers (TR = ceil(D / 16) <= 12, TC = ceil(D / 32) <= 6; 512
// threads leave 128 registers each); per step the owners publish
// the four pivot rows and columns in shared memory, every thread inverts the
// 4 x 4 pivot block (a scalar pivot below 1e-6 of the scaled unit diagonal is
// raised to 1e-6) and updates its tile.  The result is unscaled and
// symmetrised.
constexpr int kInvThreads = 512;
constexpr int kInvTR = (kCoarseMaxDim + 15) / 16;  // 12
constexpr int kInvTC = (kCoarseMaxDim + 31) / 32;  // 6
constexpr int kInvB = 4;                           // pivots per step
constexpr int kInvDimPad = ((kCoarseMaxDim + kInvB - 1) / kInvB) * kInvB;

static __global__ void __launch_bounds__(kInvThreads, 1) coarse_invert_kernel(CoarseArgs A) {
  __shared__ float rowb[kInvB][kInvDimPad], colb[kInvDimPad][kInvB], dsc[kInvDimPad];
  __shared__ float rnS[kInvB][kInvDimPad], cnS[kInvDimPad][kInvB];
  const int m = blockIdx.x;
  if (!A.active[m]) return;
  const int D = kCoarseModes * (A.model_g0[m + 1] - A.model_g0[m]);
  if (D == 0) return;
  const int TR = (D + 15) / 16, TC = (D + 31) / 32;
  const int i0 = (threadIdx.x >> 5) * TR, j0 = (threadIdx.x & 31) * TC;
  float* Em = A.E + A.model_eoff[m];
  for (int i = threadIdx.x; i < kInvDimPad; i += blockDim.x) {
    const float d = i < D ? Em[(size_t)i * D + i] : 0.0f;
    dsc[i] = d > 0.0f ? rsqrtf(d) : 0.0f;
  }
  __syncthreads();
  // Padding rows/columns up to a multiple of four are identity.
  const int Dp = ((D + kInvB - 1) / kInvB) * kInvB;
  float a[kInvTR][kInvTC];
#pragma unroll
  for (int r = 0; r < kInvTR; ++r)
#pragma unroll
    for (int c = 0; c < kInvTC; ++c) {
      const int i = i0 + r, j = j0 + c;
      float v = 0.0f;
      if (r < TR && c < TC && i < Dp && j < Dp) {
        if (i >= D || j >= D || dsc[i] == 0.0f || dsc[j] == 0.0f)
          v = i == j ? 1.0f : 0.0f;
        else  // symmetrise the assembled E (FP32 sums in two orders) while scaling
          v = 0.5f * (Em[(size_t)i * D + j] + Em[(size_t)j * D + i]) * dsc[i] * dsc[j];
      }
      a[r][c] = v;
    }
  for (int k0 = 0; k0 < Dp; k0 += kInvB) {
    __syncthreads();  // the previous step's rows and columns have been used
#pragma unroll
    for (int r = 0; r < kInvTR; ++r) {
      const int i = i0 + r, br = i - k0;
      if (r < TR && br >= 0 && br < kInvB)
#pragma unroll
        for (int c = 0; c < kInvTC; ++c)
          if (c < TC && j0 + c < Dp) rowb[br][j0 + c] = a[r][c];
    }
#pragma unroll
    for (int c = 0; c < kInvTC; ++c) {
      const int j = j0 + c, bc = j - k0;
      if (c < TC && bc >= 0 && bc < kInvB)
#pragma unroll
        for (int r = 0; r < kInvTR; ++r)
          if (r < TR && i0 + r < Dp) colb[i0 + r][bc] = a[r][c];
    }
    __syncthreads();
    // Inverse of the 4 x 4 pivot block (scalar Gauss-Jordan, registers),
    // then shared: rn = Pinv * (pivot rows), with Pinv itself in the pivot
    // columns, and cn = -(pivot columns) * Pinv.  A thread per column j < Dp
    // (Dp <= 192 < 512 threads).
    if ((int)threadIdx.x < Dp) {
      float pb[kInvB][kInvB];
#pragma unroll
      for (int x = 0; x < kInvB; ++x)
#pragma unroll
        for (int y = 0; y < kInvB; ++y) pb[x][y] = rowb[x][k0 + y];
#pragma unroll
      for (int kk = 0; kk < kInvB; ++kk) {
        const float rp = 1.0f / fmaxf(pb[kk][kk], 1e-6f);
        float rk[kInvB], ck[kInvB];
#pragma unroll
        for (int y = 0; y < kInvB; ++y) rk[y] = y == kk ? rp : pb[kk][y] * rp;
#pragma unroll
        for (int x = 0; x < kInvB; ++x) ck[x] = pb[x][kk];
#pragma unroll
        for (int x = 0; x < kInvB; ++x)
#pragma unroll
          for (int y = 0; y < kInvB; ++y)
            pb[x][y] = x == kk ? rk[y] : (y == kk ? -ck[x] * rp : pb[x][y] - ck[x] * rk[y]);
      }
      for (int j = threadIdx.x; j < Dp; j += blockDim.x) {
        const int bc = j - k0;
        const bool pc = bc >= 0 && bc < kInvB;
#pragma unroll
        for (int x = 0; x < kInvB; ++x) {
          float v = 0.0f, w = 0.0f;
#pragma unroll
          for (int y = 0; y < kInvB; ++y) {
            v += pb[x][y] * rowb[y][j];
            w += colb[j][y] * pb[y][x];
          }
          float pv = 0.0f;
#pragma unroll
          for (int y = 0; y < kInvB; ++y)
            if (y == bc) pv = pb[x][y];
          rnS[x][j] = pc ? pv : v;
          cnS[j][x] = -w;
        }
      }
    }
    __syncthreads();
    float rn[kInvB][kInvTC];
#pragma unroll
    for (int x = 0; x < kInvB; ++x)
#pragma unroll
      for (int c = 0; c < kInvTC; ++c) rn[x][c] = (c < TC && j0 + c < Dp) ? rnS[x][j0 + c] : 0.0f;
#pragma unroll
    for (int r = 0; r < kInvTR; ++r) {
      const int i = i0 + r, br = i - k0;
      if (r >= TR || i >= Dp) continue;
      if (br >= 0 && br < kInvB) {  // a pivot row: Pinv * (pivot rows)
#pragma unroll
        for (int c = 0; c < kInvTC; ++c)
          if (c < TC && j0 + c < Dp) a[r][c] = rnS[br][j0 + c];
        continue;
      }
      float ci[kInvB];
#pragma unroll
      for (int y = 0; y < kInvB; ++y) ci[y] = colb[i][y];
#pragma unroll
      for (int c = 0; c < kInvTC; ++c) {
        const int bc = j0 + c - k0;
        if (bc >= 0 && bc < kInvB) {  // a pivot column: -(pivot columns) * Pinv
          a[r][c] = cnS[i][bc];
        } else {
          float v = a[r][c];
#pragma unroll
          for (int y = 0; y < kInvB; ++y) v -= ci[y] * rn[y][c];
          a[r][c] = v;
        }
      }
    }
  }
  // Unscale into E (no longer needed), then symmetrise into E^-1.
#pragma unroll
  for (int r = 0; r < kInvTR; ++r)
#pragma unroll
    for (int c = 0; c < kInvTC; ++c) {
      const int i = i0 + r, j = j0 + c;
      if (r < TR && c < TC && i < D && j < D) Em[(size_t)i * D + j] = a[r][c] * dsc[i] * dsc[j];
    }
  __syncthreads();
  float* Im = A.Einv + A.model_eoff[m];
#pragma unroll 4
  for (int t = threadIdx.x; t < D * D; t += blockDim.x) {
    const int i = t / D, j = t - (t / D) * D;
    Im[t] = 0.5f * (Em[t] + Em[(size_t)j * D + i]);
  }
}


}  // namespace ba
