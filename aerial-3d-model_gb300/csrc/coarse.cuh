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
constexpr int kCoarseInvThreads = 1024;

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
  float* E;                  // per model D x D, D = 7 * groups of the model
  float* Einv;               // same layout
};

// W of every camera row of every group (thread per group).
static __global__ void coarse_basis_kernel(Prob P, StateView st, CoarseArgs A) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= A.ngroups || !A.active[A.grp_model[g]]) return;
  const int r0 = A.grp_row0[g], r1 = A.grp_row1[g];
  double c0 = 0.0, c1 = 0.0, c2 = 0.0;
  for (int r = r0; r < r1; ++r) {
    const double* C = st.center + 3 * (size_t)P.blk_id[r];
    c0 += C[0], c1 += C[1], c2 += C[2];
  }
  const double inv = 1.0 / (double)(r1 - r0);
  c0 *= inv, c1 *= inv, c2 *= inv;
  for (int r = r0; r < r1; ++r) {
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
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < kCoarseModes; ++j) out[kCoarseModes * i + j] = w[i][j];
  }
}

// E = W^T S W, rows of one group per CTA: the group's rows in order, and
// within a row every column group's blocks by one warp (no two warps add to
// the same entries while a row is processed), so the sums are in a fixed
// order.  S: FP32 BSR, full symmetric storage.
constexpr int kCoarseMatThreads = 256;

static __global__ void __launch_bounds__(kCoarseMatThreads)
    coarse_matrix_kernel(StructView SV, const float* S, CoarseArgs A) {
  __shared__ float acc[kCoarseModes * kCoarseMaxDim];
  const int g1 = blockIdx.x;
  const int m = A.grp_model[g1];
  if (!A.active[m]) return;
  const int gm0 = A.model_g0[m];
  const int D = kCoarseModes * (A.model_g0[m + 1] - gm0);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int t = threadIdx.x; t < kCoarseModes * D; t += kCoarseMatThreads) acc[t] = 0.0f;
  __syncthreads();
  for (int r = A.grp_row0[g1]; r < A.grp_row1[g1]; ++r) {
    const uint32_t b0 = SV.row_ptr[r], b1 = SV.row_ptr[r + 1];
    const float* Wr = A.W + (size_t)r * kCoarseW;
    // Segments of consecutive blocks with the same column group (columns are
    // sorted and groups are runs of consecutive rows).  Warp w takes the
    // segments w, w + 8, ...: found by a scan of the row by every warp.
    int sidx = 0;
    uint32_t k = b0;
    while (k < b1) {
      const int gc = A.row_grp[SV.col_idx[k]];
      uint32_t e = k + 1;
      while (e < b1 && A.row_grp[SV.col_idx[e]] == gc) ++e;
      if (gc >= 0 && (sidx % (kCoarseMatThreads / 32)) == warp) {
        // T = sum_k S_k W_col(k) (6 x 7): lane j < 7 owns column j.
        float t[6] = {0, 0, 0, 0, 0, 0};
        if (lane < kCoarseModes) {
          for (uint32_t q = k; q < e; ++q) {
            const float* blk = S + (size_t)q * 36;
            const float* Wc = A.W + (size_t)SV.col_idx[q] * kCoarseW;
            float wc[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) wc[i] = Wc[kCoarseModes * i + lane];
#pragma unroll
            for (int i = 0; i < 6; ++i) {
              float s = t[i];
#pragma unroll
              for (int j = 0; j < 6; ++j) s += blk[6 * i + j] * wc[j];
              t[i] = s;
            }
          }
          // P[:, lane] = W_r^T T[:, lane]
          const int col = kCoarseModes * (gc - gm0) + lane;
#pragma unroll
          for (int a = 0; a < kCoarseModes; ++a) {
            float s = 0.0f;
#pragma unroll
            for (int i = 0; i < 6; ++i) s += Wr[kCoarseModes * i + a] * t[i];
            acc[a * D + col] += s;
          }
        }
      }
      if (gc >= 0) ++sidx;
      k = e;
    }
    __syncthreads();
  }
  float* Em = A.E + A.model_eoff[m];
  const int row0 = kCoarseModes * (g1 - gm0);
  for (int t = threadIdx.x; t < kCoarseModes * D; t += kCoarseMatThreads)
    Em[(size_t)(row0 + t / D) * D + (t % D)] = acc[t];
}

// E^-1 per model (CTA per model): Jacobi scaling, then in-place Gauss-Jordan
// without pivoting (E is symmetric positive definite).  The 32 x 32 threads
// each hold a T x T tile of the matrix in registers (T = ceil(D / 32) <= 7);
// per pivot the owners publish the pivot row and column in shared memory and
// every thread updates its tile (T <= 6 keeps the tile in registers at
// 1024 threads).  A coarse unknown whose scaled pivot falls
// below 1e-6 is dropped (its row and column of the inverse are zero).  The
// result is unscaled and symmetrised.
constexpr int kInvTile = (kCoarseMaxDim + 31) / 32;  // 6

static __global__ void __launch_bounds__(kCoarseInvThreads, 1) coarse_invert_kernel(CoarseArgs A) {
  __shared__ float rowk[kCoarseMaxDim], colk[kCoarseMaxDim], dsc[kCoarseMaxDim];
  const int m = blockIdx.x;
  if (!A.active[m]) return;
  const int D = kCoarseModes * (A.model_g0[m + 1] - A.model_g0[m]);
  if (D == 0) return;
  const int T = (D + 31) / 32;
  const int i0 = (threadIdx.x >> 5) * T, j0 = (threadIdx.x & 31) * T;
  float* Em = A.E + A.model_eoff[m];
  for (int i = threadIdx.x; i < D; i += blockDim.x) {
    const float d = Em[(size_t)i * D + i];
    dsc[i] = d > 0.0f ? rsqrtf(d) : 0.0f;
  }
  __syncthreads();
  float a[kInvTile][kInvTile];
#pragma unroll
  for (int r = 0; r < kInvTile; ++r)
#pragma unroll
    for (int c = 0; c < kInvTile; ++c) {
      const int i = i0 + r, j = j0 + c;
      float v = 0.0f;
      if (r < T && c < T && i < D && j < D) {
        if (dsc[i] == 0.0f || dsc[j] == 0.0f)
          v = i == j ? 1.0f : 0.0f;
        else  // symmetrise the assembled E (FP32 sums in two orders) while scaling
          v = 0.5f * (Em[(size_t)i * D + j] + Em[(size_t)j * D + i]) * dsc[i] * dsc[j];
      }
      a[r][c] = v;
    }
  for (int k = 0; k < D; ++k) {
    __syncthreads();  // the previous pivot's row and column have been used
    const int rk = k - i0, ck = k - j0;
    // Only the owners of row k and column k publish them (rk, ck < T).
#pragma unroll
    for (int r = 0; r < kInvTile; ++r)
      if (r == rk && r < T)
#pragma unroll
        for (int c = 0; c < kInvTile; ++c)
          if (c < T && j0 + c < D) rowk[j0 + c] = a[r][c];
#pragma unroll
    for (int c = 0; c < kInvTile; ++c)
      if (c == ck && c < T)
#pragma unroll
        for (int r = 0; r < kInvTile; ++r)
          if (r < T && i0 + r < D) colk[i0 + r] = a[r][c];
    __syncthreads();
    const float piv = rowk[k];
    const bool drop = !(piv > 1e-6f);
    const float rp = drop ? 0.0f : 1.0f / piv;
    float rj[kInvTile];
#pragma unroll
    for (int c = 0; c < kInvTile; ++c) rj[c] = j0 + c < D ? rowk[j0 + c] * rp : 0.0f;
#pragma unroll
    for (int r = 0; r < kInvTile; ++r) {
      const int i = i0 + r;
      const float ci = i < D ? colk[i] : 0.0f;
#pragma unroll
      for (int c = 0; c < kInvTile; ++c) {
        const int j = j0 + c;
        float v = a[r][c];
        if (i == k)
          v = drop ? 0.0f : (j == k ? rp : rj[c]);
        else if (j == k)
          v = drop ? 0.0f : -ci * rp;
        else if (!drop)
          v -= ci * rj[c];
        a[r][c] = v;
      }
    }
  }
  // Unscale into E (no longer needed), then symmetrise into E^-1.
#pragma unroll
  for (int r = 0; r < kInvTile; ++r)
#pragma unroll
    for (int c = 0; c < kInvTile; ++c) {
      const int i = i0 + r, j = j0 + c;
      if (r < T && c < T && i < D && j < D) Em[(size_t)i * D + j] = a[r][c] * dsc[i] * dsc[j];
    }
  __syncthreads();
  float* Im = A.Einv + A.model_eoff[m];
  for (int t = threadIdx.x; t < D * D; t += blockDim.x) {
    const int i = t / D, j = t - (t / D) * D;
    Im[t] = 0.5f * (Em[t] + Em[(size_t)j * D + i]);
  }
}

inline size_t coarse_invert_smem(int) { return 0; }

}  // namespace ba
