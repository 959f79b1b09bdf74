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

#include <cooperative_groups.h>

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

// E^-1 per model, one thread-block cluster of kInvCl CTAs per model: Jacobi
// scaling, then in-place block Gauss-Jordan without pivoting (E is symmetric
// positive definite), four pivots per step.  The matrix, padded with identity
// to Dq = a multiple of 32 (<= 192), is split into kInvCl column slabs of
// W = Dq / kInvCl columns, one per CTA, held in registers (a thread holds 3
// rows x 3 columns).  Per step the CTA owning the four pivot columns
// publishes them and the inverse of the 4 x 4 pivot block (a scalar pivot
// below 1e-6 of the scaled unit diagonal is raised to 1e-6) in double-
// buffered shared memory; after one cluster barrier every CTA copies them
// through distributed shared memory and updates its slab:
//   pivot rows        <- Pinv * (pivot rows)   (Pinv itself in the pivot columns)
//   pivot columns     <- -(pivot columns) * Pinv
//   everything else  -= (pivot columns) * Pinv * (pivot rows).
// The result is unscaled and symmetrised.
constexpr int kInvCl = 8;
constexpr int kInvClThreads = 512;
constexpr int kInvMaxPad = 192;  // kCoarseMaxDim rounded up to a multiple of 32
static_assert(kInvMaxPad >= kCoarseMaxDim && kInvMaxPad % 32 == 0, "slab layout");
static_assert(kInvMaxPad / kInvCl <= 24 && kInvClThreads == 64 * 8, "3 x 3 elements a thread");

static __global__ void __cluster_dims__(kInvCl, 1, 1) __launch_bounds__(kInvClThreads, 1)
    coarse_invert_kernel(CoarseArgs A) {
  namespace cgi = cooperative_groups;
  cgi::cluster_group cl = cgi::this_cluster();
  __shared__ float dsc[kInvMaxPad];
  __shared__ __align__(16) float colP[2][kInvMaxPad][4];  // published pivot columns
  __shared__ float pinvP[2][4][4];                        // published pivot-block inverse
  __shared__ __align__(16) float colL[kInvMaxPad][4];     // this step's copies
  __shared__ float pinvL[4][4];
  __shared__ float rowL[4][kInvMaxPad / kInvCl];          // this slab's part of the pivot rows
  const int q = (int)cl.block_rank();
  const int m = blockIdx.x / kInvCl;  // uniform over the cluster
  if (!A.active[m]) return;
  const int D = kCoarseModes * (A.model_g0[m + 1] - A.model_g0[m]);
  if (D == 0) return;
  const int Dq = ((D + 31) / 32) * 32, W = Dq / kInvCl;
  const int t = threadIdx.x, r0 = (t >> 3) * 3, c0 = (t & 7) * 3;
  float* Em = A.E + A.model_eoff[m];
  for (int i = t; i < kInvMaxPad; i += kInvClThreads) {
    const float d = i < D ? Em[(size_t)i * D + i] : 0.0f;
    dsc[i] = d > 0.0f ? rsqrtf(d) : 0.0f;
  }
  __syncthreads();
  float a[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int i = r0 + r, jl = c0 + c, j = q * W + jl;
      float v = 0.0f;
      if (i < Dq && jl < W) {
        if (i >= D || j >= D || dsc[i] == 0.0f || dsc[j] == 0.0f)
          v = i == j ? 1.0f : 0.0f;
        else  // symmetrise the assembled E while scaling
          v = 0.5f * (Em[(size_t)i * D + j] + Em[(size_t)j * D + i]) * dsc[i] * dsc[j];
      }
      a[r][c] = v;
    }
  for (int k0 = 0, step = 0; k0 < Dq; k0 += 4, ++step) {
    const int buf = step & 1;
    const int owner = k0 / W, kl = k0 - owner * W;  // W is a multiple of 4
    __syncthreads();  // the previous step's reads of rowL, colL and pinvL are done
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const int y = r0 + r - k0;
      if (y >= 0 && y < 4)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          if (c0 + c < W) rowL[y][c0 + c] = a[r][c];
    }
    if (q == owner) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int x = c0 + c - kl;
        if (x >= 0 && x < 4)
#pragma unroll
          for (int r = 0; r < 3; ++r)
            if (r0 + r < Dq) colP[buf][r0 + r][x] = a[r][c];
      }
      __syncthreads();
      if (t == 0) {  // inverse of the 4 x 4 pivot block (scalar Gauss-Jordan)
        float pb[4][4];
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
          for (int y = 0; y < 4; ++y) pb[x][y] = colP[buf][k0 + x][y];
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const float rp = 1.0f / fmaxf(pb[kk][kk], 1e-6f);
          float rk[4], ck[4];
#pragma unroll
          for (int y = 0; y < 4; ++y) rk[y] = y == kk ? rp : pb[kk][y] * rp;
#pragma unroll
          for (int x = 0; x < 4; ++x) ck[x] = pb[x][kk];
#pragma unroll
          for (int x = 0; x < 4; ++x)
#pragma unroll
            for (int y = 0; y < 4; ++y)
              pb[x][y] = x == kk ? rk[y] : (y == kk ? -ck[x] * rp : pb[x][y] - ck[x] * rk[y]);
        }
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
          for (int y = 0; y < 4; ++y) pinvP[buf][x][y] = pb[x][y];
      }
    }
    cl.sync();  // the owner's pivot columns and Pinv, and every slab's pivot rows
    {
      const float* srcC = cl.map_shared_rank(&colP[buf][0][0], (unsigned)owner);
      const float* srcP = cl.map_shared_rank(&pinvP[buf][0][0], (unsigned)owner);
      for (int u = t; u < Dq * 4; u += kInvClThreads) (&colL[0][0])[u] = srcC[u];
      if (t < 16) (&pinvL[0][0])[t] = srcP[t];
    }
    __syncthreads();
    float rn[4][3];  // Pinv * (pivot rows) for this thread's columns
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int jl = c0 + c < W ? c0 + c : 0;
        float v = 0.0f;
#pragma unroll
        for (int y = 0; y < 4; ++y) v += pinvL[x][y] * rowL[y][jl];
        rn[x][c] = v;
      }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const int i = r0 + r, y = i - k0;
      const float4 cv = *reinterpret_cast<const float4*>(&colL[i < Dq ? i : 0][0]);
      const bool prow = y >= 0 && y < 4;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int x = c0 + c - kl;
        const bool pcol = q == owner && x >= 0 && x < 4;
        if (prow) {
          a[r][c] = pcol ? pinvL[y][x] : rn[y][c];
        } else if (pcol) {
          float w = 0.0f;
          w += cv.x * pinvL[0][x];
          w += cv.y * pinvL[1][x];
          w += cv.z * pinvL[2][x];
          w += cv.w * pinvL[3][x];
          a[r][c] = -w;
        } else {
          float v = a[r][c];
          v -= cv.x * rn[0][c];
          v -= cv.y * rn[1][c];
          v -= cv.z * rn[2][c];
          v -= cv.w * rn[3][c];
          a[r][c] = v;
        }
      }
    }
  }
  // Unscale into E (no longer needed), then symmetrise into E^-1 once every
  // slab is written.
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int i = r0 + r, jl = c0 + c, j = q * W + jl;
      if (i < D && jl < W && j < D) Em[(size_t)i * D + j] = a[r][c] * dsc[i] * dsc[j];
    }
  __threadfence();
  cl.sync();
  float* Im = A.Einv + A.model_eoff[m];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int i = r0 + r, jl = c0 + c, j = q * W + jl;
      if (i < D && jl < W && j < D)
        Im[(size_t)i * D + j] = 0.5f * (Em[(size_t)i * D + j] + Em[(size_t)j * D + i]);
    }
}


}  // namespace ba
