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
// inverted in FP32 by Gauss-Jordan in the registers of one CTA per model; the
// inverse is symmetrised and applied in FP32 inside the cluster PCG kernel.
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
  if (lo == hi) {
    // No block of row r in group g (most pairs: a camera's blocks lie in a
    // few groups): P is zero, +0.0 as the products below would give it,
    // without their FP64 instructions.
    for (int o = lane; o < kCoarseModes * kCoarseModes; o += 32) P[o] = 0.0;
    return;
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

// E^-1 per model, one CTA of kInvThreads threads per model: Jacobi scaling,
// then in-place block Gauss-Jordan without pivoting (E is symmetric positive
// definite), four pivots per step.  E is staged in shared memory and there
// symmetrised, scaled and padded with identity to Dq = a multiple of 32
// (<= 192); the matrix then lives in registers: thread t of 384 holds the
// 8 x 12 tile at rows 8 (t / 16), columns 12 (t % 16) (three warps per SM
// sub-partition to hide the FMA and shared-memory latencies), rows 2 p and
// 2 p + 1 of a column in one 64-bit register pair, so that the update runs
// on packed FP32 FMAs (fma.rn.f32x2: two round-to-nearest FP32 FMAs, the
// results of two fmaf).  Per step the threads holding the four pivot
// columns, then the four pivot rows, copy them to shared memory and zero them
// in the tile; a thread per column then inverts the 4 x 4 pivot block (a
// scalar pivot below 1e-6 of the scaled unit diagonal is raised to 1e-6) and
// forms that column of the new pivot rows rn; every thread then updates its
// tile, a <- a + cn . rn, with cn = -(pivot columns) but e_y on pivot row y:
//   pivot rows        <- Pinv * (pivot rows)   (Pinv itself in the pivot columns)
//   pivot columns     <- -(pivot columns) * Pinv
//   everything else  -= (pivot columns) * Pinv * (pivot rows).
// The shared pivot rows and columns alternate between two buffers, so a step
// takes two barriers.  The result is unscaled and symmetrised.
constexpr int kInvThreads = 384;
constexpr int kInvTileR = 8;   // rows of a thread's tile
constexpr int kInvTileC = 12;  // columns of a thread's tile
constexpr int kInvPairs = kInvTileR / 2;
constexpr int kInvMaxPad = 192;  // kCoarseMaxDim rounded up to a multiple of 32
static_assert(kInvMaxPad >= kCoarseMaxDim && kInvMaxPad % 32 == 0, "padding");
static_assert((kInvThreads / 16) * kInvTileR == kInvMaxPad && 16 * kInvTileC == kInvMaxPad,
              "8 x 12 tiles cover the padded matrix");
static_assert(kInvTileR % 4 == 0 && kInvTileC % 4 == 0, "pivot groups of four lie inside one tile");
static_assert(kInvThreads >= kInvMaxPad, "a thread per column of the pivot rows");
// E staged whole in dynamic shared memory; the even pitch keeps a row pair of
// one column 8-byte aligned.
constexpr int kInvPitch = kInvMaxPad + 2;
constexpr size_t kInvSmemBytes = (size_t)kInvMaxPad * kInvPitch * sizeof(float);
// Column j of the new pivot rows sits at j + j / 12: the 16 threads of a tile
// row read columns 12 k + c, which then fall in 16 different bank quads
// (13 k + c mod 8 differs for any 8 consecutive k).
__device__ __forceinline__ int inv_rn_slot(int j) { return j + j / kInvTileC; }
constexpr int kInvRnSlots = kInvMaxPad + kInvMaxPad / kInvTileC;

__device__ __forceinline__ uint64_t f2_pack(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_unpack(uint64_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
// acc <- x * y + acc, elementwise on two FP32 lanes, each rounded once.
__device__ __forceinline__ void f2_fma(uint64_t& acc, uint64_t x, uint64_t y) {
  asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc) : "l"(x), "l"(y));
}

// Inverse of the 4 x 4 pivot block pb (scalar Gauss-Jordan, in place).
__device__ __forceinline__ void inv4_pivot(float (&pb)[4][4]) {
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
}

static __global__ void __launch_bounds__(kInvThreads, 1) coarse_invert_kernel(CoarseArgs A) {
  __shared__ float dsc[kInvMaxPad];
  __shared__ float4 colS[2][kInvMaxPad];                  // pivot columns, a row each
  __shared__ __align__(16) float rowS[2][4][kInvMaxPad];  // pivot rows
  __shared__ ulonglong2 rnA[2][kInvRnSlots];  // new pivot rows per column: (x, x), (y, y)
  __shared__ ulonglong2 rnB[2][kInvRnSlots];  //                            (z, z), (w, w)
  __shared__ __align__(16) float cnS[2][4][kInvMaxPad];   // cn, by component
  extern __shared__ __align__(16) float smE[];            // [kInvMaxPad][kInvPitch]
  const int m = blockIdx.x;
  if (!A.active[m]) return;
  const int D = kCoarseModes * (A.model_g0[m + 1] - A.model_g0[m]);
  if (D == 0) return;
  const int Dq = ((D + 31) / 32) * 32;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const int r0 = (t >> 4) * kInvTileR, c0 = (t & 15) * kInvTileC;
  const float* Em = A.E + A.model_eoff[m];
  // Asynchronous 4-byte copies: every load in flight at once, none through
  // registers (E was just written and is read once).
  for (int i = wid; i < D; i += kInvThreads / 32)
    for (int j = lane; j < D; j += 32) {
      const uint32_t dst = (uint32_t)__cvta_generic_to_shared(smE + i * kInvPitch + j);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst),
                   "l"(Em + (size_t)i * D + j)
                   : "memory");
    }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
  for (int i = t; i < kInvMaxPad; i += kInvThreads) {
    const float d = i < D ? smE[i * kInvPitch + i] : 0.0f;
    dsc[i] = d > 0.0f ? rsqrtf(d) : 0.0f;
  }
  __syncthreads();
  // Symmetrise, scale and pad in place, a thread per pair {(i, j), (j, i)}.
  for (int i = wid; i < kInvMaxPad; i += kInvThreads / 32)
    for (int j = lane; j <= i; j += 32) {
      float vij = (i == j && i < Dq) ? 1.0f : 0.0f, vji = vij;
      if (i < D && dsc[i] != 0.0f && dsc[j] != 0.0f) {
        const float h = 0.5f * (smE[i * kInvPitch + j] + smE[j * kInvPitch + i]);
        vij = h * dsc[i] * dsc[j];
        vji = h * dsc[j] * dsc[i];
      }
      smE[i * kInvPitch + j] = vij;
      smE[j * kInvPitch + i] = vji;
    }
  __syncthreads();
  // The tile, read down the columns of the symmetric matrix: rows (2 p, 2 p + 1)
  // of column c are entries (2 p, 2 p + 1) of row c.
  uint64_t a2[kInvPairs][kInvTileC];
#pragma unroll
  for (int p = 0; p < kInvPairs; ++p)
#pragma unroll
    for (int c = 0; c < kInvTileC; ++c)
      a2[p][c] = *reinterpret_cast<const uint64_t*>(&smE[(c0 + c) * kInvPitch + r0 + 2 * p]);
  const bool live = r0 < Dq && c0 < Dq;  // tiles beyond the padded size hold nothing
  // Buffer b of step k is rewritten at step k + 2, after its barriers, which
  // every thread reaches only once done with step k + 1, hence with step k.
  for (int k0 = 0, b = 0; k0 < Dq; k0 += 4, b ^= 1) {
    if (live) {
      // Pivot columns: the tile's columns 4 g .. 4 g + 3 when c0 + 4 g = k0.
#pragma unroll
      for (int g = 0; g < kInvTileC / 4; ++g)
        if (c0 + 4 * g == k0) {
#pragma unroll
          for (int p = 0; p < kInvPairs; ++p) {
            float l[4], h[4];
#pragma unroll
            for (int x = 0; x < 4; ++x) {
              f2_unpack(a2[p][4 * g + x], l[x], h[x]);
              a2[p][4 * g + x] = 0ull;
            }
            colS[b][r0 + 2 * p] = make_float4(l[0], l[1], l[2], l[3]);
            colS[b][r0 + 2 * p + 1] = make_float4(h[0], h[1], h[2], h[3]);
          }
        }
      // Pivot rows: the tile's rows 4 g .. 4 g + 3 (pairs 2 g, 2 g + 1) when
      // r0 + 4 g = k0.  Their entries in the pivot columns are not read.
#pragma unroll
      for (int g = 0; g < kInvTileR / 4; ++g)
        if (r0 + 4 * g == k0) {
#pragma unroll
          for (int q = 0; q < 2; ++q)
#pragma unroll
            for (int c = 0; c < kInvTileC; c += 4) {
              float l[4], h[4];
#pragma unroll
              for (int x = 0; x < 4; ++x) {
                f2_unpack(a2[2 * g + q][c + x], l[x], h[x]);
                a2[2 * g + q][c + x] = 0ull;
              }
              *reinterpret_cast<float4*>(&rowS[b][2 * q][c0 + c]) = make_float4(l[0], l[1], l[2], l[3]);
              *reinterpret_cast<float4*>(&rowS[b][2 * q + 1][c0 + c]) = make_float4(h[0], h[1], h[2], h[3]);
            }
        }
    }
    __syncthreads();
    // Column t of the new pivot rows: Pinv * (pivot rows) at t, or the pivot
    // block's own column of Pinv; and row t of cn.  Every such thread inverts
    // the 4 x 4 pivot block itself (cheaper than another barrier).
    if (t < Dq) {
      float pb[4][4];
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) pb[x][y] = reinterpret_cast<const float*>(&colS[b][k0 + x])[y];
      inv4_pivot(pb);
      const int x = t - k0;
      float4 rv, cn;
      if (x >= 0 && x < 4) {
        rv.x = x == 0 ? pb[0][0] : x == 1 ? pb[0][1] : x == 2 ? pb[0][2] : pb[0][3];
        rv.y = x == 0 ? pb[1][0] : x == 1 ? pb[1][1] : x == 2 ? pb[1][2] : pb[1][3];
        rv.z = x == 0 ? pb[2][0] : x == 1 ? pb[2][1] : x == 2 ? pb[2][2] : pb[2][3];
        rv.w = x == 0 ? pb[3][0] : x == 1 ? pb[3][1] : x == 2 ? pb[3][2] : pb[3][3];
        cn = make_float4(x == 0 ? 1.0f : 0.0f, x == 1 ? 1.0f : 0.0f, x == 2 ? 1.0f : 0.0f,
                         x == 3 ? 1.0f : 0.0f);
      } else {
        const float q0 = rowS[b][0][t], q1 = rowS[b][1][t], q2 = rowS[b][2][t], q3 = rowS[b][3][t];
        rv.x = pb[0][0] * q0 + pb[0][1] * q1 + pb[0][2] * q2 + pb[0][3] * q3;
        rv.y = pb[1][0] * q0 + pb[1][1] * q1 + pb[1][2] * q2 + pb[1][3] * q3;
        rv.z = pb[2][0] * q0 + pb[2][1] * q1 + pb[2][2] * q2 + pb[2][3] * q3;
        rv.w = pb[3][0] * q0 + pb[3][1] * q1 + pb[3][2] * q2 + pb[3][3] * q3;
        const float4 cv = colS[b][t];
        cn = make_float4(-cv.x, -cv.y, -cv.z, -cv.w);
      }
      const int sl = inv_rn_slot(t);
      rnA[b][sl] = make_ulonglong2(f2_pack(rv.x, rv.x), f2_pack(rv.y, rv.y));
      rnB[b][sl] = make_ulonglong2(f2_pack(rv.z, rv.z), f2_pack(rv.w, rv.w));
      cnS[b][0][t] = cn.x, cnS[b][1][t] = cn.y, cnS[b][2][t] = cn.z, cnS[b][3][t] = cn.w;
    } else if (t < kInvMaxPad) {  // columns past Dq inside the last tiles
      const int sl = inv_rn_slot(t);
      rnA[b][sl] = make_ulonglong2(0ull, 0ull);
      rnB[b][sl] = make_ulonglong2(0ull, 0ull);
      cnS[b][0][t] = 0.0f, cnS[b][1][t] = 0.0f, cnS[b][2][t] = 0.0f, cnS[b][3][t] = 0.0f;
    }
    __syncthreads();
    if (!live) continue;
    // a <- a + cn . rn: the tile's cn row pairs stay in registers across its
    // columns; four passes over the row pairs keep consecutive FMAs apart.
    uint64_t cnp[kInvPairs][4];
#pragma unroll
    for (int p = 0; p < kInvPairs; ++p)
#pragma unroll
      for (int y = 0; y < 4; ++y) cnp[p][y] = *reinterpret_cast<const uint64_t*>(&cnS[b][y][r0 + 2 * p]);
#pragma unroll
    for (int c = 0; c < kInvTileC; ++c) {
      const int sl = inv_rn_slot(c0 + c);
      const ulonglong2 ra = rnA[b][sl], rb = rnB[b][sl];
#pragma unroll
      for (int p = 0; p < kInvPairs; ++p) f2_fma(a2[p][c], cnp[p][0], ra.x);
#pragma unroll
      for (int p = 0; p < kInvPairs; ++p) f2_fma(a2[p][c], cnp[p][1], ra.y);
#pragma unroll
      for (int p = 0; p < kInvPairs; ++p) f2_fma(a2[p][c], cnp[p][2], rb.x);
#pragma unroll
      for (int p = 0; p < kInvPairs; ++p) f2_fma(a2[p][c], cnp[p][3], rb.y);
    }
  }
  // The tile back to shared memory, transposed as it was read (the prologue's
  // reads of it ended at the first step's barriers); then unscale and
  // symmetrise into E^-1: smE[j][i] holds entry (i, j).
#pragma unroll
  for (int p = 0; p < kInvPairs; ++p)
#pragma unroll
    for (int c = 0; c < kInvTileC; ++c)
      *reinterpret_cast<uint64_t*>(&smE[(c0 + c) * kInvPitch + r0 + 2 * p]) = a2[p][c];
  __syncthreads();
  float* Im = A.Einv + A.model_eoff[m];
  for (int i = wid; i < D; i += kInvThreads / 32)
    for (int j = lane; j < D; j += 32) {
      const float xij = smE[j * kInvPitch + i] * dsc[i] * dsc[j];
      const float xji = smE[i * kInvPitch + j] * dsc[j] * dsc[i];
      Im[(size_t)i * D + j] = 0.5f * (xij + xji);
    }
}

}  // namespace ba
