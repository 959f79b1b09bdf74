// Matrix-free block-Jacobi PCG (ba.rs:155-196) for one model whose reduced
// matrix is not formed.  The product with the reduced camera system
//     S p = A p - sum over points of E_p^T (E_p p)
// is applied from the per-observation Schur factors Z_k = Y_k L_p (E_p stacks
// the point's Z_k^T and its lens entries' factors), the cameras' own blocks
// A_c (damped U_c with priors) and their camera-lens blocks X_c, and the lens
// block A_g.  Nothing of size (camera pairs) is stored: no pair list, no
// Schur sums, no S.  The factors are either stored by the point kernels
// (Z non-null) or, in the mixed form's J^T J-recompute mode (Z null),
// recomputed in every product from the stored FP32 Jacobians and the
// points' factors (z_of_obs), so nothing of size (observations x factor) is
// stored either.
//
// One persistent cooperative launch per LM iteration; the CTAs form one
// group.  An iteration has four phases separated by group exchanges:
//   0. per row: p = z + β p_prev;
//   1. per point: t_p = E_p p; the lens entries' shares Zl t_p are summed
//      per CTA;
//   2. per camera (a CTA each): q_c = A_c p_c + X_c p_g - sum_k Z_k t_p(k); p·q and the
//      lens row's transposed terms X_c^T p_c are summed per CTA; the lens row
//      q_g = A_g p_g + sum_c X_c^T p_c - sum_j Zl_j t_p(j) is formed by every
//      CTA from the exchanged sums;
//   3. per row: x += a p, r -= a q, z = M r; r·r and r·z.
// Single lens group (or none) per model.
#pragma once

#include "pcg.cuh"

namespace ba {

template <typename R>
struct ImpArgs {
  // group exchange (the fields group_reduce uses)
  unsigned long long* bar;
  unsigned long long* bar_base;
  double* part;  // [kParts][ncta]
  int32_t ncta;
  unsigned* err;
  // problem and per-iteration buffers
  Prob P;
  StructView SV;
  const R* Z;        // [no][18], or null: recomputed (mixed form, from zsrc)
  const R* Zl;       // [nl][9]
  const uint8_t* kept;
  const R* own;      // [nb][36]: A_c (cameras) / A_g (lens row)
  const double* camX;  // [nc][18]: X_c = sum w Jc^T Jg (6x3)
  const R* pre;      // [nb][36]
  const R* b;        // [nb][6]
  R* x;              // [nb][6]
  R* r;              // [nb][6]
  R* z;              // [nb][6]
  R* p2;             // [2][nb][6]
  R* q;              // [nb][6]
  R* t;              // [np][3]
  int32_t lens;      // the lens block row, or -1
  int32_t nb;
  int32_t* iters;
  int32_t max_iter;
  double tol;
  long long spin;  // spin limit of a group wait, in SM clock cycles
  const int32_t* cap = nullptr;  // [1] or null: iteration cap of the model (below max_iter)
  ZSource zsrc{};                 // the factors' source when Z is null
};

// Observation k's Schur factor: stored, or recomputed (kRecompute: the
// mixed form with Z null).
template <bool kRecompute, typename R>
__device__ __forceinline__ void imp_factor(const ImpArgs<R>& A, int64_t k, uint32_t p, R* zk) {
  if constexpr (kRecompute && sizeof(R) == 4)
    z_of_obs(A.zsrc, k, p, zk);
  else
    load_Z18(A.Z + 18 * (size_t)k, zk);
}

// Implicit-product scalars, computed once per CTA by thread 0.
template <typename R>
struct ImpScalars {
  double rz, b2, beta, a, lensq[3];
  R beta_r, a_r;
  int stop;
};

template <typename R, bool kRecompute>
__global__ void __launch_bounds__(kPcgThreads) pcg_implicit_kernel(ImpArgs<R> A) {
  __shared__ double wsm[kPcgWarps * 4];
  __shared__ double tot[4];
  __shared__ ImpScalars<R> sc;
  __shared__ R smem_q[kPcgWarps * 6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gw = blockIdx.x * kPcgWarps + warp, nw = gridDim.x * kPcgWarps;
  const PcgJob J{0, (int32_t)blockIdx.x, (int32_t)gridDim.x, 0, 0, 0};
  unsigned long long target = A.bar_base[0];
  const bool vl = lane < 6;
  const int ci = vl ? lane : 0;
  const uint32_t nc = (uint32_t)A.P.nc;
  const int32_t lens = A.lens;

  // x = 0, r = b, z = M r, p(prev) = 0 (ba.rs:164-168)
  double w2[2] = {0.0, 0.0};
  for (int32_t row = gw; row < A.nb; row += nw) {
    const R ri = vl ? A.b[6 * (size_t)row + ci] : (R)0;
    R zi = (R)0;
    const R* M = A.pre + 36 * (size_t)row;
#pragma unroll
    for (int j = 0; j < 6; ++j) zi += M[6 * ci + j] * __shfl_sync(kFull, ri, j);
    double a = 0.0, bb = 0.0;
    if (vl) {
      A.x[6 * (size_t)row + ci] = (R)0;
      A.r[6 * (size_t)row + ci] = ri;
      A.z[6 * (size_t)row + ci] = zi;
      A.p2[6 * (size_t)A.nb + 6 * (size_t)row + ci] = (R)0;
      a = (double)ri * (double)zi;
      bb = (double)ri * (double)ri;
    }
    w2[0] += sum8(a);
    w2[1] += sum8(bb);
  }
  if (!group_reduce<2>(w2, wsm, tot, A, J, 0, target, [&] {
        sc.rz = tot[0];
        sc.b2 = fmax(tot[1], 1e-300);
        sc.beta = 0.0;
        sc.beta_r = (R)0;
        sc.stop = 0;
      }))
    return;
  int32_t spmv = 0;
  const int32_t max_it = A.cap ? min(A.max_iter, A.cap[0]) : A.max_iter;
  for (int32_t it = 0; it < max_it; ++it) {
    R* pcur = A.p2 + (size_t)(it & 1) * 6 * A.nb;
    const R* pprev = A.p2 + (size_t)((it + 1) & 1) * 6 * A.nb;
    const R br = sc.beta_r;
    // Phase 0: p = z + β p_prev for every block row (thread per component).
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < 6 * (int64_t)A.nb;
         e += (int64_t)gridDim.x * blockDim.x)
      pcur[e] = (R)(__ldcg(A.z + e) + __ldcg(pprev + e) * br);
    {
      const double w1[1] = {0.0};
      if (!group_reduce<1>(w1, wsm, tot, A, J, 8, target, [] {})) return;
    }
    R pg[3] = {(R)0, (R)0, (R)0};  // the lens row's p
    if (lens >= 0)
#pragma unroll
      for (int i = 0; i < 3; ++i) pg[i] = __ldcg(pcur + 6 * (size_t)lens + i);

    // Phase 1: t_p = E_p p per point (thread per point).
    double wl[3] = {0.0, 0.0, 0.0};  // sum over lens entries of Zl t
    for (int64_t pt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; pt < A.P.np;
         pt += (int64_t)gridDim.x * blockDim.x) {
      R t0 = (R)0, t1 = (R)0, t2 = (R)0;
      if (A.kept[pt]) {
        for (uint32_t k = A.SV.pt_ptr[pt]; k < A.SV.pt_ptr[pt + 1]; ++k) {
          const uint32_t cb = A.P.cam_blk[A.P.obs_cam[k]];
          R zk[18], pv[6];
          imp_factor<kRecompute>(A, k, (uint32_t)pt, zk);
#pragma unroll
          for (int i = 0; i < 6; ++i) pv[i] = __ldcg(pcur + 6 * (size_t)cb + i);
#pragma unroll
          for (int i = 0; i < 6; ++i) {
            t0 += zk[3 * i] * pv[i];
            t1 += zk[3 * i + 1] * pv[i];
            t2 += zk[3 * i + 2] * pv[i];
          }
        }
        for (uint32_t j = A.SV.lens_ptr[pt]; j < A.SV.lens_ptr[pt + 1]; ++j) {
          const R* Zj = A.Zl + 9 * (size_t)j;
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            t0 += Zj[3 * i] * pg[i];
            t1 += Zj[3 * i + 1] * pg[i];
            t2 += Zj[3 * i + 2] * pg[i];
          }
        }
        for (uint32_t j = A.SV.lens_ptr[pt]; j < A.SV.lens_ptr[pt + 1]; ++j) {
          const R* Zj = A.Zl + 9 * (size_t)j;
#pragma unroll
          for (int i = 0; i < 3; ++i)
            wl[i] += (double)(Zj[3 * i] * t0 + Zj[3 * i + 1] * t1 + Zj[3 * i + 2] * t2);
        }
      }
      R* tp = A.t + 3 * (size_t)pt;
      tp[0] = t0, tp[1] = t1, tp[2] = t2;
    }
    {
      double w3[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) w3[i] = warp_sum(wl[i]);
      if (!group_reduce<3>(w3, wsm, tot, A, J, 9, target, [&] {
            for (int i = 0; i < 3; ++i) sc.lensq[i] = -tot[i];
          }))
        return;
    }

    // Phase 2: q_c = A_c p_c + X_c p_g - sum_k Z_k t_p(k), a CTA per camera
    // (its observations strided over the CTA, summed in a fixed order).
    double w4[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint32_t c = blockIdx.x; c < nc; c += gridDim.x) {
      const uint32_t row = A.P.cam_blk[c];
      R acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (uint32_t i = A.SV.cam_ptr[c] + threadIdx.x; i < A.SV.cam_ptr[c + 1]; i += blockDim.x) {
        const uint32_t k = A.SV.cam_obs[i];
        const uint32_t pk = A.P.obs_pt[k];
        R zk[18];
        imp_factor<kRecompute>(A, k, pk, zk);
        const R* tp = A.t + 3 * (size_t)pk;
        const R u0 = __ldcg(tp), u1 = __ldcg(tp + 1), u2 = __ldcg(tp + 2);
#pragma unroll
        for (int r = 0; r < 6; ++r) acc[r] -= zk[3 * r] * u0 + zk[3 * r + 1] * u1 + zk[3 * r + 2] * u2;
      }
      warp_sum8(acc);  // lane 4i holds this warp's Schur part of q_i
      __syncthreads();  // smem_q of the previous camera has been read
      if ((lane & 3) == 0 && lane < 24) smem_q[warp * 6 + (lane >> 2)] = acc[0];
      __syncthreads();
      if (warp == 0) {
        R si = (R)0;
        if (vl)
          for (int w = 0; w < kPcgWarps; ++w) si += smem_q[w * 6 + ci];
        const R pi = vl ? __ldcg(pcur + 6 * (size_t)row + ci) : (R)0;
        const R* Ac = A.own + 36 * (size_t)row;
        R qi = si;
#pragma unroll
        for (int j = 0; j < 6; ++j) qi += Ac[6 * ci + j] * __shfl_sync(kFull, pi, j);
        const double* X = A.camX + 18 * (size_t)c;
        if (lens >= 0)
#pragma unroll
          for (int j = 0; j < 3; ++j) qi += (R)X[3 * ci + j] * pg[j];
        if (vl) A.q[6 * (size_t)row + ci] = qi;
        w4[0] += sum8(vl ? (double)pi * (double)qi : 0.0);
        if (lens >= 0) {  // X_c^T p_c for the lens row
          double xt[3];
#pragma unroll
          for (int j = 0; j < 3; ++j) xt[j] = sum8(vl ? X[3 * ci + j] * (double)pi : 0.0);
          w4[1] += xt[0], w4[2] += xt[1], w4[3] += xt[2];
        }
      }
    }
    if (!group_reduce<4>(w4, wsm, tot, A, J, 2, target, [&] {
          double pq = tot[0];
          if (lens >= 0) {
            // q_g = A_g p_g + sum_c X_c^T p_c - sum_j Zl_j t_p(j)
            const R* Ag = A.own + 36 * (size_t)lens;
            double qg[3];
            for (int i = 0; i < 3; ++i) {
              double v = tot[1 + i] + sc.lensq[i];
              for (int j = 0; j < 3; ++j) v += (double)Ag[6 * i + j] * (double)pg[j];
              qg[i] = v;
              pq += (double)pg[i] * v;
            }
            for (int i = 0; i < 3; ++i) {
              sc.lensq[i] = qg[i];
              if (blockIdx.x == 0) A.q[6 * (size_t)lens + i] = (R)qg[i];
            }
          }
          sc.stop = fabs(pq) < 1e-300 ? 1 : 0;  // ba.rs:174
          sc.a = sc.stop ? 0.0 : sc.rz / pq;
          sc.a_r = (R)sc.a;
        }))
      return;
    ++spmv;
    if (sc.stop) break;
    const R a = sc.a_r;

    // Phase 3: x += a p, r -= a q, z = M r (warp per row).
    double w2b[2] = {0.0, 0.0};
    for (int32_t row = gw; row < A.nb; row += nw) {
      R ri = (R)0;
      if (vl) {
        const size_t o = 6 * (size_t)row + ci;
        const R qv = row == lens ? (R)sc.lensq[ci < 3 ? ci : 0] * (R)(ci < 3) : __ldcg(A.q + o);
        const R pv = __ldcg(pcur + o);
        A.x[o] = A.x[o] + pv * a;
        ri = A.r[o] - qv * a;
        A.r[o] = ri;
      }
      R zi = (R)0;
      const R* M = A.pre + 36 * (size_t)row;
#pragma unroll
      for (int j = 0; j < 6; ++j) zi += M[6 * ci + j] * __shfl_sync(kFull, ri, j);
      double rr = 0.0, rzl = 0.0;
      if (vl) {
        A.z[6 * (size_t)row + ci] = zi;
        rr = (double)ri * (double)ri;
        rzl = (double)ri * (double)zi;
      }
      w2b[0] += sum8(rr);
      w2b[1] += sum8(rzl);
    }
    if (!group_reduce<2>(w2b, wsm, tot, A, J, 6, target, [&] {
          sc.stop = tot[0] < A.tol * sc.b2 ? 1 : 0;  // ba.rs:182
          sc.beta = tot[1] / sc.rz;                    // ba.rs:189-190
          sc.beta_r = (R)sc.beta;
          sc.rz = tot[1];
        }))
      return;
    if (sc.stop) break;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    A.iters[0] = spmv;
    A.bar_base[0] = target;
  }
}

// A_b: the block row's own 6x6 block of the reduced matrix before the Schur
// subtraction (ba.rs:293-319: camera U_c with priors, or the lens block with
// its padding, damped); the preconditioner's diagonal block is A_b minus the
// row's own Schur terms sum Z Z^T (cameras: over their observations; lens
// row: over all lens entries), inverted in FP64 (ba.rs:159-160).
// Lens row's own Schur terms sum_j Zl_j Zl_j^T over every lens entry, as
// kLensChunks partial sums (CTA per chunk, fixed order).
constexpr int kLensChunks = 256;

template <typename R>
__global__ void lens_diag_kernel(StructView S, IterBufs<R> B, double* lens_part) {
  __shared__ double red[9 * 32];
  const int64_t ch = blockIdx.x;
  const int64_t j0 = S.nl * ch / kLensChunks, j1 = S.nl * (ch + 1) / kLensChunks;
  double s[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) s[i] = 0.0;
  for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const R* Zj = B.Zl + 9 * (size_t)j;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        s[3 * r + c] += (double)(Zj[3 * r] * Zj[3 * c] + Zj[3 * r + 1] * Zj[3 * c + 1] +
                                 Zj[3 * r + 2] * Zj[3 * c + 2]);
  }
  block_sum<9>(s, red);
  if (threadIdx.x == 0)
    for (int i = 0; i < 9; ++i) lens_part[9 * ch + i] = s[i];
}

// Z null: the factors recomputed from zsrc (mixed form).
template <typename R>
__global__ void implicit_blocks_kernel(Prob P, StateView st, StructView S, IterBufs<R> B,
                                       const R* Z, R* own, const int32_t* active,
                                       const double* lambda, const double* lens_part,
                                       ZSource zsrc) {
  __shared__ double red[36 * 32];
  const int64_t b = blockIdx.x;
  if (b >= P.nb) return;
  const uint32_t m = P.blk_model[b];
  if (!active[m]) return;
  const double lam = lambda[m];
  const bool lens_b = P.blk_is_lens[b] != 0;
  const uint32_t id = P.blk_id[b];
  double s[36];
#pragma unroll
  for (int i = 0; i < 36; ++i) s[i] = 0.0;
  if (!lens_b) {
    for (uint32_t i = S.cam_ptr[id] + threadIdx.x; i < S.cam_ptr[id + 1]; i += blockDim.x) {
      const uint32_t k = S.cam_obs[i];
      R zr[18];
      const R* Zk = Z ? Z + 18 * (size_t)k : zr;
      if constexpr (sizeof(R) == 4)
        if (!Z) z_of_obs(zsrc, k, P.obs_pt[k], zr);
#pragma unroll
      for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int c = 0; c < 6; ++c)
          s[6 * r + c] += (double)(Zk[3 * r] * Zk[3 * c] + Zk[3 * r + 1] * Zk[3 * c + 1] +
                                   Zk[3 * r + 2] * Zk[3 * c + 2]);
    }
  } else if (threadIdx.x == 0) {
    // the lens row (one group per matrix-free call): chunk partials in order
    for (int ch = 0; ch < kLensChunks; ++ch)
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) s[6 * r + c] += lens_part[9 * ch + 3 * r + c];
  }
  block_sum<36>(s, red);
  if (threadIdx.x != 0) return;
  double A[36], D[36], Ai[36];
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) {
      const int i0 = r < c ? r : c, i1 = r < c ? c : r;
      double u = 0.0;
      if (!lens_b) {
        u = B.camU[21 * (size_t)id + (i0 * 6 - (i0 * (i0 - 1)) / 2 + (i1 - i0))];
        if (r == c && r >= 3 && P.prior_mask && P.prior_mask[id]) {
          const double sd = P.prior[6 * (size_t)id + r];
          u += 1.0 / (sd * sd);  // ba.rs:297-302
        }
        if (r == c) u = u * (1.0 + lam) + 1e-9;  // ba.rs:306-309
      } else {
        if (i1 < 3) u = B.grpU[6 * (size_t)id + (i0 * 3 - (i0 * (i0 - 1)) / 2 + (i1 - i0))];
        if (r == c) u = u * (1.0 + lam) + 1e-9;
        if (r == c && r >= 3) u = 1.0;  // ba.rs:310-314
        if (!P.model_refine[m]) u = (r == c) ? 1.0 : 0.0;  // ba.rs:315-317
      }
      A[6 * r + c] = u;
      D[6 * r + c] = u - s[6 * r + c];
    }
  if (!inv6(D, Ai))  // ba.rs:159-160
    for (int i = 0; i < 36; ++i) Ai[i] = (i % 7 == 0) ? 1.0 : 0.0;
  for (int i = 0; i < 36; ++i) {
    own[36 * b + i] = (R)A[i];
    B.pre[36 * b + i] = (R)Ai[i];
  }
}

}  // namespace ba
