// Block-Jacobi preconditioned conjugate gradients on the reduced camera
// system (ba.rs:155-196), as one persistent cooperative kernel.
//
// Each model's block rows are split over a group of CTAs.  The reference's
// iteration
//     q = S p;  a = rz / p·q;  x += a p;  r -= a q;  stop if r·r < tol b·b;
//     z = M r;  β = r·z / rz;  p = z + β p
// needs three group-wide exchanges (p, p·q, r·r and r·z).  Here p is never
// exchanged: every CTA forms p_j = z_j + β p_j(prev) on the fly for the columns
// its matrix-vector product touches (z and the previous p are double-buffered
// and visible after the previous exchange), so an iteration costs two group
// barriers.
//
// The lens block row of a model couples to every camera, so it is not
// multiplied by one CTA: every camera row c adds S_cg^T p_c to a lens partial,
// which travels with the p·q partial sums (S is symmetric, S_gc = S_cg^T).
//
// FP64 instructions on this GPU cost ~64 cycles per SM sub-partition whatever
// the number of active lanes, so reductions pack several values per
// instruction (recursive halving) instead of one butterfly per value.
//
// Inner products are FP64 and summed in a fixed order (fixed lane trees, CTA
// partials in rank order), so every CTA of a group sees bit-identical scalars
// and results do not depend on timing.  Models never wait on each other.
#pragma once

#include "lm_kernels.cuh"

namespace ba {

constexpr int kPcgThreads = 256;
constexpr int kPcgWarps = kPcgThreads / 32;
constexpr uint32_t kLongRow = 64;  // blocks; longer rows (other than the lens row) use all warps

struct PcgJob {
  int32_t model, rank, gsize, base;  // base: first CTA of the group
  uint32_t row0, row1;               // this CTA's block rows
};

template <typename R>
struct PcgArgs {
  const PcgJob* jobs;
  const int32_t* cta_job0;  // [ncta+1]
  unsigned long long* bar;  // [nm] arrival counters
  double* part;             // [kParts][ncta]
  int32_t ncta;
  const uint32_t* row_ptr;
  const uint32_t* col_idx;
  const R* S;
  const R* pre;  // block-Jacobi inverses, computed in FP64, stored in R
  const R* b;
  R *x, *r, *z, *q;
  R* p2;  // [2][nb][6] double-buffered search direction
  int64_t nb;
  const int32_t* lens_row;  // [nm]: the model's single lens block row, or -1
  const int32_t* active;
  int32_t* iters;
  int32_t max_iter;
  double tol;
  unsigned* err;
};

// partial slots: 0,1 init (rz, bb) | 2..5 (pq, lens q 0..2) | 6,7 (rr, rz)
constexpr int kParts = 8;

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long atom_add_release_u64(unsigned long long* p,
                                                                   unsigned long long v) {
  unsigned long long old;
  asm volatile("atom.add.release.gpu.global.u64 %0, [%1], %2;"
               : "=l"(old)
               : "l"(p), "l"(v)
               : "memory");
  return old;
}

// Barrier over the n CTAs of a group: a monotonic 64-bit arrival counter
// (release on arrival, acquire while polling).  Bounded: after kSpinCycles
// the waiter sets ERR_BARRIER_TIMEOUT; every CTA leaves at its next wait.
__device__ __forceinline__ bool counter_sync(unsigned long long* ctr, unsigned n,
                                             unsigned* err) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    if (n > 1) {
      const unsigned long long old = atom_add_release_u64(ctr, 1ULL);
      const unsigned long long target = (old / n + 1) * n;
      const long long t0 = clock64();
      while (ld_acquire_u64(ctr) < target) {
        if ((*(volatile unsigned*)err) & ERR_BARRIER_TIMEOUT) {
          ok = 0;
          break;
        }
        if (clock64() - t0 > kSpinCycles) {
          atomicOr(err, ERR_BARRIER_TIMEOUT);
          ok = 0;
          break;
        }
      }
    }
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// Warp sum of 8 values per lane by recursive halving: afterwards lane 4k
// (k < 8) holds the full sum of value k.  9 adds instead of 8 x 5.
template <typename T>
__device__ __forceinline__ void warp_sum8(T (&v)[8]) {
  const int lane = threadIdx.x & 31;
  {
    const bool up = lane & 16;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const T send = up ? v[i] : v[4 + i];
      const T recv = __shfl_xor_sync(kFull, send, 16);
      v[i] = (up ? v[4 + i] : v[i]) + recv;
    }
  }
  {
    const bool up = lane & 8;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const T send = up ? v[i] : v[2 + i];
      const T recv = __shfl_xor_sync(kFull, send, 8);
      v[i] = (up ? v[2 + i] : v[i]) + recv;
    }
  }
  {
    const bool up = lane & 4;
    const T send = up ? v[0] : v[1];
    const T recv = __shfl_xor_sync(kFull, send, 4);
    v[0] = (up ? v[1] : v[0]) + recv;
  }
  v[0] += __shfl_xor_sync(kFull, v[0], 2);
  v[0] += __shfl_xor_sync(kFull, v[0], 1);
}

// Sum N (<= 8) per-warp values over the CTA's warps, then over the group's
// CTAs in rank order; every thread receives the totals in tot[].
template <int N, typename R>
__device__ __forceinline__ bool group_reduce(const double (&wv)[N], double* wsm, double* tot,
                                             const PcgArgs<R>& A, const PcgJob& J, int slot) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < N; ++i) wsm[warp * 8 + i] = wv[i];
  __syncthreads();
  if (warp == 0) {
    // CTA partial: value i summed over the warps in order.
    double c = 0.0;
    if (lane < N)
      for (int w = 0; w < kPcgWarps; ++w) c += wsm[w * 8 + lane];
    if (J.gsize > 1) {
      if (lane < N) A.part[(size_t)(slot + lane) * A.ncta + J.base + J.rank] = c;
      __threadfence();
    } else if (lane < N) {
      tot[lane] = c;
    }
  }
  if (J.gsize > 1) {
    if (!counter_sync(A.bar + J.model, (unsigned)J.gsize, A.err)) return false;
    if (warp == 0) {
      double v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        double s = 0.0;
        if (i < N) {
          const double* src = A.part + (size_t)(slot + i) * A.ncta + J.base;
          for (int k = lane; k < J.gsize; k += 32) s += __ldcg(src + k);
        }
        v[i] = s;
      }
      warp_sum8(v);
      if ((lane & 3) == 0 && (lane >> 2) < N) tot[lane >> 2] = v[0];
    }
  }
  __syncthreads();
  return true;
}

// A 6x6 block into registers with 16-byte loads.
template <typename A>
__device__ __forceinline__ void load_block(const double* blk, A* m) {
  const double2* v = reinterpret_cast<const double2*>(blk);
#pragma unroll
  for (int i = 0; i < 18; ++i) {
    const double2 t = __ldg(v + i);
    m[2 * i] = (A)t.x, m[2 * i + 1] = (A)t.y;
  }
}
template <typename A>
__device__ __forceinline__ void load_block(const float* blk, A* m) {
  const float4* v = reinterpret_cast<const float4*>(blk);
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const float4 t = __ldg(v + i);
    m[4 * i] = (A)t.x, m[4 * i + 1] = (A)t.y, m[4 * i + 2] = (A)t.z, m[4 * i + 3] = (A)t.w;
  }
}

// p_j = z_j + β p_j(prev), the reference's update (ba.rs:192), in storage
// precision; the same expression for own rows and for gathered columns.
template <typename R>
__device__ __forceinline__ R p_of(R zj, R pj, double beta) {
  return (R)(zj + pj * (R)beta);
}

template <typename R>
__device__ __forceinline__ void gather_p(const PcgArgs<R>& A, const R* pprev, uint32_t col,
                                         double beta, R* pp) {
  const R* zv = A.z + 6 * (size_t)col;
  const R* pv = pprev + 6 * (size_t)col;
#pragma unroll
  for (int j = 0; j < 6; ++j) pp[j] = p_of<R>(__ldcg(zv + j), __ldcg(pv + j), beta);
}

template <typename R>
__device__ bool pcg_job(const PcgArgs<R>& A, const PcgJob& J, double* wsm, double* tot,
                        double* long_part) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int32_t lens = A.lens_row[J.model];  // -1: no transposed lens row
  // Six threads per block row for the vector phases: lanes 6s..6s+5 of a
  // warp hold row (warp*5 + s), component lane%6.
  const int sub = lane / 6, comp = lane - 6 * sub;
  const bool vlane = sub < 5;
  // x = 0, r = b, z = M r, p(prev) = 0 (ba.rs:164-168; β = 0 gives p = z)
  double acc2[2] = {0.0, 0.0};
  for (uint32_t grp = warp; grp * 5 < J.row1 - J.row0; grp += kPcgWarps) {
    const uint32_t row = J.row0 + grp * 5 + sub;
    const bool on = vlane && row < J.row1;
    const size_t o = 6 * (size_t)row + comp;
    const R rb = on ? A.b[o] : (R)0;
    R zi = (R)0;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const R rj = __shfl_sync(kFull, rb, min(6 * sub + j, 31));
      if (on) zi += A.pre[36 * (size_t)row + 6 * comp + j] * rj;
    }
    if (on) {
      A.x[o] = (R)0;
      A.r[o] = rb;
      A.z[o] = zi;
      A.p2[(size_t)6 * A.nb + o] = (R)0;
      acc2[0] += (double)rb * (double)zi;
      acc2[1] += (double)rb * (double)rb;
    }
  }
  {
    double v[8] = {acc2[0], acc2[1], 0, 0, 0, 0, 0, 0};
    warp_sum8(v);
    double wv[2] = {__shfl_sync(kFull, v[0], 0), __shfl_sync(kFull, v[0], 4)};
    if (!group_reduce<2>(wv, wsm, tot, A, J, 0)) return false;
  }
  double rz = tot[0];
  const double b2 = fmax(tot[1], 1e-300);
  double beta = 0.0;
  int32_t spmv = 0;
  for (int32_t it = 0; it < A.max_iter; ++it) {
    R* pcur = A.p2 + (size_t)(it & 1) * 6 * A.nb;
    const R* pprev = A.p2 + (size_t)((it + 1) & 1) * 6 * A.nb;
    // q = S p (ba.rs:144-152), warp per camera block row; per warp: p·q and
    // the lens partial Σ S_cg^T p_c (3 components; the rest of S_cg^T is 0).
    double wpq = 0.0, wl0 = 0.0, wl1 = 0.0, wl2 = 0.0;
    for (uint32_t row = J.row0 + warp; row < J.row1; row += kPcgWarps) {
      const uint32_t b0 = A.row_ptr[row], b1 = A.row_ptr[row + 1];
      const bool is_lens = (int32_t)row == lens;
      if (!is_lens && b1 - b0 > kLongRow) continue;
      R pown[6];
#pragma unroll
      for (int j = 0; j < 6; ++j) pown[j] = p_of<R>(A.z[6 * (size_t)row + j], pprev[6 * (size_t)row + j], beta);
      R acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      R tl0 = 0, tl1 = 0, tl2 = 0;
      for (uint32_t k = b0 + lane; k < b1; k += 32) {
        const uint32_t col = A.col_idx[k];
        // Lens row: only its blocks with the lens column (the diagonal);
        // camera columns arrive through the camera rows' transposed terms.
        if (is_lens && (int32_t)col != lens) continue;
        R m[36], pp[6];
        load_block(A.S + (size_t)k * 36, m);
        gather_p<R>(A, pprev, col, beta, pp);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          R a = 0;
#pragma unroll
          for (int j = 0; j < 6; ++j) a += m[6 * i + j] * pp[j];
          acc[i] += a;
        }
        if (!is_lens && (int32_t)col == lens) {
#pragma unroll
          for (int t = 0; t < 6; ++t) {
            tl0 += m[6 * t + 0] * pown[t];
            tl1 += m[6 * t + 1] * pown[t];
            tl2 += m[6 * t + 2] * pown[t];
          }
        }
      }
      acc[6] = tl0, acc[7] = tl1;
      warp_sum8(acc);  // lane 4i holds q_i (i < 6) and lens terms 0, 1
      R tl2s = tl2;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) tl2s += __shfl_xor_sync(kFull, tl2s, o);
      // q_i lives in lane 4i; p·q = Σ p_i q_i over lanes 0, 4, .., 20.
      const int qi = lane >> 2;
      const bool qlane = (lane & 3) == 0 && qi < 6;
      if (qlane) A.q[6 * (size_t)row + qi] = acc[0];
      double d = 0.0;
      if (qlane)
        d = (double)p_of<R>(A.z[6 * (size_t)row + qi], pprev[6 * (size_t)row + qi], beta) *
            (double)acc[0];
      d += __shfl_xor_sync(kFull, d, 4);
      d += __shfl_xor_sync(kFull, d, 8);
      d += __shfl_xor_sync(kFull, d, 16);
      wpq += __shfl_sync(kFull, d, 0);
      wl0 += (double)__shfl_sync(kFull, acc[0], 24);
      wl1 += (double)__shfl_sync(kFull, acc[0], 28);
      wl2 += (double)tl2s;
    }
    // Rows longer than kLongRow that are not a transposed lens row: all warps.
    for (uint32_t row = J.row0; row < J.row1; ++row) {  // CTA-uniform
      const uint32_t b0 = A.row_ptr[row], b1 = A.row_ptr[row + 1];
      if ((int32_t)row == lens || b1 - b0 <= kLongRow) continue;
      const uint32_t chunk = (b1 - b0 + kPcgWarps - 1) / kPcgWarps;
      const uint32_t k0 = b0 + warp * chunk, k1 = min(b1, k0 + chunk);
      R acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (uint32_t k = k0 + lane; k < k1; k += 32) {
        R m[36], pp[6];
        load_block(A.S + (size_t)k * 36, m);
        gather_p<R>(A, pprev, A.col_idx[k], beta, pp);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          R a = 0;
#pragma unroll
          for (int j = 0; j < 6; ++j) a += m[6 * i + j] * pp[j];
          acc[i] += a;
        }
      }
      warp_sum8(acc);
      if ((lane & 3) == 0 && (lane >> 2) < 6) long_part[6 * warp + (lane >> 2)] = (double)acc[0];
      __syncthreads();
      if (threadIdx.x == 0) {
        double d = 0.0;
        for (int i = 0; i < 6; ++i) {
          R s = 0;
          for (int w = 0; w < kPcgWarps; ++w) s += (R)long_part[6 * w + i];
          A.q[6 * (size_t)row + i] = s;
          d += (double)p_of<R>(A.z[6 * (size_t)row + i], pprev[6 * (size_t)row + i], beta) *
               (double)s;
        }
        wpq += d;
      }
      __syncthreads();
    }
    // own rows: p = z + β p(prev) for the update below and the next gather
    for (uint32_t grp = warp; grp * 5 < J.row1 - J.row0; grp += kPcgWarps) {
      const uint32_t row = J.row0 + grp * 5 + sub;
      if (vlane && row < J.row1) {
        const size_t o = 6 * (size_t)row + comp;
        pcur[o] = p_of<R>(A.z[o], pprev[o], beta);
      }
    }
    {
      double wv[4] = {wpq, wl0, wl1, wl2};
      if (!group_reduce<4>(wv, wsm, tot, A, J, 2)) return false;
    }
    ++spmv;
    double pq = tot[0];
    // The lens row's q: its diagonal product (computed by its owner in the
    // row loop above) plus the reduced transposed partials.
    if (lens >= 0 && (uint32_t)lens >= J.row0 && (uint32_t)lens < J.row1 && threadIdx.x < 3) {
      const size_t o = 6 * (size_t)lens + threadIdx.x;
      A.q[o] = (R)((double)A.q[o] + tot[1 + threadIdx.x]);
    }
    if (lens >= 0) {
      // p_g · (Σ S_cg^T p_c): the lens row's share of p·q.
      const R* pg = pcur + 6 * (size_t)lens;
      const R* zg = A.z + 6 * (size_t)lens;
      const R* pgp = pprev + 6 * (size_t)lens;
      (void)pg;
      pq += (double)p_of<R>(__ldcg(zg + 0), __ldcg(pgp + 0), beta) * tot[1] +
            (double)p_of<R>(__ldcg(zg + 1), __ldcg(pgp + 1), beta) * tot[2] +
            (double)p_of<R>(__ldcg(zg + 2), __ldcg(pgp + 2), beta) * tot[3];
    }
    __syncthreads();
    if (fabs(pq) < 1e-300) break;  // ba.rs:174
    const double a = rz / pq;
    // x += a p, r -= a q, z = M r (ba.rs:178-188), six threads per row.
    double acc3[2] = {0.0, 0.0};
    for (uint32_t grp = warp; grp * 5 < J.row1 - J.row0; grp += kPcgWarps) {
      const uint32_t row = J.row0 + grp * 5 + sub;
      const bool on = vlane && row < J.row1;
      const size_t o = 6 * (size_t)row + comp;
      R ri = (R)0;
      if (on) {
        A.x[o] = A.x[o] + pcur[o] * (R)a;
        ri = A.r[o] - A.q[o] * (R)a;
        A.r[o] = ri;
      }
      R zi = (R)0;
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        const R rj = __shfl_sync(kFull, ri, min(6 * sub + j, 31));
        if (on) zi += A.pre[36 * (size_t)row + 6 * comp + j] * rj;
      }
      if (on) {
        A.z[o] = zi;
        acc3[0] += (double)ri * (double)ri;
        acc3[1] += (double)ri * (double)zi;
      }
    }
    {
      double v[8] = {acc3[0], acc3[1], 0, 0, 0, 0, 0, 0};
      warp_sum8(v);
      double wv[2] = {__shfl_sync(kFull, v[0], 0), __shfl_sync(kFull, v[0], 4)};
      if (!group_reduce<2>(wv, wsm, tot, A, J, 6)) return false;
    }
    const double rr = tot[0], rz2 = tot[1];
    __syncthreads();
    if (rr < A.tol * b2) break;  // ba.rs:182
    beta = rz2 / rz;             // ba.rs:189-190
    rz = rz2;
  }
  if (J.rank == 0 && threadIdx.x == 0) A.iters[J.model] = spmv;
  return true;
}

template <typename R>
__global__ void __launch_bounds__(kPcgThreads) pcg_kernel(PcgArgs<R> A) {
  __shared__ double wsm[kPcgWarps * 8];
  __shared__ double tot[8];
  __shared__ double long_part[6 * kPcgWarps];
  for (int jb = A.cta_job0[blockIdx.x]; jb < A.cta_job0[blockIdx.x + 1]; ++jb) {
    const PcgJob J = A.jobs[jb];
    if (!A.active[J.model]) continue;
    if (!pcg_job<R>(A, J, wsm, tot, long_part)) return;
  }
}

}  // namespace ba
