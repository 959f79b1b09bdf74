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
// barriers.  The arithmetic of the recurrence is the reference's; inner
// products are FP64 and summed in a fixed order (CTA partials in rank order,
// then a fixed warp tree), so every CTA of a group sees bit-identical scalars
// and results do not depend on timing.  Models never wait on each other.
#pragma once

#include "lm_kernels.cuh"

namespace ba {

constexpr int kPcgThreads = 256;
constexpr uint32_t kLongRow = 64;  // blocks; longer rows use every warp of the CTA

struct PcgJob {
  int32_t model, rank, gsize, base;  // base: first CTA of the group
  uint32_t row0, row1;               // this CTA's block rows
};

template <typename R>
struct PcgArgs {
  const PcgJob* jobs;
  const int32_t* cta_job0;  // [ncta+1]
  unsigned long long* bar;  // [nm] arrival counters
  double* part;             // [5][ncta]: rz0, bb | pq | rr, rz
  int32_t ncta;
  const uint32_t* row_ptr;
  const uint32_t* col_idx;
  const R* S;
  const double* pre;
  const R* b;
  R *x, *r, *z, *q;
  R* p2;  // [2][nb][6] double-buffered search direction
  int64_t nb;
  const int32_t* active;
  int32_t* iters;
  int32_t max_iter;
  double tol;
  unsigned* err;
};

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

// Sum N per-thread values over the CTA, then over the group's CTAs in rank
// order; every thread receives the totals.
template <int N, typename R>
__device__ __forceinline__ bool pcg_reduce(double (&v)[N], double* scratch, double* tot,
                                           const PcgArgs<R>& A, const PcgJob& J, int slot) {
  block_sum<N>(v, scratch);
  if (J.gsize > 1) {
    if (threadIdx.x == 0)
#pragma unroll
      for (int i = 0; i < N; ++i) A.part[(size_t)(slot + i) * A.ncta + J.base + J.rank] = v[i];
    if (!counter_sync(A.bar + J.model, (unsigned)J.gsize, A.err)) return false;
    // Warp 0 reads the group's partials in parallel and sums them with a
    // fixed tree, so every CTA of the group gets bit-identical totals.
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const double* src = A.part + (size_t)(slot + i) * A.ncta + J.base;
        double s = 0.0;
        for (int k = lane; k < J.gsize; k += 32) s += __ldcg(src + k);
        s = warp_sum(s);
        if (lane == 0) tot[i] = s;
      }
    }
  } else if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < N; ++i) tot[i] = v[i];
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = tot[i];
  __syncthreads();
  return true;
}

__device__ __forceinline__ void apply_pre(const double* M, const double* rv, double* zv) {
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double a = 0.0;
#pragma unroll
    for (int j = 0; j < 6; ++j) a += M[6 * i + j] * rv[j];
    zv[i] = a;
  }
}

// A 6x6 block into registers with 16-byte loads.
__device__ __forceinline__ void load_block(const double* blk, double* m) {
  const double2* v = reinterpret_cast<const double2*>(blk);
#pragma unroll
  for (int i = 0; i < 18; ++i) {
    const double2 t = __ldg(v + i);
    m[2 * i] = t.x, m[2 * i + 1] = t.y;
  }
}
__device__ __forceinline__ void load_block(const float* blk, double* m) {
  const float4* v = reinterpret_cast<const float4*>(blk);
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const float4 t = __ldg(v + i);
    m[4 * i] = t.x, m[4 * i + 1] = t.y, m[4 * i + 2] = t.z, m[4 * i + 3] = t.w;
  }
}

// p_j = z_j + β p_j(prev), the reference's update (ba.rs:192), in storage
// precision; the same expression for own rows and for gathered columns.
template <typename R>
__device__ __forceinline__ R p_of(R zj, R pj, double beta) {
  return (R)((double)zj + (double)pj * beta);
}

template <typename R>
__device__ __forceinline__ void gather_p(const PcgArgs<R>& A, const R* pprev, uint32_t col,
                                         double beta, double* pp) {
  const R* zv = A.z + 6 * (size_t)col;
  const R* pv = pprev + 6 * (size_t)col;
#pragma unroll
  for (int j = 0; j < 6; ++j) pp[j] = (double)p_of<R>(__ldcg(zv + j), __ldcg(pv + j), beta);
}

template <typename R>
__device__ bool pcg_job(const PcgArgs<R>& A, const PcgJob& J, double* scratch, double* tot,
                        double* long_part) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // x = 0, r = b, z = M r, p(prev) = 0 (ba.rs:164-168; β = 0 gives p = z)
  double v2[2] = {0.0, 0.0};
  for (uint32_t row = J.row0 + threadIdx.x; row < J.row1; row += blockDim.x) {
    double rv[6], zv[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      rv[i] = (double)A.b[6 * (size_t)row + i];
      A.x[6 * (size_t)row + i] = (R)0;
      A.r[6 * (size_t)row + i] = (R)rv[i];
      A.p2[(size_t)6 * A.nb + 6 * (size_t)row + i] = (R)0;
    }
    apply_pre(A.pre + 36 * (size_t)row, rv, zv);
    double rz = 0.0, bb = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const R zr = (R)zv[i];
      A.z[6 * (size_t)row + i] = zr;
      rz += rv[i] * (double)zr;
      bb += rv[i] * rv[i];
    }
    v2[0] += rz;
    v2[1] += bb;
  }
  if (!pcg_reduce<2>(v2, scratch, tot, A, J, 0)) return false;
  double rz = v2[0];
  const double b2 = fmax(v2[1], 1e-300);
  double beta = 0.0;
  int32_t spmv = 0;
  for (int32_t it = 0; it < A.max_iter; ++it) {
    R* pcur = A.p2 + (size_t)(it & 1) * 6 * A.nb;
    const R* pprev = A.p2 + (size_t)((it + 1) & 1) * 6 * A.nb;
    // own rows: p = z + β p(prev)
    for (uint32_t row = J.row0 + threadIdx.x; row < J.row1; row += blockDim.x)
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        const size_t o = 6 * (size_t)row + i;
        pcur[o] = p_of<R>(A.z[o], pprev[o], beta);
      }
    // q = S p (ba.rs:144-152): warp per block row, p gathered on the fly.
    double pq_part = 0.0;
    for (uint32_t row = J.row0 + warp; row < J.row1; row += nw) {
      const uint32_t b0 = A.row_ptr[row], b1 = A.row_ptr[row + 1];
      if (b1 - b0 > kLongRow) continue;
      double acc[6] = {0, 0, 0, 0, 0, 0};
      for (uint32_t k = b0 + lane; k < b1; k += 32) {
        double m[36], pp[6];
        load_block(A.S + (size_t)k * 36, m);
        gather_p<R>(A, pprev, A.col_idx[k], beta, pp);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          double a = 0.0;
#pragma unroll
          for (int j = 0; j < 6; ++j) a += m[6 * i + j] * pp[j];
          acc[i] += a;
        }
      }
#pragma unroll
      for (int i = 0; i < 6; ++i) acc[i] = warp_sum(acc[i]);
      if (lane == 0) {
        double d = 0.0;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          const R qi = (R)acc[i];
          A.q[6 * (size_t)row + i] = qi;
          d += (double)p_of<R>(A.z[6 * (size_t)row + i], pprev[6 * (size_t)row + i], beta) *
               (double)qi;
        }
        pq_part += d;
      }
    }
    // Rows longer than kLongRow (lens rows couple to every camera): all warps.
    for (uint32_t row = J.row0; row < J.row1; ++row) {  // CTA-uniform
      const uint32_t b0 = A.row_ptr[row], b1 = A.row_ptr[row + 1];
      if (b1 - b0 <= kLongRow) continue;
      const uint32_t chunk = (b1 - b0 + nw - 1) / nw;
      const uint32_t k0 = b0 + warp * chunk, k1 = min(b1, k0 + chunk);
      double acc[6] = {0, 0, 0, 0, 0, 0};
      for (uint32_t k = k0 + lane; k < k1; k += 32) {
        double m[36], pp[6];
        load_block(A.S + (size_t)k * 36, m);
        gather_p<R>(A, pprev, A.col_idx[k], beta, pp);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          double a = 0.0;
#pragma unroll
          for (int j = 0; j < 6; ++j) a += m[6 * i + j] * pp[j];
          acc[i] += a;
        }
      }
#pragma unroll
      for (int i = 0; i < 6; ++i) acc[i] = warp_sum(acc[i]);
      if (lane == 0)
#pragma unroll
        for (int i = 0; i < 6; ++i) long_part[6 * warp + i] = acc[i];
      __syncthreads();
      if (threadIdx.x == 0) {
        double d = 0.0;
        for (int i = 0; i < 6; ++i) {
          double s = 0.0;
          for (int w = 0; w < nw; ++w) s += long_part[6 * w + i];
          const R qi = (R)s;
          A.q[6 * (size_t)row + i] = qi;
          d += (double)p_of<R>(A.z[6 * (size_t)row + i], pprev[6 * (size_t)row + i], beta) *
               (double)qi;
        }
        pq_part += d;
      }
      __syncthreads();
    }
    double v1[1] = {pq_part};
    if (!pcg_reduce<1>(v1, scratch, tot, A, J, 2)) return false;
    ++spmv;
    const double pq = v1[0];
    if (fabs(pq) < 1e-300) break;  // ba.rs:174
    const double a = rz / pq;
    // x += a p, r -= a q, z = M r (ba.rs:178-188)
    double v3[2] = {0.0, 0.0};
    for (uint32_t row = J.row0 + threadIdx.x; row < J.row1; row += blockDim.x) {
      double rv[6], zv[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        const size_t o = 6 * (size_t)row + i;
        A.x[o] = (R)((double)A.x[o] + (double)pcur[o] * a);
        rv[i] = (double)(R)((double)A.r[o] - (double)A.q[o] * a);
        A.r[o] = (R)rv[i];
      }
      apply_pre(A.pre + 36 * (size_t)row, rv, zv);
      double rr = 0.0, rzp = 0.0;
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        const R zr = (R)zv[i];
        A.z[6 * (size_t)row + i] = zr;
        rr += rv[i] * rv[i];
        rzp += rv[i] * (double)zr;
      }
      v3[0] += rr;
      v3[1] += rzp;
    }
    if (!pcg_reduce<2>(v3, scratch, tot, A, J, 3)) return false;
    if (v3[0] < A.tol * b2) break;  // ba.rs:182
    beta = v3[1] / rz;               // ba.rs:189-190
    rz = v3[1];
  }
  if (J.rank == 0 && threadIdx.x == 0) A.iters[J.model] = spmv;
  return true;
}

template <typename R>
__global__ void __launch_bounds__(kPcgThreads) pcg_kernel(PcgArgs<R> A) {
  __shared__ double scratch[2 * 32];
  __shared__ double tot[2];
  __shared__ double long_part[6 * (kPcgThreads / 32)];
  for (int jb = A.cta_job0[blockIdx.x]; jb < A.cta_job0[blockIdx.x + 1]; ++jb) {
    const PcgJob J = A.jobs[jb];
    if (!A.active[J.model]) continue;
    if (!pcg_job<R>(A, J, scratch, tot, long_part)) return;
  }
}

}  // namespace ba
