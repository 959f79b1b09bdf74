// Block-Jacobi preconditioned conjugate gradients on the reduced camera
// system (ba.rs:155-196), as one persistent cooperative kernel.
//
// Each model's block rows are split over a group of CTAs and, inside a CTA,
// over its warps: a warp owns whole block rows.  The reference's iteration
//     q = S p;  a = rz / p·q;  x += a p;  r -= a q;  stop if r·r < tol b·b;
//     z = M r;  β = r·z / rz;  p = z + β p
// needs three group-wide exchanges (p, p·q, r·r and r·z).  Here p is never
// exchanged: every warp forms p_j = z_j + β p_j(prev) on the fly for the
// columns its rows touch (z and the previous p are double-buffered in global
// memory and visible after the previous exchange), so an iteration costs two
// group barriers.
//
// A CTA keeps its rows' state (x, r, z, p, q and the 6x6 block-Jacobi
// inverse) in shared memory for the whole solve, and its S blocks too when
// they fit; only the gathered neighbour z / p come from L2 each iteration.
//
// The lens block row of a model couples to every camera, so it is not
// multiplied by one warp: every camera row c adds S_cg^T p_c to a lens
// partial that travels with the p·q partial sums (S is symmetric).
//
// FP64 instructions on this GPU cost ~64 cycles per SM sub-partition whatever
// the number of active lanes, so row vectors live one component per lane and
// reductions pack several values per instruction.
//
// Inner products are FP64 and summed in a fixed order (fixed lane trees, CTA
// partials in rank order), so every CTA of a group sees bit-identical scalars
// and results do not depend on timing.  Models never wait on each other.
#pragma once

#include "lm_kernels.cuh"

namespace ba {

constexpr int kPcgThreads = 256;
constexpr int kPcgWarps = kPcgThreads / 32;

struct PcgJob {
  int32_t model, rank, gsize, base;  // base: first CTA of the group
  uint32_t row0, row1;               // this CTA's block rows
};

template <typename R>
struct PcgArgs {
  const PcgJob* jobs;
  const int32_t* cta_job0;  // [ncta+1]
  unsigned long long* bar;       // [nm] arrival counter of each model's group
  unsigned long long* bar_base;  // [nm] counter value when the next launch starts
  double* part;                  // [kParts][ncta] partial sums
  int32_t ncta;
  const uint32_t* row_ptr;
  const uint32_t* col_idx;
  const R* S;
  const R* pre;  // block-Jacobi inverses, computed in FP64, stored in R
  const R* b;
  R* x;
  R* z;   // [nb][6] z = M r, gathered by neighbours
  R* p2;  // [2][nb][6] double-buffered search direction
  int64_t nb;
  const int32_t* lens_row;  // [nm]: the model's single lens block row, or -1
  const int32_t* lens_pos;  // [nb]: block index of (row, lens row), or -1
  const uint32_t* diag_pos; // [nb]: block index of the diagonal block
  uint32_t smem_rows;       // row-state capacity of the dynamic shared memory
  uint32_t smem_blocks;     // S blocks cached per CTA (the rest read from global)
  const int32_t* active;
  int32_t* iters;
  int32_t max_iter;
  double tol;
  unsigned* err;
  long long spin;    // spin limit of a group wait, in SM clock cycles
  int32_t hold_cta;  // fault injection: CTA hold_cta - 1 leaves before its first exchange (0: off)
  const int32_t* cap = nullptr;  // [nm] or null: per-model iteration cap (below max_iter)
};

// Partial-sum slots.  Grid kernel: 0,1 init (rz, bb) | 2..5 (pq, lens q
// 0..2) | 6,7 (rr, rz).  Matrix-free kernel adds 8 (barrier) and 9..11 (lens
// terms).  Consecutive exchanges must use disjoint slots: a CTA may still be
// reading one exchange's partials while a faster one writes the next.
constexpr int kParts = 12;
// A reader lane loads up to kReadUnroll members' partials at once.
constexpr int kReadUnroll = 4;
constexpr int kMaxGroupCtas = 32 * kReadUnroll * 4;

// Row state per local row in shared memory: x, r, z, p, q (6 each), M (36),
// padded to a multiple of 16 bytes in both precisions.
constexpr int kRowState = 68;

// Dynamic shared memory: row state, cached S blocks, their columns, and per
// row its block range and lens block (3 words).
template <typename R>
constexpr size_t pcg_smem_bytes(uint32_t rows, uint32_t blocks) {
  return (size_t)rows * kRowState * sizeof(R) + (size_t)blocks * (36 * sizeof(R) + 4) +
         (size_t)rows * 12;
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_add_release_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
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

// Sum over lanes 0..7 (lanes >= 8 must hold 0): result in lanes 0..7.
__device__ __forceinline__ double sum8(double v) {
  v += __shfl_xor_sync(kFull, v, 1);
  v += __shfl_xor_sync(kFull, v, 2);
  v += __shfl_xor_sync(kFull, v, 4);
  return v;
}

// N (<= 4) values per warp (held by lane 0) summed over the CTA's warps with
// one shuffle tree, then over the group's CTAs in rank order; every thread
// receives the totals in tot[].
//
// Group barrier: every member adds 1 to the group's monotonic 64-bit counter
// (release) after publishing its partials, and waits (acquire) until the
// counter reaches `target`, which grows by the group size per exchange from
// the launch's base value.  Only warp 0 of a CTA takes part; the partials are
// then read with all loads in flight at once.  Bounded: after A.spin cycles
// the waiter sets ERR_BARRIER_TIMEOUT; every CTA leaves at its next exchange.
// Args: any type with part, ncta, bar, err and spin as in PcgArgs.
template <int N, typename Args, typename Post>
__device__ __forceinline__ bool group_reduce(const double (&wv)[N], double* wsm, double* tot,
                                             const Args& A, const PcgJob& J, int slot,
                                             unsigned long long& target, Post&& post) {
  __shared__ int ok_s;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < 4; ++i) wsm[warp * 4 + i] = i < N ? wv[i < N ? i : 0] : 0.0;
  __syncthreads();
  if (warp == 0) {
    // lane = 4 w + i: warp w, value i; sum over w in a fixed tree.
    double c = wsm[lane];
    c += __shfl_xor_sync(kFull, c, 4);
    c += __shfl_xor_sync(kFull, c, 8);
    c += __shfl_xor_sync(kFull, c, 16);
    if (J.gsize == 1) {
      if (lane < N) tot[lane] = c;
      __syncwarp();
      if (lane == 0) {
        ok_s = 1;
        post();  // the iteration's scalars, once per CTA
      }
    } else {
      if (lane < N) A.part[(size_t)(slot + lane) * A.ncta + J.base + J.rank] = c;
      __threadfence();
      __syncwarp();
      int ok = 1;
      if (lane == 0) {
        target += (unsigned long long)J.gsize;
        unsigned long long* ctr = A.bar + J.model;
        red_add_release_u64(ctr, 1ULL);
        const long long t0 = clock64();
        while (ld_acquire_u64(ctr) < target) {
          if ((*(volatile unsigned*)A.err) & ERR_BARRIER_TIMEOUT) {
            ok = 0;
            break;
          }
          if (clock64() - t0 > A.spin) {
            atomicOr(A.err, ERR_BARRIER_TIMEOUT);
            ok = 0;
            break;
          }
        }
        ok_s = ok;
      }
      __syncwarp();
      double v[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      for (int k0 = 0; k0 < J.gsize; k0 += 32 * kReadUnroll) {
        double t[4][kReadUnroll];
#pragma unroll
        for (int u = 0; u < kReadUnroll; ++u) {
          const int k = k0 + lane + 32 * u;
#pragma unroll
          for (int i = 0; i < 4; ++i)
            t[i][u] = (i < N && k < J.gsize)
                          ? __ldcg(A.part + (size_t)(slot + i) * A.ncta + J.base + k)
                          : 0.0;
        }
#pragma unroll
        for (int u = 0; u < kReadUnroll; ++u)
#pragma unroll
          for (int i = 0; i < 4; ++i) v[i] += t[i][u];
      }
      warp_sum8(v);  // lane 4i holds value i
      if ((lane & 3) == 0 && (lane >> 2) < N) tot[lane >> 2] = v[0];
      __syncwarp();
      if (lane == 0) post();  // the iteration's scalars, once per CTA
    }
  }
  __syncthreads();
  return ok_s != 0;
}

// Scalars of an iteration, computed once per CTA by thread 0 (FP64 division
// and conversions would otherwise run on every warp's FP64 pipe).
template <typename R>
struct PcgScalars {
  double rz, b2, beta, a;
  R beta_r, a_r;  // beta and a in storage precision
  int stop;
};

// A 6x6 block into registers with 16-byte loads (global or shared).
template <typename A>
__device__ __forceinline__ void load_block(const double* blk, A* m) {
  const double2* v = reinterpret_cast<const double2*>(blk);
#pragma unroll
  for (int i = 0; i < 18; ++i) {
    const double2 t = v[i];
    m[2 * i] = (A)t.x, m[2 * i + 1] = (A)t.y;
  }
}
template <typename A>
__device__ __forceinline__ void load_block(const float* blk, A* m) {
  const float4* v = reinterpret_cast<const float4*>(blk);
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const float4 t = v[i];
    m[4 * i] = (A)t.x, m[4 * i + 1] = (A)t.y, m[4 * i + 2] = (A)t.z, m[4 * i + 3] = (A)t.w;
  }
}

// p_j = z_j + β p_j(prev), the reference's update (ba.rs:192), in storage
// precision; the same expression for own rows and for gathered columns.
template <typename R>
__device__ __forceinline__ R p_of(R zj, R pj, R beta_r) {
  return (R)(zj + pj * beta_r);
}

template <typename R>
__device__ bool pcg_job(const PcgArgs<R>& A, const PcgJob& J, double* wsm, double* tot,
                        PcgScalars<R>& sc, R* rs) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nrows = J.row1 - J.row0;
  const uint32_t B0 = A.row_ptr[J.row0];
  const uint32_t nblk = A.row_ptr[J.row1] - B0;
  if (nrows > A.smem_rows) {  // the planner never does this; fail loudly
    if (threadIdx.x == 0) atomicOr(A.err, ERR_STRUCTURE);
    return false;
  }
  // The first ncached blocks of the CTA's rows (camera rows come first; the
  // lens row, last, uses only its diagonal block) live in shared memory.
  const uint32_t ncached = nblk < A.smem_blocks ? nblk : A.smem_blocks;
  // Barrier counter value at this launch's start (written by the previous
  // launch's rank 0: every member made the same number of arrivals).
  unsigned long long target = A.bar_base[J.model];
  // Shared-memory carve-up: row state, then cached S blocks and columns.
  R* sS = rs + (size_t)A.smem_rows * kRowState;
  uint32_t* sC = reinterpret_cast<uint32_t*>(sS + (size_t)A.smem_blocks * 36);
  int32_t* sM = reinterpret_cast<int32_t*>(sC + A.smem_blocks);
  const int32_t lens = A.lens_row[J.model];  // -1: no transposed lens row
  {
    const uint32_t chunks = ncached * (uint32_t)(36 * sizeof(R) / 16);
    const float4* src = reinterpret_cast<const float4*>(A.S + (size_t)B0 * 36);
    float4* dst = reinterpret_cast<float4*>(sS);
    for (uint32_t c = threadIdx.x; c < chunks; c += blockDim.x) dst[c] = src[c];
    for (uint32_t t = threadIdx.x; t < ncached; t += blockDim.x) sC[t] = A.col_idx[B0 + t];
    // Per row: its block range (the lens row: only its diagonal block; its
    // camera columns arrive through the camera rows' transposed terms) and
    // the position of its lens block.
    for (uint32_t lr = threadIdx.x; lr < nrows; lr += blockDim.x) {
      const uint32_t row = J.row0 + lr;
      uint32_t b0 = A.row_ptr[row], b1 = A.row_ptr[row + 1];
      if ((int32_t)row == lens) b0 = A.diag_pos[row], b1 = b0 + 1;
      sM[3 * lr] = (int32_t)b0;
      sM[3 * lr + 1] = (int32_t)b1;
      sM[3 * lr + 2] = (int32_t)row == lens ? -1 : A.lens_pos[row];
    }
  }
  for (uint32_t t = threadIdx.x; t < nrows * 36; t += blockDim.x)
    rs[(t / 36) * kRowState + 30 + (t % 36)] = A.pre[36 * (size_t)J.row0 + t];
  __syncthreads();
  const bool vl = lane < 6;
  const int ci = vl ? lane : 0;
  // row state: x 0..5 | r 6..11 | z 12..17 | p 18..23 | q 24..29 | M 30..65
#define ROW(lr) (rs + (size_t)(lr) * kRowState)

  // x = 0, r = b, z = M r, p(prev) = 0 (ba.rs:164-168; β = 0 gives p = z)
  double w2[2] = {0.0, 0.0};
  for (uint32_t lr = warp; lr < nrows; lr += kPcgWarps) {
    const uint32_t row = J.row0 + lr;
    R* st = ROW(lr);
    const R ri = vl ? A.b[6 * (size_t)row + ci] : (R)0;
    R zi = (R)0;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const R rj = __shfl_sync(kFull, ri, j);
      zi += st[30 + 6 * ci + j] * rj;
    }
    double a = 0.0, bb = 0.0;
    if (vl) {
      st[ci] = (R)0;
      st[6 + ci] = ri;
      st[12 + ci] = zi;
      st[18 + ci] = (R)0;
      A.z[6 * (size_t)row + ci] = zi;
      A.p2[(size_t)6 * A.nb + 6 * (size_t)row + ci] = (R)0;
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
    return false;
  int32_t spmv = 0;
  const int32_t max_it = A.cap ? min(A.max_iter, A.cap[J.model]) : A.max_iter;
  for (int32_t it = 0; it < max_it; ++it) {
    R* pcur = A.p2 + (size_t)(it & 1) * 6 * A.nb;
    const R* pprev = A.p2 + (size_t)((it + 1) & 1) * 6 * A.nb;
    const R beta = sc.beta_r;
    // q = S p (ba.rs:144-152) for the warp's rows.
    double w4[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint32_t lr = warp; lr < nrows; lr += kPcgWarps) {
      const uint32_t row = J.row0 + lr;
      R* st = ROW(lr);
      const uint32_t b0 = (uint32_t)sM[3 * lr], b1 = (uint32_t)sM[3 * lr + 1];
      R acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (uint32_t k = b0 + lane; k < b1; k += 32) {
        const uint32_t kk = k - B0;
        const bool in_smem = kk < ncached;
        const uint32_t col = in_smem ? sC[kk] : A.col_idx[k];
        R m[36], pp[6];
        load_block(in_smem ? sS + (size_t)kk * 36 : A.S + (size_t)k * 36, m);
        const R* zv = A.z + 6 * (size_t)col;
        const R* pv = pprev + 6 * (size_t)col;
#pragma unroll
        for (int j = 0; j < 6; ++j) pp[j] = p_of<R>(__ldcg(zv + j), __ldcg(pv + j), beta);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          R s = acc[i];
#pragma unroll
          for (int j = 0; j < 6; ++j) s += m[6 * i + j] * pp[j];
          acc[i] = s;
        }
      }
      warp_sum8(acc);  // lane 4i holds q_i
      const R qi = __shfl_sync(kFull, acc[0], 4 * ci);
      // own p = z + β p(prev)
      const R pi = p_of<R>(st[12 + ci], st[18 + ci], beta);
      __syncwarp();
      if (vl) {
        st[24 + ci] = qi;
        st[18 + ci] = pi;
        pcur[6 * (size_t)row + ci] = pi;
      }
      w4[0] += sum8(vl ? (double)pi * (double)qi : 0.0);
      // S_cg^T p_c for the lens column: lane 3t + j multiplies S_cg[t][j] p_t.
      const int32_t lp = sM[3 * lr + 2];
      if (lp >= 0) {
        const int t = lane / 3, j = lane - 3 * (lane / 3);
        const R pt = __shfl_sync(kFull, pi, t < 6 ? t : 0);
        R v = (R)0;
        if (lane < 18) {
          const uint32_t kk = (uint32_t)lp - B0;
          const R* blk = kk < ncached ? sS + (size_t)kk * 36 : A.S + (size_t)lp * 36;
          v = blk[6 * t + j] * pt;
        }
        v += __shfl_down_sync(kFull, v, 3);
        v += __shfl_down_sync(kFull, v, 6);
        v += __shfl_down_sync(kFull, v, 12);
        // lanes 0, 1, 2 hold the three components; every lane adds the same
        w4[1] += (double)__shfl_sync(kFull, v, 0);
        w4[2] += (double)__shfl_sync(kFull, v, 1);
        w4[3] += (double)__shfl_sync(kFull, v, 2);
      }
    }
    const bool lens_here = lens >= 0 && (uint32_t)lens >= J.row0 && (uint32_t)lens < J.row1;
    if (!group_reduce<4>(w4, wsm, tot, A, J, 2, target, [&] {
          double pq = tot[0];
          if (lens >= 0) {
            // The lens row's q: its diagonal product plus the transposed
            // partials; its share of p·q: p_g · (Σ S_cg^T p_c).
            const R* zg = A.z + 6 * (size_t)lens;
            const R* pg = pprev + 6 * (size_t)lens;
            pq += (double)p_of<R>(__ldcg(zg + 0), __ldcg(pg + 0), beta) * tot[1] +
                  (double)p_of<R>(__ldcg(zg + 1), __ldcg(pg + 1), beta) * tot[2] +
                  (double)p_of<R>(__ldcg(zg + 2), __ldcg(pg + 2), beta) * tot[3];
            if (lens_here) {
              R* q = ROW((uint32_t)lens - J.row0) + 24;
              for (int c = 0; c < 3; ++c) q[c] = (R)((double)q[c] + tot[1 + c]);
            }
          }
          sc.stop = fabs(pq) < 1e-300 ? 1 : 0;  // ba.rs:174
          sc.a = sc.stop ? 0.0 : sc.rz / pq;
          sc.a_r = (R)sc.a;
        }))
      return false;
    ++spmv;
    if (sc.stop) break;
    const R a = sc.a_r;
    // x += a p, r -= a q, z = M r (ba.rs:178-188), one component per lane.
    double w2b[2] = {0.0, 0.0};
    for (uint32_t lr = warp; lr < nrows; lr += kPcgWarps) {
      const uint32_t row = J.row0 + lr;
      R* st = ROW(lr);
      R ri = (R)0;
      if (vl) {
        st[ci] = st[ci] + st[18 + ci] * a;
        ri = st[6 + ci] - st[24 + ci] * a;
        st[6 + ci] = ri;
      }
      R zi = (R)0;
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        const R rj = __shfl_sync(kFull, ri, j);
        zi += st[30 + 6 * ci + j] * rj;
      }
      double rr = 0.0, rzl = 0.0;
      if (vl) {
        st[12 + ci] = zi;
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
      return false;
    if (sc.stop) break;
  }
  for (uint32_t lr = warp; lr < nrows; lr += kPcgWarps)
    if (vl) A.x[6 * (size_t)(J.row0 + lr) + ci] = ROW(lr)[ci];
#undef ROW
  if (J.rank == 0 && threadIdx.x == 0) {
    A.iters[J.model] = spmv;
    A.bar_base[J.model] = target;  // every member made the same arrivals
  }
  __syncthreads();
  return true;
}

template <typename R>
__global__ void __launch_bounds__(kPcgThreads) pcg_kernel(PcgArgs<R> A) {
  __shared__ double wsm[kPcgWarps * 4];
  __shared__ double tot[4];
  __shared__ PcgScalars<R> sc;
  extern __shared__ __align__(16) unsigned char pcg_smem[];
  R* rs = reinterpret_cast<R*>(pcg_smem);
  // Fault injection (tests of the timeout path): this CTA never arrives, so
  // the other members of its group give up after A.spin cycles.
  if (A.hold_cta > 0 && (int32_t)blockIdx.x == A.hold_cta - 1) return;
  for (int jb = A.cta_job0[blockIdx.x]; jb < A.cta_job0[blockIdx.x + 1]; ++jb) {
    const PcgJob J = A.jobs[jb];
    if (!A.active[J.model]) continue;
    if (!pcg_job<R>(A, J, wsm, tot, sc, rs)) return;
  }
}

// lens_pos[row] = index of the block (row, lens row of its model), or -1.
__global__ static void lens_pos_kernel(int64_t nb, const uint32_t* row_ptr,
                                       const uint32_t* col_idx, const uint32_t* blk_model,
                                       const int32_t* lens_row, int32_t* lens_pos) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nb) return;
  const int32_t L = lens_row[blk_model[r]];
  int32_t pos = -1;
  if (L >= 0 && L != (int32_t)r)
    for (uint32_t k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
      if ((int32_t)col_idx[k] == L) {
        pos = (int32_t)k;
        break;
      }
  lens_pos[r] = pos;
}

}  // namespace ba
