// Block-Jacobi PCG of the reduced camera system (ba.rs:155-196) with one
// thread-block cluster per model and the whole solve in the cluster's
// distributed shared memory: mixed form only (FP32 matrix and vectors,
// double-float inner products).
//
// A model's block rows are split over the CTAs of its cluster (balanced by
// blocks); each CTA keeps its rows' state (x, r, z, two buffers of p, q and
// the block-Jacobi inverse) and its rows' S blocks in shared memory for the
// whole solve.  Every value another CTA needs is pushed to it: a CTA keeps a
// cache of the neighbour rows its blocks multiply (z_j and both buffers of
// p_j), and each row's owner stores the row's new z and p into the caches of
// the CTAs that read it (a host-built subscriber list) before the cluster
// barrier after which they are read.  Remote loads would be round trips a
// warp waits on (~4.5k cycles when its lanes read from 16 CTAs); remote
// stores complete behind the barrier's release.  The two reductions of an
// iteration meet at hardware cluster barriers: no global memory traffic and
// no software spin inside the iteration.  The iteration is the reference's,
// with p_j = z_j + β p_j(prev) formed on the fly as in the grid kernel.
//
// Two-level form (coarse correction z = B^-1 r + W E^-1 W^T r): the coarse
// vector of the next residual, w = W^T r_{k+1}, is formed as W^T r_k −
// α W^T q_k from group sums every CTA publishes before the iteration's first
// barrier (α is known right after it), so an iteration still needs only two
// cluster reductions: p·q (then α, the coarse gather and c = E^-1 w), and
// r·r with r·z (then β).  The coarse step runs on the warps beside warp 0
// after the p·q barrier: each of them sums the inbox and forms α as warp 0
// does (the same sums in the same order, so the same α), then its rows of
// E^-1 w, so the step adds no CTA barrier to the iteration.
//
// Every CTA of a cluster executes the same sequence of cluster barriers:
// loop exits depend only on reduced scalars, which every CTA computes from
// the same partials in the same order (bit-identical), and the kernel has no
// early return after its first barrier.
#pragma once

#include <cooperative_groups.h>

#include "coarse.cuh"
#include "pcg.cuh"

namespace ba {

namespace cgx = cooperative_groups;

// Threads per CTA: 512, or 1024 for a warp per block row where a CTA holds
// about 32 rows (the autotuner picks per problem shape).  The row loops take
// rows warp, warp + warps, ...; the reductions sum the warps' partials in a
// fixed order for either size.
constexpr int kCgThreads = 512;
constexpr int kCgThreadsWide = 1024;
constexpr int kCgMaxCluster = 16;
// Row state in floats: x r z p0 p1 q (6 each) | M (36) | the row's first and
// end block, its lens block, its coarse group slot and its subscriber range
// (int bits) | pad.  Accessed one component per lane.
constexpr int kCgX = 0, kCgR = 6, kCgZ = 12, kCgP = 18, kCgQ = 30, kCgM = 36, kCgIdx = 72;
constexpr int kCgRow = 80;
// A block's column is one of the CTA's own rows when its slot carries this
// bit (the low bits are the local row), else a slot of the neighbour cache.
constexpr uint32_t kCgOwnRow = 0x80000000u;
// Neighbour cache slot in floats: z (8, 6 used) | p buffer 0 (8) | p buffer 1.
constexpr int kCgCache = 24;

struct CgJob {
  int32_t model;
  uint32_t row0, row1;  // this CTA's block rows
};

struct CgArgs {
  const CgJob* jobs;        // [grid]
  const uint32_t* row_loc;  // [nb]: owner rank << 16 | local row index
  const uint32_t* row_ptr;
  const uint32_t* col_idx;
  const float* S;
  const float* pre;
  const float* b;
  float* x;
  const int32_t* lens_row;  // [nm]
  const int32_t* lens_pos;  // [nb]
  const uint32_t* diag_pos; // [nb]
  uint32_t cap_rows;        // row-state capacity (same in every CTA)
  uint32_t cap_blocks;      // cached S blocks per CTA (the rest read from global)
  const int32_t* active;
  int32_t* iters;
  int32_t max_iter;
  double tol;
  // Two-level (coarse) form only: see coarse.cuh.
  const float* W;            // [nb * 42]
  const float* Einv;         // per model, D x D
  const int64_t* model_eoff; // [nm]
  const int32_t* model_g0;   // [nm + 1]
  const int32_t* grp_row0;   // [groups]
  const int32_t* grp_row1;   // [groups]
  const int32_t* job_g0;     // [grid]: this CTA's groups [job_g0, job_g1)
  const int32_t* job_g1;
  const uint32_t* grp_loc;   // [groups]: owner rank << 16 | local group slot
  uint32_t cap_groups;       // group slots per CTA
  uint32_t cap_dim;          // largest model coarse dimension
  // Neighbour caches: the cache slot of every block's column in its row's
  // CTA, and per row the (CTA rank << 16 | slot) entries of the caches that
  // hold it.
  const uint32_t* blk_slot;  // [nz]
  const uint32_t* sub_ptr;   // [nb + 1]
  const uint32_t* sub_ent;
  uint32_t cap_cache;        // cache slots per CTA
  const int32_t* cap = nullptr;  // [nm] or null: per-model iteration cap (below max_iter)
  unsigned* err = nullptr;   // device error bits (a staging wait that gave up)
  long long spin = 0;        // limit of that wait, in SM clock cycles
};

// The CTA's S blocks are one contiguous run of global memory (rows are
// consecutive, blocks row-major): one bulk asynchronous copy (the TMA engine,
// cp.async.bulk) brings them to shared memory while the threads stage the
// rest, completing on an mbarrier.  Both addresses are 16-byte aligned (a
// block is 144 bytes; the run and the shared row state before it are
// multiples of 16 bytes) and the size is a multiple of 16.
__device__ __forceinline__ void cg_bulk_stage(uint64_t* bar, float* dst, const float* src,
                                              uint32_t bytes) {
  const uint32_t b = (uint32_t)__cvta_generic_to_shared(bar);
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(d), "l"(src), "r"(bytes), "r"(b)
      : "memory");
}
// Wait for phase 0 of the staging mbarrier, at most `spin` cycles (<= 0: the
// default 4e9); false if it gave up.
__device__ __forceinline__ bool cg_bulk_wait(uint64_t* bar, long long spin) {
  const uint32_t b = (uint32_t)__cvta_generic_to_shared(bar);
  const long long limit = spin > 0 ? spin : 4000000000LL;
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(b)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > limit) return false;
  }
}

inline size_t cg_smem_bytes(uint32_t cap_rows, uint32_t cap_blocks, uint32_t cap_cache) {
  return (size_t)cap_rows * kCgRow * 4 + (size_t)cap_blocks * (36 * 4 + 4) +
         (size_t)cap_cache * kCgCache * 4;
}

// Extra shared memory of the two-level form, in floats: per row W (42); per
// own group its rows of E^-1 (7 x D) and c (7); the model's group sums of
// W^T r (two buffers by iteration parity: owners push the next one while the
// current one is read) and of W^T q (D each), pushed by every group's owner.
constexpr int kCgCoarseRowF = 42;
__host__ __device__ constexpr size_t cg_coarse_fixed_floats(uint32_t cap_groups,
                                                            uint32_t cap_dim) {
  return (size_t)cap_groups * (kCoarseModes * cap_dim + kCoarseModes) + 3 * (size_t)cap_dim;
}
inline size_t cg_coarse_smem_bytes(uint32_t cap_rows, uint32_t cap_groups, uint32_t cap_dim) {
  return ((size_t)cap_rows * kCgCoarseRowF + cg_coarse_fixed_floats(cap_groups, cap_dim)) * 4;
}

// Sum over lanes 0..7 (lanes >= 8 hold 0); lanes 0..7 receive it.
__device__ __forceinline__ float cg_sum8f(float v) {
  v += __shfl_xor_sync(kFull, v, 1);
  v += __shfl_xor_sync(kFull, v, 2);
  v += __shfl_xor_sync(kFull, v, 4);
  return v;
}

// Double-float numbers: hi + lo with |lo| <= ulp(hi) / 2, about 48 bits from
// FP32 instructions (on this GPU an FP64 warp instruction occupies its SM
// sub-partition for ~64 cycles).
struct DFloat {
  float hi, lo;
};
// Sum of two double-floats (Knuth's two-sum of the high parts, the low parts
// added to the error, renormalised).
__device__ __forceinline__ DFloat df_sum(DFloat a, DFloat b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = ((a.hi - (s - bb)) + (b.hi - bb)) + (a.lo + b.lo);
  const float hi = s + e;
  return DFloat{hi, e - (hi - s)};
}
// x y for FP32 x and a double-float y: the exact product x y.hi (split by an
// FMA) plus x y.lo.
__device__ __forceinline__ DFloat df_scale(float x, DFloat y) {
  const float p = x * y.hi;
  const float e = fmaf(x, y.hi, -p) + x * y.lo;
  const float hi = p + e;
  return DFloat{hi, e - (hi - p)};
}
__device__ __forceinline__ DFloat df_shfl_xor(DFloat v, int o) {
  return DFloat{__shfl_xor_sync(kFull, v.hi, o), __shfl_xor_sync(kFull, v.lo, o)};
}

// The cluster's totals from an inbox: lane r < cluster size (<= 16) holds CTA
// r's values, lanes 16..31 hold zeros, and a butterfly within each half-warp
// leaves the totals in lanes 0..15.
template <int N>
__device__ __forceinline__ void cg_inbox_sum(const DFloat (*inbox)[4], int csize, int lane,
                                             DFloat (&v)[N]) {
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = lane < csize ? inbox[lane][i] : DFloat{0.0f, 0.0f};
#pragma unroll
  for (int o = 8; o > 0; o >>= 1)
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = df_sum(v[i], df_shfl_xor(v[i], o));
}

// Inner products: a warp sums its rows' products in FP32 (a few rows of six
// components); the warps' partials are summed as double-floats over the CTA
// and then over the cluster's CTAs, in a fixed order, by warp 0.  wv: N
// (<= 4) values held by lane 0 of every warp; all threads receive the totals
// in tot (shared memory).  Every CTA sums the same partials in the same
// order, so every CTA sees bit-identical totals.  While warp 0 sums and
// pushes the CTA's partials, warps 1.. run side(w) with w = warp - 1 (the
// coarse group sums, which read the same row state after the same CTA
// barrier); while warp 0 sums the inbox after the cluster barrier, they run
// after(w) (coarse work that reads what the barrier published).
//
// Exchange by push: before the cluster barrier, lane r of warp 0 stores the
// CTA's partials into CTA r's inbox (inbox[source rank][value]); after it,
// every CTA reads its own inbox.  A warp that loads from many CTAs waits on
// each remote round trip (measured: ~4.5k cycles for one load per CTA of a
// 16-CTA cluster), while remote stores complete behind the barrier's
// release.  Consecutive reductions use different inboxes: a CTA can only
// write inbox n + 2 after the barrier of reduction n + 1, which every reader
// of inbox n has passed.
template <int kWarps, int N, typename Side, typename Post, typename After>
__device__ __forceinline__ void cg_reduce(cgx::cluster_group& cl, const float (&wv)[N],
                                          float* wsm, DFloat (*inbox)[4], DFloat* tot,
                                          Side&& side, Post&& post, After&& after) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < 4; ++i) wsm[warp * 4 + i] = i < N ? wv[i < N ? i : 0] : 0.0f;
  __syncthreads();
  const int csize = (int)cl.num_blocks();
  if (warp == 0) {
    // lane = 4 w + i: warps w, w + 8, ... (value i) in order, then over w in
    // a fixed tree
    static_assert(kWarps % 8 == 0 && kWarps >= 16 && kWarps <= 32, "2-4 warp partials per lane");
    DFloat c = df_sum(DFloat{wsm[lane], 0.0f}, DFloat{wsm[32 + lane], 0.0f});
#pragma unroll
    for (int h = 2; h < kWarps / 8; ++h) c = df_sum(c, DFloat{wsm[32 * h + lane], 0.0f});
    c = df_sum(c, df_shfl_xor(c, 4));
    c = df_sum(c, df_shfl_xor(c, 8));
    c = df_sum(c, df_shfl_xor(c, 16));
    DFloat v[N];
#pragma unroll
    for (int i = 0; i < N; ++i)
      v[i] = DFloat{__shfl_sync(kFull, c.hi, i), __shfl_sync(kFull, c.lo, i)};
    if (lane < csize) {
      DFloat* dst = cl.map_shared_rank(&inbox[0][0], (unsigned)lane) + 4 * cl.block_rank();
#pragma unroll
      for (int i = 0; i < N; ++i) dst[i] = v[i];
    }
  } else {
    side(warp - 1);
  }
  cl.sync();
  if (warp == 0) {
    DFloat v[N];
    cg_inbox_sum<N>(inbox, csize, lane, v);
    if (lane == 0) {
#pragma unroll
      for (int i = 0; i < N; ++i) tot[i] = v[i];
      post();  // the iteration's scalars, once per CTA
    }
  } else {
    after(warp - 1);
  }
  __syncthreads();
}

// Scalars of the iteration, computed by thread 0 and read by every thread:
// r.z as a double-float, b.b, α and β in FP32 (the precision of the vectors
// they scale).
struct CgScalars {
  DFloat rz;
  float b2, af, bf;
  int stop;
};

// One output of the coarse step: sc[o] = (E^-1 w)_o for this CTA's (group,
// mode) output o, with the model's w = W^T r − α W^T q (wq null at the
// start: w = W^T b); a warp, then a fixed butterfly.
__device__ __forceinline__ void cg_coarse_dot(const float* sEi, uint32_t cap_dim, int D, int o,
                                              const float* wr, const float* wq, float alpha,
                                              float* sc) {
  const int lane = threadIdx.x & 31;
  const float* er = sEi + (size_t)o * cap_dim;
  float v = 0.0f;
  if (wq)
    for (int t = lane; t < D; t += 32) v += er[t] * (wr[t] - alpha * wq[t]);
  else
    for (int t = lane; t < D; t += 32) v += er[t] * wr[t];
#pragma unroll
  for (int q = 16; q > 0; q >>= 1) v += __shfl_xor_sync(kFull, v, q);
  if (lane == 0) sc[o] = v;
}

// The iteration's α as the p.q reduction's post forms it (the same sums in
// the same order, so the same value), in every lane of the calling warp:
// p.q from inbox 0 plus the lens row's share, α = r.z / p.q (0 where p.q
// vanishes).
__device__ __forceinline__ float cg_alpha(const DFloat (*inbox)[4], int csize, int lane,
                                          int32_t lens, const float* lens_p, float rz) {
  DFloat v[4];
  cg_inbox_sum<4>(inbox, csize, lane, v);
  DFloat t[4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
    t[i] = DFloat{__shfl_sync(kFull, v[i].hi, 0), __shfl_sync(kFull, v[i].lo, 0)};
  DFloat pq = t[0];
  if (lens >= 0)
#pragma unroll
    for (int c = 0; c < 3; ++c) pq = df_sum(pq, df_scale(lens_p[c], t[1 + c]));
  return fabsf(pq.hi) < 1.17549435e-38f ? 0.0f : rz / pq.hi;
}

// A row's coarse share of z, (W c)_i for lane i < 6 (rows outside every
// group, such as the lens row, add nothing).
__device__ __forceinline__ float cg_row_wc(const float* sWrow, int32_t lg, const float* sc,
                                           int ci) {
  if (lg < 0) return 0.0f;
  const float* w = sWrow + kCoarseModes * ci;
  const float* c = sc + kCoarseModes * lg;
  float add = 0.0f;
#pragma unroll
  for (int j = 0; j < kCoarseModes; ++j) add += w[j] * c[j];
  return add;
}

// Per own group: the sum over its rows of W^T x, x the row-state vector at
// float offset `xoff`, pushed into the model-wide array `dst` (D floats, at
// this CTA's groups' offset) of every CTA.  A warp per (group, mode), warp
// `w` of kWorkers taking (group, mode) w, w + kWorkers, ...: lane l takes
// rows l, l + 32, ... (each row's six products in component order), then a
// fixed butterfly.
__device__ __forceinline__ void cg_group_sum_push(cgx::cluster_group& cl, int o,
                                                  const int32_t* grp_row0,
                                                  const int32_t* grp_row1, int32_t g0,
                                                  int32_t goff, uint32_t row0, const float* sW,
                                                  const float* rs, int xoff, float* dst) {
  const int lane = threadIdx.x & 31;
  const int csize = (int)cl.num_blocks();
  const int l = o / kCoarseModes, j = o % kCoarseModes;
  float v = 0.0f;
  for (int32_t r = grp_row0[g0 + l] + lane; r < grp_row1[g0 + l]; r += 32) {
    const float* w = sW + (size_t)(r - row0) * 42 + j;
    const float* x = rs + (size_t)(r - row0) * kCgRow + xoff;
#pragma unroll
    for (int i = 0; i < 6; ++i) v += w[kCoarseModes * i] * x[i];
  }
#pragma unroll
  for (int q = 16; q > 0; q >>= 1) v += __shfl_xor_sync(kFull, v, q);
  if (lane < csize) cl.map_shared_rank(dst, (unsigned)lane)[goff + o] = v;
}
template <int kWorkers>
__device__ __forceinline__ void cg_group_sums_push(cgx::cluster_group& cl, int w, int32_t ngr,
                                                   const int32_t* grp_row0,
                                                   const int32_t* grp_row1, int32_t g0,
                                                   int32_t goff, uint32_t row0, const float* sW,
                                                   const float* rs, int xoff, float* dst) {
  for (int o = w; o < ngr * kCoarseModes; o += kWorkers)
    cg_group_sum_push(cl, o, grp_row0, grp_row1, g0, goff, row0, sW, rs, xoff, dst);
}

// Push a row's six values (lane i < 6 holds x_i) into the neighbour cache of
// every CTA that reads the row, at float offset `off` of its slot there.
__device__ __forceinline__ void cg_push_row(cgx::cluster_group& cl, float* cache,
                                            const uint32_t* sub_ent, uint32_t s0, uint32_t s1,
                                            float xi, int off) {
  const int lane = threadIdx.x & 31;
  float x[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) x[i] = __shfl_sync(kFull, xi, i);
  for (uint32_t t = s0 + lane; t < s1; t += 32) {
    const uint32_t e = __ldg(sub_ent + t);
    float* dst = cl.map_shared_rank(cache, e >> 16) + (size_t)(e & 0xffffu) * kCgCache + off;
    *reinterpret_cast<float4*>(dst) = make_float4(x[0], x[1], x[2], x[3]);
    *reinterpret_cast<float2*>(dst + 4) = make_float2(x[4], x[5]);
  }
}

template <bool kCoarse, int kThreads>
static __global__ void __launch_bounds__(kThreads) pcg_cluster_kernel(CgArgs A) {
  constexpr int kCgWarps = kThreads / 32;
  __shared__ float wsm[kCgWarps * 4];
  __shared__ DFloat inbox[3][kCgMaxCluster][4];  // reduction inboxes (push)
  __shared__ DFloat tot[4];
  __shared__ float lens_p[4];  // the lens row's p, pushed by its owner
  __shared__ CgScalars sc;
  __shared__ uint64_t stage_bar;  // completion of the S blocks' bulk copy
  extern __shared__ __align__(16) unsigned char cg_smem[];
  cgx::cluster_group cl = cgx::this_cluster();
  const CgJob J = A.jobs[blockIdx.x];
  if (!A.active[J.model]) return;  // uniform over the cluster
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nrows = J.row1 - J.row0;
  const uint32_t B0 = A.row_ptr[J.row0];
  const uint32_t nblk = A.row_ptr[J.row1] - B0;
  const uint32_t ncached = nblk < A.cap_blocks ? nblk : A.cap_blocks;
  // Shared memory: row state | cached S blocks | neighbour cache | cached
  // blocks' cache slots | two-level form: W per row, E^-1 rows and c per own
  // group, the model's group sums of W^T r (two buffers) and W^T q.
  float* rs = reinterpret_cast<float*>(cg_smem);
  float* sS = rs + (size_t)A.cap_rows * kCgRow;
  float* cache = sS + (size_t)A.cap_blocks * 36;
  uint32_t* sL = reinterpret_cast<uint32_t*>(cache + (size_t)A.cap_cache * kCgCache);
  float* sW = reinterpret_cast<float*>(sL + A.cap_blocks);
  float* sEi = sW + (size_t)A.cap_rows * 42;
  const size_t gsz = (size_t)A.cap_groups * kCoarseModes;
  float* scf = sEi + gsz * A.cap_dim;        // c, own outputs
  float* wall_r = scf + gsz;                  // [2][D]
  float* wall_q = wall_r + 2 * (size_t)A.cap_dim;  // [D]
  const int32_t cg0 = kCoarse ? A.job_g0[blockIdx.x] : 0;
  const int32_t ngr = kCoarse ? A.job_g1[blockIdx.x] - cg0 : 0;
  const int32_t goff = kCoarse ? kCoarseModes * (cg0 - A.model_g0[J.model]) : 0;
  const int32_t lens = A.lens_row[J.model];
  // the model's coarse dimension and this CTA's coarse outputs (two-level form)
  const int cD = kCoarse ? kCoarseModes * (A.model_g0[J.model + 1] - A.model_g0[J.model]) : 0;
  const int nco = kCoarseModes * ngr;
  {
    if (threadIdx.x == 0 && ncached > 0)
      cg_bulk_stage(&stage_bar, sS, A.S + (size_t)B0 * 36, ncached * 36u * 4u);
    for (uint32_t t = threadIdx.x; t < ncached; t += blockDim.x) sL[t] = A.blk_slot[B0 + t];
    // p(prev) of iteration 0 is 0 in every cached row; the z values arrive
    // by push after the first cluster barrier.
    for (uint32_t t = threadIdx.x; t < A.cap_cache * kCgCache; t += blockDim.x) cache[t] = 0.0f;
    for (uint32_t t = threadIdx.x; t < nrows * 36; t += blockDim.x)
      rs[(size_t)(t / 36) * kCgRow + kCgM + (t % 36)] = A.pre[36 * (size_t)J.row0 + t];
    // Per row: its block range (the lens row: its diagonal block only; its
    // camera columns arrive through the camera rows' transposed terms) and
    // the position of its lens block.
    for (uint32_t lr = threadIdx.x; lr < nrows; lr += blockDim.x) {
      const uint32_t row = J.row0 + lr;
      float* st = rs + (size_t)lr * kCgRow;
      uint32_t b0 = A.row_ptr[row], b1 = A.row_ptr[row + 1];
      if ((int32_t)row == lens) b0 = A.diag_pos[row], b1 = b0 + 1;
      st[kCgIdx] = __int_as_float((int)b0);
      st[kCgIdx + 1] = __int_as_float((int)b1);
      st[kCgIdx + 2] = __int_as_float((int32_t)row == lens ? -1 : A.lens_pos[row]);
      int32_t lg = -1;  // local group slot (two-level form)
      if constexpr (kCoarse)
        for (int32_t l = 0; l < ngr; ++l)
          if ((int32_t)row >= A.grp_row0[cg0 + l] && (int32_t)row < A.grp_row1[cg0 + l]) lg = l;
      st[kCgIdx + 3] = __int_as_float(lg);
      st[kCgIdx + 4] = __int_as_float((int)A.sub_ptr[row]);
      st[kCgIdx + 5] = __int_as_float((int)A.sub_ptr[row + 1]);
    }
    if constexpr (kCoarse) {
      for (uint32_t t = threadIdx.x; t < nrows * 42; t += blockDim.x)
        sW[t] = A.W[42 * (size_t)J.row0 + t];
      const int32_t gm0 = A.model_g0[J.model];
      const int D = kCoarseModes * (A.model_g0[J.model + 1] - gm0);
      const float* Ei = A.Einv + A.model_eoff[J.model];
      for (int t = threadIdx.x; t < ngr * kCoarseModes * D; t += blockDim.x) {
        const int o = t / D, col = t % D;
        sEi[(size_t)o * A.cap_dim + col] =
            Ei[(size_t)(kCoarseModes * (cg0 - gm0) + o) * D + col];
      }
    }
  }
  // The S blocks' copy has landed: thread 0 waits on the mbarrier (the
  // cluster barrier below then orders the copy before every thread's reads).
  // A wait that gives up records the error; the kernel still runs its
  // barriers to the end, and the call fails.
  if (threadIdx.x == 0 && ncached > 0 && !cg_bulk_wait(&stage_bar, A.spin) && A.err)
    atomicOr(A.err, ERR_BARRIER_TIMEOUT);
  // Every CTA of the cluster has started (its shared memory is live for the
  // pushes below) and its staging is done.
  cl.sync();
  const bool vl = lane < 6;
  const int ci = vl ? lane : 0;
#define CGROW(lr) (rs + (size_t)(lr) * kCgRow)
  // x = 0, r = b, z = M r, p(prev) = 0 (ba.rs:164-168).  Inner products:
  // each lane accumulates its component's FP64 products over the warp's rows;
  // the lanes are summed once per phase.
  float drz = 0.0f, dbb = 0.0f;
  for (uint32_t lr = warp; lr < nrows; lr += kCgWarps) {
    float* st = CGROW(lr);
    const float ri = vl ? A.b[6 * (size_t)(J.row0 + lr) + ci] : 0.0f;
    float zi = 0.0f;
#pragma unroll
    for (int j = 0; j < 6; ++j) zi += st[kCgM + 6 * ci + j] * __shfl_sync(kFull, ri, j);
    if (vl) {
      st[kCgX + ci] = 0.0f;
      st[kCgR + ci] = ri;
      st[kCgZ + ci] = zi;
      st[kCgP + 6 + ci] = 0.0f;  // p buffer 1 = p(prev) of iteration 0
      drz += ri * zi;
      dbb += ri * ri;
    }
  }
  const float w2[2] = {cg_sum8f(drz), cg_sum8f(dbb)};
  // r.z and b.b; the two-level form pushes the group sums of W^T b beside it
  // and forms c = E^-1 W^T b after the barrier (z = B^-1 b + W c below)
  cg_reduce<kCgWarps, 2>(
      cl, w2, wsm, inbox[1], tot,
      [&](int w) {
        if constexpr (kCoarse)
          cg_group_sums_push<kCgWarps - 1>(cl, w, ngr, A.grp_row0, A.grp_row1, cg0, goff, J.row0,
                                           sW, rs, kCgR, wall_r);
      },
      [&] {
        sc.rz = tot[0];
        sc.b2 = tot[1].hi;
        sc.bf = 0.0f;
        sc.stop = 0;
      },
      [&](int w) {
        if constexpr (kCoarse) {
          for (int o = w; o < nco; o += kCgWarps - 1)
            cg_coarse_dot(sEi, A.cap_dim, cD, o, wall_r, nullptr, 0.0f, scf);
        }
      });
  if constexpr (kCoarse) {
    // z = B^-1 b + W E^-1 W^T b, and r . z with it.
    float drz0 = 0.0f;
    for (uint32_t lr = warp; lr < nrows; lr += kCgWarps) {
      float* st = CGROW(lr);
      const int32_t lg = __float_as_int(st[kCgIdx + 3]);
      const float add = cg_row_wc(sW + (size_t)lr * 42, lg, scf, ci);
      float zi = 0.0f;
      if (vl) {
        zi = st[kCgZ + ci] + add;
        st[kCgZ + ci] = zi;
        drz0 += st[kCgR + ci] * zi;
      }
      cg_push_row(cl, cache, A.sub_ent, (uint32_t)__float_as_int(st[kCgIdx + 4]),
                  (uint32_t)__float_as_int(st[kCgIdx + 5]), zi, 0);
    }
    const float w1[1] = {cg_sum8f(drz0)};
    cg_reduce<kCgWarps, 1>(cl, w1, wsm, inbox[2], tot, [](int) {}, [&] { sc.rz = tot[0]; },
                           [](int) {});
  } else {
    for (uint32_t lr = warp; lr < nrows; lr += kCgWarps) {
      const float* st = CGROW(lr);
      cg_push_row(cl, cache, A.sub_ent, (uint32_t)__float_as_int(st[kCgIdx + 4]),
                  (uint32_t)__float_as_int(st[kCgIdx + 5]), vl ? st[kCgZ + ci] : 0.0f, 0);
    }
    cl.sync();  // z of iteration 0 in every cache
  }
  int32_t spmv = 0;
  const int32_t max_it = A.cap ? min(A.max_iter, A.cap[J.model]) : A.max_iter;
  for (int32_t it = 0; it < max_it; ++it) {
    const int cur = it & 1, prv = cur ^ 1;
    const float bf = sc.bf;
    float dpq = 0.0f, dlens = 0.0f;
    for (uint32_t lr = warp; lr < nrows; lr += kCgWarps) {
      float* st = CGROW(lr);
      const uint32_t b0 = (uint32_t)__float_as_int(st[kCgIdx]);
      const uint32_t b1 = (uint32_t)__float_as_int(st[kCgIdx + 1]);
      float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (uint32_t k = b0 + lane; k < b1; k += 32) {
        const uint32_t kk = k - B0;
        const uint32_t slot = kk < ncached ? sL[kk] : __ldg(A.blk_slot + k);
        float pp[6];
        if (slot & kCgOwnRow) {  // one of this CTA's rows: its row state
          const float* o = CGROW(slot & ~kCgOwnRow);
#pragma unroll
          for (int j = 0; j < 6; ++j) pp[j] = o[kCgZ + j] + o[kCgP + 6 * prv + j] * bf;
        } else {
          const float* crow = cache + (size_t)slot * kCgCache;
          const float4 z0 = *reinterpret_cast<const float4*>(crow);
          const float4 z1 = *reinterpret_cast<const float4*>(crow + 4);
          const float4 q0 = *reinterpret_cast<const float4*>(crow + 8 + 8 * prv);
          const float4 q1 = *reinterpret_cast<const float4*>(crow + 8 + 8 * prv + 4);
          pp[0] = z0.x + q0.x * bf, pp[1] = z0.y + q0.y * bf, pp[2] = z0.z + q0.z * bf;
          pp[3] = z0.w + q0.w * bf, pp[4] = z1.x + q1.x * bf, pp[5] = z1.y + q1.y * bf;
        }
        float m[36];
        load_block(kk < ncached ? sS + (size_t)kk * 36 : A.S + (size_t)k * 36, m);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          float s = acc[i];
#pragma unroll
          for (int j = 0; j < 6; ++j) s += m[6 * i + j] * pp[j];
          acc[i] = s;
        }
      }
      warp_sum8(acc);  // lane 4i holds q_i
      const float qi = __shfl_sync(kFull, acc[0], 4 * ci);
      const float pi = st[kCgZ + ci] + st[kCgP + 6 * prv + ci] * bf;
      __syncwarp();
      if (vl) {
        st[kCgQ + ci] = qi;
        st[kCgP + 6 * cur + ci] = pi;
      }
      if (vl) dpq += pi * qi;
      cg_push_row(cl, cache, A.sub_ent, (uint32_t)__float_as_int(st[kCgIdx + 4]),
                  (uint32_t)__float_as_int(st[kCgIdx + 5]), pi, 8 + 8 * cur);
      if ((int32_t)(J.row0 + lr) == lens) {
        // every CTA's post needs the lens row's p (its share of p.q): push it
        const float p0 = __shfl_sync(kFull, pi, 0), p1 = __shfl_sync(kFull, pi, 1),
                    p2 = __shfl_sync(kFull, pi, 2);
        if (lane < (int)cl.num_blocks()) {
          float* dst = cl.map_shared_rank(lens_p, (unsigned)lane);
          dst[0] = p0, dst[1] = p1, dst[2] = p2;
        }
      }
      // W^T q of the row for the next coarse vector (the lens row, in no
      // group, has W = 0; its transposed terms arrive after the reduction).
      const int32_t lp = __float_as_int(st[kCgIdx + 2]);
      if (lp >= 0) {  // S_cg^T p_c for the lens column
        const int t = lane / 3, j = lane - 3 * (lane / 3);
        const float pt = __shfl_sync(kFull, pi, t < 6 ? t : 0);
        float v = 0.0f;
        if (lane < 18) {
          const uint32_t kk = (uint32_t)lp - B0;
          const float* blk = kk < ncached ? sS + (size_t)kk * 36 : A.S + (size_t)lp * 36;
          v = blk[6 * t + j] * pt;
        }
        v += __shfl_down_sync(kFull, v, 3);
        v += __shfl_down_sync(kFull, v, 6);
        v += __shfl_down_sync(kFull, v, 12);
        if (lane < 3) dlens += v;  // lanes 0, 1, 2: components 0, 1, 2
      }
    }
    const float w4[4] = {cg_sum8f(dpq), __shfl_sync(kFull, dlens, 0), __shfl_sync(kFull, dlens, 1),
                         __shfl_sync(kFull, dlens, 2)};
    const bool lens_here = lens >= 0 && (uint32_t)lens >= J.row0 && (uint32_t)lens < J.row1;
    // p.q; the two-level form pushes the group sums of W^T q beside it and,
    // after the barrier, forms c = E^-1 (W^T r − α W^T q) of the next
    // residual beside warp 0
    const float* wr_cur = wall_r + (size_t)cur * A.cap_dim;
    cg_reduce<kCgWarps, 4>(cl, w4, wsm, inbox[0], tot, [&](int w) {
      if constexpr (kCoarse)
        cg_group_sums_push<kCgWarps - 1>(cl, w, ngr, A.grp_row0, A.grp_row1, cg0, goff, J.row0,
                                         sW, rs, kCgQ, wall_q);
    }, [&] {
      DFloat pq = tot[0];
      if (lens >= 0) {
        // The lens row's q gets the transposed camera terms; its share of
        // p.q is p_g . (sum S_cg^T p_c), with p_g pushed by its owner before
        // the barrier.
#pragma unroll
        for (int c = 0; c < 3; ++c) pq = df_sum(pq, df_scale(lens_p[c], tot[1 + c]));
        if (lens_here) {
          float* q = CGROW((uint32_t)lens - J.row0) + kCgQ;
          for (int c = 0; c < 3; ++c) q[c] = df_sum(DFloat{q[c], 0.0f}, tot[1 + c]).hi;
        }
      }
      // ba.rs:174 breaks on a vanishing p.q; an FP32 quotient needs it normal
      sc.stop = fabsf(pq.hi) < 1.17549435e-38f ? 1 : 0;
      sc.af = sc.stop ? 0.0f : sc.rz.hi / pq.hi;
    }, [&](int w) {
      if constexpr (kCoarse) {
        if (w < nco) {
          const float a = cg_alpha(inbox[0], (int)cl.num_blocks(), lane, lens, lens_p, sc.rz.hi);
          for (int o = w; o < nco; o += kCgWarps - 1)
            cg_coarse_dot(sEi, A.cap_dim, cD, o, wr_cur, wall_q, a, scf);
        }
      }
    });
    ++spmv;
    if (sc.stop) break;
    const float af = sc.af;
    float drr = 0.0f, drz2 = 0.0f;
    for (uint32_t lr = warp; lr < nrows; lr += kCgWarps) {
      float* st = CGROW(lr);
      float ri = 0.0f;
      if (vl) {
        st[kCgX + ci] += st[kCgP + 6 * cur + ci] * af;
        ri = st[kCgR + ci] - st[kCgQ + ci] * af;
        st[kCgR + ci] = ri;
      }
      float zi = 0.0f;
#pragma unroll
      for (int j = 0; j < 6; ++j) zi += st[kCgM + 6 * ci + j] * __shfl_sync(kFull, ri, j);
      if constexpr (kCoarse) {
        // z = B^-1 r + W c
        zi += cg_row_wc(sW + (size_t)lr * 42, __float_as_int(st[kCgIdx + 3]), scf, ci);
      }
      if (vl) {
        st[kCgZ + ci] = zi;
        drr += ri * ri;
        drz2 += ri * zi;
      }
      cg_push_row(cl, cache, A.sub_ent, (uint32_t)__float_as_int(st[kCgIdx + 4]),
                  (uint32_t)__float_as_int(st[kCgIdx + 5]), zi, 0);
    }
    const float w2b[2] = {cg_sum8f(drr), cg_sum8f(drz2)};
    // r.r and r.z; the two-level form pushes the group sums of the next
    // W^T r beside them
    cg_reduce<kCgWarps, 2>(cl, w2b, wsm, inbox[1], tot, [&](int w) {
      if constexpr (kCoarse)
        cg_group_sums_push<kCgWarps - 1>(cl, w, ngr, A.grp_row0, A.grp_row1, cg0, goff, J.row0,
                                         sW, rs, kCgR, wall_r + (size_t)prv * A.cap_dim);
    }, [&] {
      sc.stop = tot[0].hi < (float)A.tol * sc.b2 ? 1 : 0;  // ba.rs:182
      sc.bf = tot[1].hi / sc.rz.hi;                        // ba.rs:189-190
      sc.rz = tot[1];
    }, [](int) {});
    if (sc.stop) break;
  }
  for (uint32_t lr = warp; lr < nrows; lr += kCgWarps)
    if (vl) A.x[6 * (size_t)(J.row0 + lr) + ci] = CGROW(lr)[kCgX + ci];
#undef CGROW
  if (cl.block_rank() == 0 && threadIdx.x == 0) A.iters[J.model] = spmv;
  cl.sync();  // no CTA leaves while another may still read its shared memory
}

}  // namespace ba
