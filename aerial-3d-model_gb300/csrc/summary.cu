// Per-camera summary of a finished sparse reconstruction, the part of
// cameras.json computed from the bundle-adjusted problem (sparse.rs:470-483
// and 515-533), and the f32 point copy stored in sparse.ply (mod.rs:31-35):
//
//  * neighbours: the cameras sharing the most points with each camera, best
//    first (the reference sorts a HashMap's entries by count, so the order
//    of equal counts is unspecified there; here it is ascending camera
//    index), at most `max_nb` of them (8 in sparse.rs:532);
//  * depth range: camera-frame depths z of the camera's observed points,
//    sorted by total order, (d[n/20] * 0.8, d[19n/20] * 1.25) when n >= 10,
//    else (0.3 agl, 3 agl) (sparse.rs:519-525);
//  * points as f32, rounded to nearest.
//
// Observations are grouped by camera with one stable radix sort; a CTA per
// camera walks its observations' points and counts co-observing cameras in
// a shared-memory histogram (global scratch when the camera count does not
// fit), then picks the top entries by CTA-wide argmax. Depths are sorted
// within each camera by two stable radix sorts (depth bits, then camera).
#include <algorithm>
#include <cmath>
#include <vector>

#include "ba_gb300.h"
#include "context.cuh"
#include "primitives.cuh"

namespace ba {
namespace {

constexpr int kNbThreads = 256;
constexpr int kMaxNeighbours = 64;
constexpr int64_t kSmemHistCams = 24576;  // 96 KB of u32 counts

__global__ void check_obs_kernel(int64_t no, int64_t nc, int64_t np, const uint32_t* obs_cam,
                                 const uint32_t* obs_pt, uint32_t* err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= no) return;
  if (obs_cam[i] >= (uint64_t)nc || obs_pt[i] >= (uint64_t)np) atomicOr(err, ERR_BAD_INDEX);
  if (i > 0 && obs_pt[i - 1] > obs_pt[i]) atomicOr(err, ERR_UNSORTED);
}

__global__ void cam_keys_kernel(int64_t no, const uint32_t* obs_cam, uint64_t* key,
                                uint32_t* idx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= no) return;
  key[i] = obs_cam[i];
  idx[i] = (uint32_t)i;
}

// f64 bits -> u64 whose unsigned order is f64::total_cmp's order.
__device__ __forceinline__ uint64_t total_order_key(double z) {
  const uint64_t b = (uint64_t)__double_as_longlong(z);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_total_order_key(uint64_t k) {
  const uint64_t b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}

// Camera-frame depth of every observation, (R (X - C)).z with the products
// summed left to right and no fused multiply-add (Pose::to_cam,
// geometry.rs:57-59, as sparse.rs:476 uses it).
__global__ void depth_keys_kernel(int64_t no, const uint32_t* obs_cam, const uint32_t* obs_pt,
                                  const double* rot, const double* center, const double* points,
                                  uint64_t* dkey, uint32_t* dcam) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= no) return;
  const uint32_t c = obs_cam[i], p = obs_pt[i];
  const double* R = rot + 9 * (size_t)c + 6;
  const double* C = center + 3 * (size_t)c;
  const double* X = points + 3 * (size_t)p;
  const double d0 = __dsub_rn(X[0], C[0]), d1 = __dsub_rn(X[1], C[1]),
               d2 = __dsub_rn(X[2], C[2]);
  const double z = __dadd_rn(__dadd_rn(__dmul_rn(R[0], d0), __dmul_rn(R[1], d1)),
                             __dmul_rn(R[2], d2));
  dkey[i] = total_order_key(z);
  dcam[i] = c;
}

// (depth key, camera) -> (camera, depth key) for the second, stable sort.
__global__ void swap_keys_kernel(int64_t n, const uint64_t* dkey, const uint32_t* dcam,
                                 uint64_t* ckey, uint64_t* cval) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  ckey[i] = dcam[i];
  cval[i] = dkey[i];
}

__global__ void depth_range_kernel(int64_t nc, const uint32_t* cam_ptr, const uint64_t* sorted,
                                   double agl, double* range) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nc) return;
  const uint32_t b = cam_ptr[a], n = cam_ptr[a + 1] - b;
  if (n >= 10) {
    range[2 * a] = from_total_order_key(sorted[b + n / 20]) * 0.8;
    range[2 * a + 1] = from_total_order_key(sorted[b + (uint64_t)n * 19 / 20]) * 1.25;
  } else {
    range[2 * a] = agl * 0.3;
    range[2 * a + 1] = agl * 3.0;
  }
}

__device__ __forceinline__ uint64_t block_max_u64(uint64_t v, uint64_t* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, (uint64_t)__shfl_xor_sync(kFull, v, o));
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < kNbThreads / 32 ? red[lane] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, (uint64_t)__shfl_xor_sync(kFull, v, o));
    if (lane == 0) red[kNbThreads / 32] = v;
  }
  __syncthreads();
  const uint64_t r = red[kNbThreads / 32];
  __syncthreads();
  return r;
}

struct NbArgs {
  int64_t nc;
  const uint32_t* cam_ptr;  // [nc + 1] into cam_obs
  const uint32_t* cam_obs;  // observation indices grouped by camera
  const uint32_t* pt_ptr;   // [np + 1] into the (point-sorted) observations
  const uint32_t* obs_cam;
  const uint32_t* obs_pt;
  int max_nb;
  uint32_t* hist_global;  // gridDim.x * nc counts when not in shared memory
  uint32_t* nb;           // [nc * max_nb], UINT32_MAX padded
  uint32_t* shared;       // [nc * max_nb], 0 padded
  int32_t* n_nb;          // [nc]
};

// Persistent CTAs, one camera at a time: count the cameras that observe the
// points this camera observes (sparse.rs:477-481: every ordered pair of
// distinct cameras of a point), then take the largest counts.
template <bool kSmem>
__global__ void __launch_bounds__(kNbThreads) neighbours_kernel(NbArgs A) {
  extern __shared__ uint32_t smem_hist[];
  __shared__ uint64_t red[kNbThreads / 32 + 1];
  uint32_t* hist = kSmem ? smem_hist : A.hist_global + (size_t)blockIdx.x * A.nc;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t c = threadIdx.x; c < A.nc; c += kNbThreads) hist[c] = 0;
  __syncthreads();
  for (int64_t a = blockIdx.x; a < A.nc; a += gridDim.x) {
    for (uint32_t k = A.cam_ptr[a] + warp; k < A.cam_ptr[a + 1]; k += kNbThreads / 32) {
      const uint32_t p = A.obs_pt[A.cam_obs[k]];
      for (uint32_t j = A.pt_ptr[p] + lane; j < A.pt_ptr[p + 1]; j += 32) {
        const uint32_t b = A.obs_cam[j];
        if (b != (uint32_t)a) atomicAdd(&hist[b], 1u);
      }
    }
    __syncthreads();
    int r = 0;
    for (; r < A.max_nb; ++r) {
      uint64_t best = 0;
      for (int64_t c = threadIdx.x; c < A.nc; c += kNbThreads) {
        const uint32_t h = hist[c];
        if (h) best = max(best, ((uint64_t)h << 32) | (uint32_t)(0xffffffffu - (uint32_t)c));
      }
      best = block_max_u64(best, red);
      if (best == 0) break;
      const uint32_t b = 0xffffffffu - (uint32_t)best;
      if (threadIdx.x == 0) {
        A.nb[a * A.max_nb + r] = b;
        A.shared[a * A.max_nb + r] = (uint32_t)(best >> 32);
        hist[b] = 0;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      A.n_nb[a] = r;
      for (int q = r; q < A.max_nb; ++q) A.nb[a * A.max_nb + q] = 0xffffffffu, A.shared[a * A.max_nb + q] = 0;
    }
    for (int64_t c = threadIdx.x; c < A.nc; c += kNbThreads) hist[c] = 0;
    __syncthreads();
  }
}

__global__ void points_f32_kernel(int64_t n, const double* p, float* q) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) q[i] = __double2float_rn(p[i]);
}

int bit_width(uint64_t v) {
  int b = 0;
  while (v) ++b, v >>= 1;
  return b;
}

// Device outputs of one summary.
struct SummaryRun {
  DevBuf<uint32_t> err, pt_ptr, cam_ptr, cam_obs, nb, shared, hist;
  DevBuf<int32_t> n_nb;
  DevBuf<double> range;
  DevBuf<float> pts32;

  // All pointers are device pointers.
  void run(int64_t nc, int64_t np, int64_t no, const uint32_t* obs_cam, const uint32_t* obs_pt,
           const double* rot, const double* center, const double* points, int max_nb,
           double agl, int n_sm, cudaStream_t s) {
    if (max_nb < 1 || max_nb > kMaxNeighbours) throw BadInput("max_neighbours must be in 1..64");
    if (!std::isfinite(agl)) throw BadInput("agl must be finite");
    if (no > 0xfffffff0LL || np > 0xfffffff0LL || nc > 0xfffffff0LL)
      throw BadInput("too many cameras, points or observations for 32-bit indexing");
    auto A = [&](auto& d, int64_t n) { d.alloc(std::max<int64_t>(n, 1), s); };
    A(err, 1), A(pt_ptr, np + 1), A(cam_ptr, nc + 1), A(cam_obs, no);
    A(nb, nc * max_nb), A(shared, nc * max_nb), A(n_nb, nc), A(range, 2 * nc), A(pts32, 3 * np);
    err.zero();
    if (no > 0)
      BA_LAUNCH(check_obs_kernel<<<grid_for(no, 256), 256, 0, s>>>(no, nc, np, obs_cam, obs_pt, err));
    uint32_t e = 0;
    check(cudaMemcpyAsync(&e, err.p, 4, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaStreamSynchronize(s), "summary check");
    if (e & ERR_BAD_INDEX) throw BadInput("obs_cam or obs_pt out of range");
    if (e & ERR_UNSORTED) throw BadInput("observations must be sorted by point");
    if (np > 0) lower_bounds_u32(obs_pt, no, pt_ptr, np, s);
    {
      // Observations grouped by camera (stable: index order within a camera).
      DevBuf<uint64_t> key(std::max<int64_t>(no, 1), s), ktmp(std::max<int64_t>(no, 1), s);
      DevBuf<uint32_t> vtmp(std::max<int64_t>(no, 1), s);
      if (no > 0) {
        BA_LAUNCH(cam_keys_kernel<<<grid_for(no, 256), 256, 0, s>>>(no, obs_cam, key, cam_obs));
        radix_sort_u64_u32(key, cam_obs, ktmp, vtmp, no, bit_width(nc), s);
      }
      if (nc > 0) lower_bounds_u64(key, no, cam_ptr, nc, 1, s);
    }
    if (nc > 0) {
      // Depths sorted within each camera: by total order, then (stably) by camera.
      DevBuf<uint64_t> dkey(std::max<int64_t>(no, 1), s), dtmp(std::max<int64_t>(no, 1), s);
      DevBuf<uint32_t> dcam(std::max<int64_t>(no, 1), s), ctmp(std::max<int64_t>(no, 1), s);
      if (no > 0) {
        BA_LAUNCH(depth_keys_kernel<<<grid_for(no, 256), 256, 0, s>>>(no, obs_cam, obs_pt, rot, center,
                                                                     points, dkey, dcam));
        radix_sort_u64_u32(dkey, dcam, dtmp, ctmp, no, 64, s);
      }
      DevBuf<uint64_t> ckey(std::max<int64_t>(no, 1), s), cval(std::max<int64_t>(no, 1), s);
      if (no > 0) {
        BA_LAUNCH(swap_keys_kernel<<<grid_for(no, 256), 256, 0, s>>>(no, dkey, dcam, ckey, cval));
        // The sort scratch of the first sort is reused for the second.
        radix_sort_u64_u64(ckey, cval, dtmp, dkey, no, bit_width(nc), s);
      }
      BA_LAUNCH(depth_range_kernel<<<grid_for(nc, 128), 128, 0, s>>>(nc, cam_ptr, cval, agl, range));
      const bool in_smem = nc <= kSmemHistCams;
      const unsigned grid = (unsigned)std::min<int64_t>(nc, 2 * (int64_t)std::max(n_sm, 1));
      if (!in_smem) A(hist, (int64_t)grid * nc);
      NbArgs na{nc, cam_ptr, cam_obs, pt_ptr, obs_cam, obs_pt, max_nb, hist, nb, shared, n_nb};
      if (in_smem) {
        const size_t smem = (size_t)nc * 4;
        check(cudaFuncSetAttribute(neighbours_kernel<true>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
              "neighbours smem");
        BA_LAUNCH(neighbours_kernel<true><<<grid, kNbThreads, smem, s>>>(na));
      } else {
        BA_LAUNCH(neighbours_kernel<false><<<grid, kNbThreads, 0, s>>>(na));
      }
    }
    if (np > 0) BA_LAUNCH(points_f32_kernel<<<grid_for(3 * np, 256), 256, 0, s>>>(3 * np, points, pts32));
  }

  void copy_out(int64_t nc, int64_t np, int max_nb, uint32_t* o_nb, uint32_t* o_shared,
                int32_t* o_n_nb, double* o_range, float* o_pts, cudaStream_t s) const {
    auto down = [&](auto* h, const auto& d, int64_t n) {
      if (h && n > 0) check(cudaMemcpyAsync(h, d.p, n * sizeof(*h), cudaMemcpyDefault, s), "copy out");
    };
    down(o_nb, nb, nc * max_nb), down(o_shared, shared, nc * max_nb), down(o_n_nb, n_nb, nc);
    down(o_range, range, 2 * nc), down(o_pts, pts32, 3 * np);
    check(cudaStreamSynchronize(s), "summary");
  }
};

int sm_count() {
  int dev = 0, n = 0;
  check(cudaGetDevice(&dev), "cudaGetDevice");
  check(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev), "attribute");
  return n;
}

}  // namespace
}  // namespace ba

using namespace ba;

extern "C" ba_status ba_sparse_summary(const ba_problem* problem, const ba_state* state,
                                       int32_t max_neighbours, double agl, void* stream,
                                       uint32_t* neighbours, uint32_t* shared,
                                       int32_t* n_neighbours, double* depth_range,
                                       float* points_f32) {
  return guarded([&] {
    if (!problem || !state) throw BadInput("null problem or state");
    const int64_t nc = problem->n_cams, np = problem->n_points, no = problem->n_obs;
    if (nc < 0 || np < 0 || no < 0) throw BadInput("negative size");
    if ((no > 0 && (!problem->obs_cam || !problem->obs_pt)) ||
        (nc > 0 && (!state->rot || !state->center)) || (np > 0 && !state->points))
      throw BadInput("null array");
    cudaStream_t s = (cudaStream_t)stream;
    auto A = [&](auto& d, int64_t n) { d.alloc(std::max<int64_t>(n, 1), s); };
    DevBuf<uint32_t> cam, pt;
    DevBuf<double> rot, center, points;
    A(cam, no), A(pt, no), A(rot, 9 * nc), A(center, 3 * nc), A(points, 3 * np);
    auto up = [&](auto& d, const auto* h, int64_t n) {
      if (n > 0) check(cudaMemcpyAsync(d.p, h, n * sizeof(*h), cudaMemcpyDefault, s), "copy in");
    };
    up(cam, problem->obs_cam, no), up(pt, problem->obs_pt, no);
    up(rot, state->rot, 9 * nc), up(center, state->center, 3 * nc), up(points, state->points, 3 * np);
    SummaryRun R;
    R.run(nc, np, no, cam, pt, rot, center, points, max_neighbours, agl, sm_count(), s);
    R.copy_out(nc, np, max_neighbours, neighbours, shared, n_neighbours, depth_range, points_f32, s);
  });
}

extern "C" ba_status ba_context_sparse_summary(ba_context* ctx, int32_t max_neighbours, double agl,
                                               uint32_t* neighbours, uint32_t* shared,
                                               int32_t* n_neighbours, double* depth_range,
                                               float* points_f32) {
  return guarded([&] {
    if (!ctx) throw BadInput("null context");
    if (!ctx->uploaded) throw BadInput("no problem uploaded");
    if (ctx->nm != 1) throw BadInput("the context must hold one model");
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t s = ctx->stream;
    SummaryRun R;
    R.run(ctx->nc, ctx->np, ctx->no, ctx->obs_cam, ctx->obs_pt, ctx->rot, ctx->center,
          ctx->points, max_neighbours, agl, ctx->n_sm, s);
    R.copy_out(ctx->nc, ctx->np, max_neighbours, neighbours, shared, n_neighbours, depth_range,
               points_f32, s);
  });
}
