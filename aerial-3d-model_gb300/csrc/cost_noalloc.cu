// Robust cost of one problem held in device memory, without allocating.
//
// ba_robust_cost_noalloc evaluates the cost the solver accepts or rejects a
// step on (ba.rs:103-128) for callers that must not allocate device memory:
// a host that has handed the whole device to another runtime's caching
// allocator (nothing left for cudaMalloc), or a latency-critical loop — such
// as the per-round reprojection gating before each bundle adjustment
// (sparse.rs:389-421) — where cudaMalloc / cudaFree would synchronise the
// whole device.  Inputs and outputs are the caller's; the per-chunk partial
// sums live in a fixed device array of this file (kNoAllocChunks chunks of
// kNoAllocChunkObs observations, so at most 33,554,432 observations per call).
//
// The array is shared by every call on a device and keeps the last call's
// contents.  Each call writes every partial it later reads, so nothing needs
// clearing; but calls whose kernels overlap on the GPU (different streams, or
// different host threads on one stream without ordering) race on it.
//
// Indices are checked in the kernel: an observation whose camera, point or
// lens group is out of range is skipped and counted, and the call returns
// BA_BAD_INPUT (the solver's own upload check, ERR_BAD_INDEX, rejects the
// same inputs).
#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include "ba_gb300.h"
#include "camera_model.h"
#include "context.cuh"

namespace ba {
namespace {

constexpr int kNoAllocThreads = 256;
constexpr int64_t kNoAllocChunkObs = 4096;
constexpr int64_t kNoAllocChunks = 8192;  // 8192 x 4096 = 33,554,432 observations
constexpr int kMaxDevices = 64;

// Scratch of ba_robust_cost_noalloc: [kNoAllocChunks][4] partials (cost, sum
// of squares, count, observations with an index out of range), then 4
// doubles of result.  262,176 bytes per device.
constexpr int kNoAllocParts = 4;
__device__ __align__(256) double g_noalloc_scratch[kNoAllocChunks * kNoAllocParts + kNoAllocParts];

__device__ __forceinline__ double rho(double e2, double sigma, int loss) {
  if (loss == BA_LOSS_HUBER) {
    const double a = sqrt(e2);
    return a <= sigma ? e2 : 2.0 * sigma * a - sigma * sigma;
  }
  const double s2 = sigma * sigma;
  return s2 * log(1.0 + e2 / s2);
}

__global__ void __launch_bounds__(kNoAllocThreads)
    noalloc_chunk_kernel(ba_problem P, ba_state st, double sigma, int loss, double* scratch) {
  __shared__ double red[kNoAllocParts * 32];
  const int64_t ch = blockIdx.x;
  const int64_t b = ch * kNoAllocChunkObs;
  const int64_t e = min(P.n_obs, b + kNoAllocChunkObs);
  const double behind = sigma * sigma * 10.0;  // ba.rs:116
  double acc[kNoAllocParts] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t k = b + threadIdx.x; k < e; k += blockDim.x) {
    const uint32_t cam = P.obs_cam[k], pt = P.obs_pt[k];
    // Every index is checked before it addresses memory.
    if ((int64_t)cam >= P.n_cams || (int64_t)pt >= P.n_points) {
      acc[3] += 1.0;
      continue;
    }
    const uint32_t grp = P.cam_group[cam];
    if ((int64_t)grp >= P.n_groups) {
      acc[3] += 1.0;
      continue;
    }
    double u[2];
    if (bacam::project(st.rot + 9 * (size_t)cam, st.center + 3 * (size_t)cam,
                       st.intr + 5 * (size_t)grp, st.points + 3 * (size_t)pt, u)) {
      const double ex = P.obs_uv[2 * k] - u[0], ey = P.obs_uv[2 * k + 1] - u[1];
      const double e2 = ex * ex + ey * ey;
      acc[0] += rho(e2, sigma, loss);
      acc[1] += e2;
      acc[2] += 1.0;
    } else {
      acc[0] += behind;
    }
  }
  block_sum<kNoAllocParts>(acc, red);
  if (threadIdx.x == 0)
    for (int i = 0; i < kNoAllocParts; ++i) scratch[kNoAllocParts * ch + i] = acc[i];
}

__global__ void noalloc_final_kernel(ba_problem P, ba_state st, int64_t nchunks,
                                     double* scratch) {
  const int lane = threadIdx.x;
  double a[kNoAllocParts] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t c = lane; c < nchunks; c += 32)
    for (int i = 0; i < kNoAllocParts; ++i) a[i] += scratch[kNoAllocParts * c + i];
  double pr = 0.0;  // ba.rs:120-126
  if (P.prior_mask) {
    for (int64_t c = lane; c < P.n_cams; c += 32) {
      if (!P.prior_mask[c]) continue;
      const double* q = P.prior + 6 * c;
      const double dx = st.center[3 * c] - q[0], dy = st.center[3 * c + 1] - q[1],
                   dz = st.center[3 * c + 2] - q[2];
      pr += (dx / q[3]) * (dx / q[3]) + (dy / q[4]) * (dy / q[4]) + (dz / q[5]) * (dz / q[5]);
    }
  }
  for (int i = 0; i < kNoAllocParts; ++i) a[i] = warp_sum(a[i]);
  pr = warp_sum(pr);
  if (lane == 0) {
    double* out = scratch + kNoAllocParts * kNoAllocChunks;
    out[0] = a[0] + pr;
    out[1] = a[1];
    out[2] = a[2];
    out[3] = a[3];
  }
}

// Device address of the scratch array, looked up once per device with that
// device current.
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kMaxDevices] = {};

double* noalloc_scratch(int dev) {
  if (dev < 0 || dev >= kMaxDevices) throw BadInput("device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    double* p = nullptr;
    check(cudaGetSymbolAddress((void**)&p, g_noalloc_scratch), "cudaGetSymbolAddress");
    if (!p) throw CudaError(cudaErrorInvalidSymbol, "scratch symbol has no device address");
    g_noalloc_ptr[dev] = p;
  }
  return g_noalloc_ptr[dev];
}

}  // namespace
}  // namespace ba

using namespace ba;

extern "C" ba_status ba_robust_cost_noalloc(const ba_problem* problem, const ba_state* state,
                                            double sigma_px, int32_t loss, void* stream,
                                            double* cost, double* rms, int64_t* n_in_front) {
  return guarded([&] {
    if (!problem || !state) throw BadInput("null problem or state");
    const ba_problem P = *problem;
    const ba_state S = *state;
    if (P.n_cams < 0 || P.n_obs < 0 || P.n_points < 0 || P.n_groups < 0)
      throw BadInput("negative size");
    if (P.n_obs > kNoAllocChunks * kNoAllocChunkObs)
      throw BadInput("n_obs " + std::to_string(P.n_obs) +
                     " exceeds the no-allocation limit of " +
                     std::to_string(kNoAllocChunks * kNoAllocChunkObs) + " observations");
    if (!(sigma_px > 0.0) || !std::isfinite(sigma_px)) throw BadInput("sigma_px must be > 0");
    if (loss != BA_LOSS_CAUCHY && loss != BA_LOSS_HUBER) throw BadInput("unknown loss");
    if (P.n_obs > 0 && (!P.obs_cam || !P.obs_pt || !P.obs_uv || !P.cam_group || !S.rot ||
                        !S.center || !S.intr || !S.points))
      throw BadInput("null device array");
    if (P.prior_mask && !P.prior) throw BadInput("prior_mask without prior");
    int dev = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    double* scratch = noalloc_scratch(dev);
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t nchunks = (P.n_obs + kNoAllocChunkObs - 1) / kNoAllocChunkObs;
    if (nchunks > 0)
      BA_LAUNCH(noalloc_chunk_kernel<<<(unsigned)nchunks, kNoAllocThreads, 0, s>>>(
          P, S, sigma_px, loss, scratch));
    BA_LAUNCH(noalloc_final_kernel<<<1, 32, 0, s>>>(P, S, nchunks, scratch));
    double out[kNoAllocParts];
    check(cudaMemcpyAsync(out, scratch + kNoAllocParts * kNoAllocChunks, sizeof out,
                          cudaMemcpyDeviceToHost, s),
          "d2h");
    check(cudaStreamSynchronize(s), "cost");
    if (out[3] > 0.0)
      throw BadInput(std::to_string((int64_t)out[3]) +
                     " observations have a camera, point or lens group index out of range");
    if (cost) *cost = out[0];
    if (rms) *rms = std::sqrt(out[1] / std::max(out[2], 1.0));
    if (n_in_front) *n_in_front = (int64_t)out[2];
  });
}
