// One round of the sparse stage's triangulation and reprojection gating,
// run over every track on the device (sparse.rs:389-421 with triangulate,
// geometry.rs:115-144, and max_ray_angle, geometry.rs:146-156), and the
// build of the bundle-adjustment problem from the kept tracks in HBM
// (sparse.rs:429-449), so a round's problem never leaves the device.
//
// Thread per track, FP64 throughout: undistort each observation (8
// fixed-point steps), accumulate A^T A of the linear triangulation, take the
// eigenvector of its smallest eigenvalue (cyclic Jacobi on the 4x4), keep
// the observations that reproject within the threshold, and keep the track
// if two or more remain and their rays span more than 2 degrees (three or
// more views) or 6 degrees (two views).
#include <cmath>
#include <vector>

#include "ba_gb300.h"
#include "camera_model.h"
#include "context.cuh"
#include "primitives.cuh"

namespace ba {
namespace {

constexpr int kTriThreads = 128;

struct TriArgs {
  int64_t nt, no, nc, ng;
  const uint32_t* track_ptr;
  const uint32_t* obs_cam;
  const double* obs_uv;
  const uint32_t* cam_group;
  const double* rot;
  const double* center;
  const double* intr;
  double thr;
  uint8_t* kept;
  double* points;
  uint8_t* good;
  uint32_t* err;
  uint32_t* obs_track;  // [no] track of each observation
  double* pn;           // [2 no] undistorted normalised coordinates
  double* ray;          // [3 no] unit ray from the camera to the point (good obs)
};

// Symmetric 4x4 eigen-decomposition by cyclic Jacobi rotations: on return A
// is (numerically) diagonal and V's columns are the eigenvectors.
__device__ void jacobi4(double A[4][4], double V[4][4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) V[i][j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = 0.0, diag = 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      diag += A[i][i] * A[i][i];
#pragma unroll
      for (int j = i + 1; j < 4; ++j) off += A[i][j] * A[i][j];
    }
    if (off <= 1e-34 * diag || off == 0.0) break;
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = p + 1; q < 4; ++q) {
        if (A[p][q] == 0.0) continue;
        const double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - sn * akq;
          A[k][q] = sn * akp + c * akq;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - sn * aqk;
          A[q][k] = sn * apk + c * aqk;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - sn * vkq;
          V[k][q] = sn * vkp + c * vkq;
        }
      }
  }
}

// Intrinsics::undistort (geometry.rs:35-44): pixel -> normalised, 8 steps.
__device__ __forceinline__ void undistort(const double* K, const double* u, double* p) {
  const double qx = (u[0] - K[1]) / K[0], qy = (u[1] - K[2]) / K[0];
  double px = qx, py = qy;
  for (int i = 0; i < 8; ++i) {
    const double r2 = px * px + py * py;
    const double d = 1.0 + K[3] * r2 + K[4] * r2 * r2;
    px = qx / d;
    py = qy / d;
  }
  p[0] = px, p[1] = py;
}

// The round runs in four passes, so that per-observation work is spread
// over threads of observations rather than serialised per track: (1) track
// checks and the observation -> track map (thread per track); (2) undistort
// (thread per observation); (3) A^T A, its smallest eigenvector and the
// point (thread per track); (4) the reprojection gate and the unit ray of
// each observation (thread per observation); (5) the ray-angle test and the
// keep decision (thread per track).  The arithmetic and its order are those
// of a single pass per track.

__global__ void tri_check_kernel(TriArgs T) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T.nt) return;
  const uint32_t b = T.track_ptr[t], e = T.track_ptr[t + 1];
  T.kept[t] = 0;
  T.points[3 * t] = T.points[3 * t + 1] = T.points[3 * t + 2] = 0.0;
  if (e < b || e > (uint64_t)T.no) {
    atomicOr(T.err, ERR_BAD_INDEX);
    return;
  }
  for (uint32_t k = b; k < e; ++k) {
    T.good[k] = 0;
    T.obs_track[k] = (uint32_t)t;
    if (T.obs_cam[k] >= (uint64_t)T.nc || T.cam_group[T.obs_cam[k]] >= (uint64_t)T.ng)
      atomicOr(T.err, ERR_BAD_INDEX);
  }
}

__global__ void tri_undistort_kernel(TriArgs T) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= T.no || T.obs_track[k] == 0xffffffffu) return;
  undistort(T.intr + 5 * (size_t)T.cam_group[T.obs_cam[k]], T.obs_uv + 2 * (size_t)k, T.pn + 2 * k);
}

__global__ void __launch_bounds__(kTriThreads) tri_point_kernel(TriArgs T) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T.nt) return;
  const uint32_t b = T.track_ptr[t], e = T.track_ptr[t + 1];
  if (e - b < 2) return;
  // A^T A of the linear triangulation (geometry.rs:118-131).
  double ata[4][4] = {};
  for (uint32_t k = b; k < e; ++k) {
    const uint32_t c = T.obs_cam[k];
    const double* R = T.rot + 9 * (size_t)c;
    const double* C = T.center + 3 * (size_t)c;
    const double pn[2] = {T.pn[2 * (size_t)k], T.pn[2 * (size_t)k + 1]};
    double tr[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) tr[r] = -(R[3 * r] * C[0] + R[3 * r + 1] * C[1] + R[3 * r + 2] * C[2]);
    double a0[4], a1[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double r0 = q < 3 ? R[q] : tr[0], r1 = q < 3 ? R[3 + q] : tr[1],
                   r2 = q < 3 ? R[6 + q] : tr[2];
      a0[q] = pn[0] * r2 - r0;
      a1[q] = pn[1] * r2 - r1;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int q = 0; q < 4; ++q) ata[r][q] += a0[r] * a0[q] + a1[r] * a1[q];
  }
  double V[4][4];
  jacobi4(ata, V);
  int best = 0;
#pragma unroll
  for (int i = 1; i < 4; ++i)
    if (ata[i][i] < ata[best][best]) best = i;
  double v[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = best == 0 ? V[i][0] : best == 1 ? V[i][1] : best == 2 ? V[i][2] : V[i][3];
  if (fabs(v[3]) < 1e-12) return;  // geometry.rs:139-141
  T.points[3 * t] = v[0] / v[3], T.points[3 * t + 1] = v[1] / v[3], T.points[3 * t + 2] = v[2] / v[3];
  T.kept[t] = 2;  // triangulated; decided in tri_keep_kernel
}

// Reprojection gate (sparse.rs:397-405) and the unit ray of each good
// observation (geometry.rs:147).
__global__ void tri_gate_kernel(TriArgs T) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= T.no) return;
  const uint32_t t = T.obs_track[k];
  if (t == 0xffffffffu || T.kept[t] != 2) return;
  const double X[3] = {T.points[3 * (size_t)t], T.points[3 * (size_t)t + 1], T.points[3 * (size_t)t + 2]};
  const uint32_t c = T.obs_cam[k];
  const double* C = T.center + 3 * (size_t)c;
  double u[2];
  if (!bacam::project(T.rot + 9 * (size_t)c, C, T.intr + 5 * (size_t)T.cam_group[c], X, u)) return;
  const double dx = u[0] - T.obs_uv[2 * (size_t)k], dy = u[1] - T.obs_uv[2 * (size_t)k + 1];
  if (!(sqrt(dx * dx + dy * dy) < T.thr)) return;
  T.good[k] = 1;
  double r[3] = {X[0] - C[0], X[1] - C[1], X[2] - C[2]};
  const double l = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  T.ray[3 * k] = r[0] / l, T.ray[3 * k + 1] = r[1] / l, T.ray[3 * k + 2] = r[2] / l;
}

// Keep the track if two or more observations remain and their rays span
// more than 2 degrees (three or more views) or 6 degrees (two views):
// acos is decreasing, so the largest angle is acos of the smallest clamped
// dot product (the value the reference's running max of acos keeps).
__global__ void __launch_bounds__(kTriThreads) tri_keep_kernel(TriArgs T) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T.nt || T.kept[t] != 2) return;
  const uint32_t b = T.track_ptr[t], e = T.track_ptr[t + 1];
  int ng = 0;
  double min_d = 1.0;
  for (uint32_t i = b; i < e; ++i) {
    if (!T.good[i]) continue;
    ++ng;
    const double r0 = T.ray[3 * (size_t)i], r1 = T.ray[3 * (size_t)i + 1], r2 = T.ray[3 * (size_t)i + 2];
    for (uint32_t j = i + 1; j < e; ++j) {
      if (!T.good[j]) continue;
      const double d = r0 * T.ray[3 * (size_t)j] + r1 * T.ray[3 * (size_t)j + 1] + r2 * T.ray[3 * (size_t)j + 2];
      min_d = fmin(min_d, fmin(1.0, fmax(-1.0, d)));
    }
  }
  bool ok = ng >= 2;
  if (ok) {
    const double deg = acos(min_d) * (180.0 / 3.14159265358979323846);
    ok = ng >= 3 ? deg > 2.0 : deg > 6.0;  // sparse.rs:411-415
  }
  if (!ok) {
    for (uint32_t k = b; k < e; ++k) T.good[k] = 0;
    T.kept[t] = 0;
    T.points[3 * t] = T.points[3 * t + 1] = T.points[3 * t + 2] = 0.0;
    return;
  }
  T.kept[t] = 1;
}

// Problem of the kept tracks (sparse.rs:429-440): points in track order,
// observations of each kept track in order (so sorted by point).
__global__ void compact_kernel(int64_t nt, const uint32_t* track_ptr, const uint8_t* kept,
                               const uint32_t* pt_idx, const uint32_t* obs_pos,
                               const uint8_t* good, const uint32_t* obs_cam, const double* obs_uv,
                               const double* points, uint32_t* o_cam, uint32_t* o_pt,
                               double* o_uv, double* o_points) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt || !kept[t]) return;
  const uint32_t pi = pt_idx[t];
  o_points[3 * (size_t)pi] = points[3 * t];
  o_points[3 * (size_t)pi + 1] = points[3 * t + 1];
  o_points[3 * (size_t)pi + 2] = points[3 * t + 2];
  for (uint32_t k = track_ptr[t]; k < track_ptr[t + 1]; ++k) {
    if (!good[k]) continue;
    const uint32_t o = obs_pos[k];
    o_cam[o] = obs_cam[k];
    o_pt[o] = pi;
    o_uv[2 * (size_t)o] = obs_uv[2 * (size_t)k];
    o_uv[2 * (size_t)o + 1] = obs_uv[2 * (size_t)k + 1];
  }
}

__global__ void u8_to_u32_kernel(const uint8_t* a, uint32_t* b, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

void check_tracks(const ba_tracks* tr) {
  if (!tr) throw BadInput("null tracks");
  if (tr->n_tracks < 0 || tr->n_obs < 0 || tr->n_cams < 0 || tr->n_groups < 0)
    throw BadInput("negative size");
  if (tr->n_obs > 0xfffffff0LL || tr->n_tracks > 0xfffffff0LL)
    throw BadInput("too many tracks or observations for 32-bit indexing");
  if (tr->n_tracks > 0 && !tr->track_ptr) throw BadInput("null track_ptr");
  if (tr->n_obs > 0 && (!tr->obs_cam || !tr->obs_uv)) throw BadInput("null observation array");
  if (tr->n_cams > 0 && !tr->cam_group) throw BadInput("null cam_group");
}

// Device copies of the tracks and cameras, the triangulation, and the
// device outputs (kept, points, good).
struct TriRun {
  DevBuf<uint32_t> track_ptr, obs_cam, cam_group, err, obs_track;
  DevBuf<double> obs_uv, rot, center, intr, points, pn, ray;
  DevBuf<uint8_t> kept, good;

  void run(const ba_tracks* tr, const double* h_rot, const double* h_center, const double* h_intr,
           double thr, cudaStream_t s) {
    check_tracks(tr);
    if (!(thr > 0.0) || !std::isfinite(thr)) throw BadInput("thr_px must be finite and > 0");
    if ((tr->n_cams > 0 && (!h_rot || !h_center)) || (tr->n_groups > 0 && !h_intr))
      throw BadInput("null camera array");
    const int64_t nt = tr->n_tracks, no = tr->n_obs, nc = tr->n_cams, ng = tr->n_groups;
    auto A = [&](auto& d, int64_t n) { d.alloc(std::max<int64_t>(n, 1), s); };
    A(track_ptr, nt + 1), A(obs_cam, no), A(cam_group, nc), A(err, 1);
    A(obs_uv, 2 * no), A(rot, 9 * nc), A(center, 3 * nc), A(intr, 5 * ng), A(points, 3 * nt);
    A(kept, nt), A(good, no), A(obs_track, no), A(pn, 2 * no), A(ray, 3 * no);
    auto up = [&](auto& d, const auto* h, int64_t n) {
      if (n > 0)
        check(cudaMemcpyAsync(d.p, h, n * sizeof(*h), cudaMemcpyDefault, s), "copy in");
    };
    if (nt > 0) up(track_ptr, tr->track_ptr, nt + 1);
    up(obs_cam, tr->obs_cam, no), up(obs_uv, tr->obs_uv, 2 * no), up(cam_group, tr->cam_group, nc);
    up(rot, h_rot, 9 * nc), up(center, h_center, 3 * nc), up(intr, h_intr, 5 * ng);
    err.zero();
    TriArgs T{nt, no, nc, ng, track_ptr, obs_cam, obs_uv, cam_group, rot, center, intr, thr,
              kept, points, good, err, obs_track, pn, ray};
    // Observations outside every track's range stay unmarked (no track, not good).
    if (no > 0) {
      check(cudaMemsetAsync(obs_track.p, 0xff, 4 * no, s), "memset");
      check(cudaMemsetAsync(good.p, 0, no, s), "memset");
    }
    if (nt > 0) BA_LAUNCH(tri_check_kernel<<<grid_for(nt, 256), 256, 0, s>>>(T));
    {
      uint32_t e0 = 0;  // indices are checked before any other pass uses them
      check(cudaMemcpyAsync(&e0, err.p, 4, cudaMemcpyDeviceToHost, s), "d2h");
      check(cudaStreamSynchronize(s), "triangulate check");
      if (e0 & ERR_BAD_INDEX)
        throw BadInput("track_ptr, obs_cam or cam_group out of range (or track_ptr decreasing)");
    }
    if (nt > 0 && no > 0) {
      BA_LAUNCH(tri_undistort_kernel<<<grid_for(no, 256), 256, 0, s>>>(T));
      BA_LAUNCH(tri_point_kernel<<<grid_for(nt, kTriThreads), kTriThreads, 0, s>>>(T));
      BA_LAUNCH(tri_gate_kernel<<<grid_for(no, 256), 256, 0, s>>>(T));
      BA_LAUNCH(tri_keep_kernel<<<grid_for(nt, kTriThreads), kTriThreads, 0, s>>>(T));
    }
    uint32_t e = 0;
    check(cudaMemcpyAsync(&e, err.p, 4, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaStreamSynchronize(s), "triangulate");
    if (e & ERR_BAD_INDEX)
      throw BadInput("track_ptr, obs_cam or cam_group out of range (or track_ptr decreasing)");
  }
};

}  // namespace
}  // namespace ba

using namespace ba;

extern "C" ba_status ba_triangulate(const ba_tracks* tracks, const double* rot,
                                    const double* center, const double* intr, double thr_px,
                                    void* stream, uint8_t* kept, double* points, uint8_t* good,
                                    int64_t* n_kept) {
  return guarded([&] {
    cudaStream_t s = (cudaStream_t)stream;
    TriRun R;
    R.run(tracks, rot, center, intr, thr_px, s);
    const int64_t nt = tracks->n_tracks, no = tracks->n_obs;
    std::vector<uint8_t> hk(std::max<int64_t>(nt, 1));
    if (nt > 0)
      check(cudaMemcpyAsync(hk.data(), R.kept.p, nt, cudaMemcpyDeviceToHost, s), "d2h");
    if (kept && nt > 0) check(cudaMemcpyAsync(kept, R.kept.p, nt, cudaMemcpyDeviceToHost, s), "d2h");
    if (points && nt > 0)
      check(cudaMemcpyAsync(points, R.points.p, 24 * nt, cudaMemcpyDeviceToHost, s), "d2h");
    if (good && no > 0) check(cudaMemcpyAsync(good, R.good.p, no, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaStreamSynchronize(s), "d2h");
    if (n_kept) {
      int64_t n = 0;
      for (int64_t t = 0; t < nt; ++t) n += hk[t];
      *n_kept = n;
    }
  });
}

extern "C" ba_status ba_context_upload_tracks(ba_context* ctx, const ba_tracks* tracks,
                                              const ba_state* cams, const uint8_t* prior_mask,
                                              const double* prior, int32_t refine_intrinsics,
                                              double thr_px, int64_t* n_points, int64_t* n_obs) {
  return guarded([&] {
    if (!ctx) throw BadInput("null context");
    if (!cams) throw BadInput("null camera state");
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t s = ctx->stream;
    TriRun R;
    R.run(tracks, cams->rot, cams->center, cams->intr, thr_px, s);
    const int64_t nt = tracks->n_tracks, no = tracks->n_obs;
    // Point index of each kept track, position of each good observation.
    DevBuf<uint32_t> k32(nt + 1, s), g32(no + 1, s), pt_idx(nt + 1, s), obs_pos(no + 1, s);
    k32.zero(), g32.zero();
    if (nt > 0) BA_LAUNCH(u8_to_u32_kernel<<<grid_for(nt, 256), 256, 0, s>>>(R.kept, k32, nt));
    if (no > 0) BA_LAUNCH(u8_to_u32_kernel<<<grid_for(no, 256), 256, 0, s>>>(R.good, g32, no));
    const int64_t np = (int64_t)exclusive_scan_u32(k32, pt_idx, nt + 1, s);
    const int64_t nk = (int64_t)exclusive_scan_u32(g32, obs_pos, no + 1, s);
    DevBuf<uint32_t> o_cam(std::max<int64_t>(nk, 1), s), o_pt(std::max<int64_t>(nk, 1), s);
    DevBuf<double> o_uv(std::max<int64_t>(2 * nk, 1), s), o_points(std::max<int64_t>(3 * np, 1), s);
    if (nt > 0)
      BA_LAUNCH(compact_kernel<<<grid_for(nt, 256), 256, 0, s>>>(
          nt, R.track_ptr, R.kept, pt_idx, obs_pos, R.good, R.obs_cam, R.obs_uv, R.points, o_cam,
          o_pt, o_uv, o_points));
    check(cudaStreamSynchronize(s), "compact");
    // The problem's arrays are device pointers: the context copies them
    // device-to-device (copies use cudaMemcpyDefault).
    ba_problem P{};
    P.n_cams = tracks->n_cams, P.n_points = np, P.n_obs = nk, P.n_groups = tracks->n_groups;
    P.obs_cam = o_cam, P.obs_pt = o_pt, P.obs_uv = o_uv, P.cam_group = R.cam_group;
    P.prior_mask = prior_mask, P.prior = prior, P.refine_intrinsics = refine_intrinsics;
    ba_state S{};
    S.rot = R.rot, S.center = R.center, S.intr = R.intr, S.points = o_points;
    upload(*ctx, &P, &S, 1);
    if (n_points) *n_points = np;
    if (n_obs) *n_obs = nk;
  });
}
