// Camera model shared by the CUDA kernels and the host-side survey generator.
//
// Pinhole camera with two radial terms in full-resolution pixels, and a pose
// stored as R (world->camera, row-major) plus the centre C; a world point X
// lands at R·(X − C).  Conventions follow stitch-core's camera model
// (crates/stitch-core/src/recon/geometry.rs:13-112): OpenCV camera frame
// (x right, y down, z forward), local east/north/up world frame.
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define BA_HD __host__ __device__ __forceinline__
#else
#define BA_HD inline
#endif

namespace bacam {

// R·(X − C)   (geometry.rs:57-59)
template <typename T>
BA_HD void to_cam(const T* R, const T* C, const T* X, T* xc) {
  const T d0 = X[0] - C[0], d1 = X[1] - C[1], d2 = X[2] - C[2];
  xc[0] = R[0] * d0 + R[1] * d1 + R[2] * d2;
  xc[1] = R[3] * d0 + R[4] * d1 + R[5] * d2;
  xc[2] = R[6] * d0 + R[7] * d1 + R[8] * d2;
}

// Pose::project + Intrinsics::distort (geometry.rs:28-32, 66-72).
// K = {f, cx, cy, k1, k2}.  False when the point is not in front (z ≤ 1e-6).
template <typename T>
BA_HD bool project(const T* R, const T* C, const T* K, const T* X, T* u) {
  T xc[3];
  to_cam(R, C, X, xc);
  if (xc[2] <= T(1e-6)) return false;
  const T px = xc[0] / xc[2], py = xc[1] / xc[2];
  const T r2 = px * px + py * py;
  const T d = T(1) + K[3] * r2 + K[4] * r2 * r2;
  u[0] = K[0] * d * px + K[1];
  u[1] = K[0] * d * py + K[2];
  return true;
}

BA_HD void skew(const double* v, double* S) {
  S[0] = 0.0;   S[1] = -v[2]; S[2] = v[1];
  S[3] = v[2];  S[4] = 0.0;   S[5] = -v[0];
  S[6] = -v[1]; S[7] = v[0];  S[8] = 0.0;
}

BA_HD void matmul3(const double* A, const double* B, double* Cm) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      Cm[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] +
                      A[3 * i + 2] * B[6 + j];
}

// Rotation by `angle` about the unit `axis`: I + K sin + K² (1 − cos)
// (geometry.rs:100-103).
BA_HD void rot_axis(const double* axis, double angle, double* R) {
  double K[9], K2[9];
  skew(axis, K);
  matmul3(K, K, K2);
  const double s = sin(angle), c1 = 1.0 - cos(angle);
  for (int i = 0; i < 9; ++i)
    R[i] = ((i % 4 == 0) ? 1.0 : 0.0) + K[i] * s + K2[i] * c1;
}

// Rodrigues map; below 1e-12 rad the first-order form I + [w]x
// (geometry.rs:106-112).
BA_HD void exp_so3(const double* w, double* R) {
  const double th = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  if (th < 1e-12) {
    double K[9];
    skew(w, K);
    for (int i = 0; i < 9; ++i) R[i] = ((i % 4 == 0) ? 1.0 : 0.0) + K[i];
    return;
  }
  const double a[3] = {w[0] / th, w[1] / th, w[2] / th};
  rot_axis(a, th, R);
}

// Pose of a camera facing `yaw` (degrees clockwise from north), tilted by
// `pitch` (−90 straight down) with `roll` (geometry.rs:76-92).  Writes R.
BA_HD void from_angles(double yaw_deg, double pitch_deg, double roll_deg,
                       double* R) {
  const double dr = 3.14159265358979323846 / 180.0;
  const double sy = sin(yaw_deg * dr), cy = cos(yaw_deg * dr);
  const double sp = sin(pitch_deg * dr), cp = cos(pitch_deg * dr);
  const double x[3] = {cy, -sy, 0.0};
  const double z[3] = {sy * cp, cy * cp, sp};
  const double y[3] = {z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2],
                       z[0] * x[1] - z[1] * x[0]};
  double rwc[9] = {x[0], y[0], z[0], x[1], y[1], z[1], x[2], y[2], z[2]};
  if (fabs(roll_deg) > 1e-9) {
    const double ax[3] = {0.0, 0.0, 1.0};
    double Rr[9], T[9];
    rot_axis(ax, roll_deg * dr, Rr);
    matmul3(rwc, Rr, T);
    for (int i = 0; i < 9; ++i) rwc[i] = T[i];
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = rwc[3 * j + i];
}

}  // namespace bacam
