// Seeded synthetic aerial surveys for bundle adjustment.
//
// Stands in for real drone datasets: a lawnmower grid of nadir cameras
// (image long side across the flight line, heading along it), optionally an
// inward-looking oblique edge ring at offset = altitude / tan(tilt), over a
// sinusoidal heightfield.  Points are kept when they land inside at least two
// images.  Observations carry Gaussian pixel noise and a fraction of uniform
// outliers.  A track keeps its outlier observations, but a track with fewer
// than `min_inlier_views` inlier observations is not emitted: the sparse
// stage's per-round gating (crates/stitch-core/src/recon/sparse.rs:389-421)
// passes a track to bundle adjustment only if at least two of its
// observations reproject within the gate from its triangulated point, which
// a track of outliers does not.  GPS priors are the true centres plus
// Gaussian noise; the initial
// state is the truth with poses rotated about a random axis and shifted in a
// random direction, points displaced by Gaussian noise, focal length scaled
// and distortion zeroed.
//
// Every random draw comes from a counter-based stream keyed on (seed, stream,
// index), so the output does not depend on the thread count.
//
// Host code only; compiled into libba_survey.so.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "camera_model.h"

extern "C" {

typedef struct survey_params {
  uint64_t seed;
  int32_t n_cams;     // total cameras, nadir + oblique
  int32_t n_points;   // points kept (visible in >= 2 images)
  double altitude;    // metres above the datum
  int32_t width, height;
  double f, cx, cy;
  double k_range;         // true k1, k2 ~ U(-k_range, k_range)
  double along_overlap;   // forward overlap of nadir images
  double across_overlap;  // side overlap of nadir images
  double oblique_frac;    // fraction of cameras on the oblique ring
  double oblique_pitch;   // degrees, e.g. -45
  double tilt_jitter_deg; // random roll/pitch of nadir cameras
  double terrain_amp, terrain_wavelength;
  double noise_px, outlier_frac;
  double prior_sigma_h, prior_sigma_v;
  double rot_perturb_deg, centre_perturb_m, point_perturb_m;
  double f_scale_init;
  int32_t refine_intrinsics;
  int32_t min_inlier_views;  // tracks with fewer inlier observations are dropped (0: keep all)
} survey_params;

typedef struct survey_arrays {
  uint32_t* obs_cam;
  uint32_t* obs_pt;
  double* obs_uv;
  uint32_t* cam_group;
  uint8_t* prior_mask;
  double* prior;
  double* rot;
  double* center;
  double* intr;
  double* points;
  double* true_rot;
  double* true_center;
  double* true_intr;
  double* true_points;
} survey_arrays;

struct survey_handle;

}  // extern "C"

namespace {

inline uint64_t splitmix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}

struct Stream {
  uint64_t key, ctr = 0;
  Stream(uint64_t seed, uint64_t stream, uint64_t index)
      : key(splitmix(splitmix(seed ^ (stream * 0xD1B54A32D192ED03ULL)) ^
                     (index * 0x9E3779B97F4A7C15ULL))) {}
  uint64_t next() { return splitmix(key + 0x632BE59BD9B4E019ULL * (++ctr)); }
  double uniform() { return (double)(next() >> 11) / (double)(1ULL << 53); }
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
  double normal() {  // Box–Muller
    double u1 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    const double u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

struct Cam {
  double R[9], C[3];
  double bx0, bx1, by0, by1;  // ground footprint bbox (with margin)
};

double terrain(const survey_params& p, double x, double y) {
  const double k = 6.283185307179586 / p.terrain_wavelength;
  return p.terrain_amp * std::sin(k * x) * std::sin(k * y);
}

// Intersections of the image corner rays with z = 0, clipped far away.
void footprint(const survey_params& p, Cam& c) {
  const double us[5][2] = {{0, 0}, {(double)p.width, 0}, {0, (double)p.height},
                           {(double)p.width, (double)p.height},
                           {p.cx, p.cy}};
  double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300;
  const double far = 10.0 * p.altitude;
  for (auto& u : us) {
    const double dc[3] = {(u[0] - p.cx) / p.f, (u[1] - p.cy) / p.f, 1.0};
    // world direction = Rᵀ dc
    double dw[3];
    for (int i = 0; i < 3; ++i)
      dw[i] = c.R[i] * dc[0] + c.R[3 + i] * dc[1] + c.R[6 + i] * dc[2];
    double t;
    if (dw[2] < -1e-9) {
      t = -c.C[2] / dw[2];
      const double h = std::sqrt(dw[0] * dw[0] + dw[1] * dw[1]) * t;
      if (h > far) t *= far / h;
    } else {
      const double h = std::sqrt(dw[0] * dw[0] + dw[1] * dw[1]);
      t = h > 0 ? far / h : 0.0;
    }
    const double gx = c.C[0] + dw[0] * t, gy = c.C[1] + dw[1] * t;
    x0 = std::min(x0, gx), x1 = std::max(x1, gx);
    y0 = std::min(y0, gy), y1 = std::max(y1, gy);
  }
  const double m = 10.0 + 2.0 * p.terrain_amp;
  c.bx0 = x0 - m, c.bx1 = x1 + m, c.by0 = y0 - m, c.by1 = y1 + m;
}

}  // namespace

struct survey_handle {
  std::vector<uint32_t> obs_cam, obs_pt;
  std::vector<double> obs_uv;
  std::vector<double> prior;
  std::vector<double> rot, center, points;
  std::vector<double> true_rot, true_center, true_points;
  double intr[5], true_intr[5];
  int64_t nc = 0, np = 0, no = 0;
};

extern "C" {

survey_handle* survey_generate(const survey_params* pp) {
  if (!pp || pp->n_cams < 2 || pp->n_points < 1) return nullptr;
  const survey_params& p = *pp;
  auto* h = new survey_handle();
  const int nc = p.n_cams;
  const int n_obl = (int)std::lround(p.oblique_frac * nc);
  const int n_nad = nc - n_obl;
  std::vector<Cam> cams(nc);

  // Nadir lawnmower: lines run north-south, spaced east-west.
  const double foot_along = p.altitude * p.height / p.f;
  const double foot_across = p.altitude * p.width / p.f;
  const double s_a = std::max(1e-3, (1.0 - p.along_overlap) * foot_along);
  const double s_c = std::max(1e-3, (1.0 - p.across_overlap) * foot_across);
  int lines = std::max(1, (int)std::lround(std::sqrt(n_nad * s_a / s_c)));
  const int per_line = (n_nad + lines - 1) / std::max(lines, 1);
  lines = (n_nad + per_line - 1) / std::max(per_line, 1);
  double hx0 = 1e300, hx1 = -1e300, hy0 = 1e300, hy1 = -1e300;
  for (int i = 0; i < n_nad; ++i) {
    const int l = i / per_line, s = i % per_line;
    const bool north = (l % 2 == 0);
    const int st = north ? s : per_line - 1 - s;
    Stream rs(p.seed, 10, (uint64_t)i);
    const double jr = rs.uniform(-1, 1) * p.tilt_jitter_deg;
    const double jp = rs.uniform(-1, 1) * p.tilt_jitter_deg;
    Cam& c = cams[i];
    bacam::from_angles(north ? 0.0 : 180.0, -90.0 + jp, jr, c.R);
    c.C[0] = l * s_c;
    c.C[1] = st * s_a;
    c.C[2] = p.altitude + rs.uniform(-1, 1) * 0.02 * p.altitude;
    hx0 = std::min(hx0, c.C[0]), hx1 = std::max(hx1, c.C[0]);
    hy0 = std::min(hy0, c.C[1]), hy1 = std::max(hy1, c.C[1]);
  }
  // Oblique edge ring: rectangle around the nadir hull offset outward by
  // altitude / tan(tilt), rounded corners, heading at the nearest hull point.
  if (n_obl > 0) {
    const double tilt = std::fabs(p.oblique_pitch) * 3.14159265358979323846 / 180.0;
    const double off = p.altitude / std::tan(tilt);
    const double W = hx1 - hx0, H = hy1 - hy0;
    const double per = 2.0 * (W + H) + 2.0 * 3.14159265358979323846 * off;
    for (int k = 0; k < n_obl; ++k) {
      double t = per * (k + 0.5) / n_obl;
      double x, y, hx, hy;  // position and the hull point it faces
      const double segs[4] = {W, H, W, H};
      int side = 0;
      bool on_arc = false;
      const double arc = 0.5 * 3.14159265358979323846 * off;
      for (;;) {
        if (t < segs[side]) break;
        t -= segs[side];
        if (t < arc) {
          on_arc = true;
          break;
        }
        t -= arc;
        side = (side + 1) % 4;
      }
      if (!on_arc) {
        switch (side) {
          case 0: hx = hx0 + t, hy = hy0, x = hx, y = hy - off; break;
          case 1: hx = hx1, hy = hy0 + t, x = hx + off, y = hy; break;
          case 2: hx = hx1 - t, hy = hy1, x = hx, y = hy + off; break;
          default: hx = hx0, hy = hy1 - t, x = hx - off, y = hy; break;
        }
      } else {
        const double a = t / off;  // radians around the corner
        switch (side) {
          case 0: hx = hx1, hy = hy0; x = hx + off * std::sin(a), y = hy - off * std::cos(a); break;
          case 1: hx = hx1, hy = hy1; x = hx + off * std::cos(a), y = hy + off * std::sin(a); break;
          case 2: hx = hx0, hy = hy1; x = hx - off * std::sin(a), y = hy + off * std::cos(a); break;
          default: hx = hx0, hy = hy0; x = hx - off * std::cos(a), y = hy - off * std::sin(a); break;
        }
      }
      const double yaw = std::atan2(hx - x, hy - y) * 180.0 / 3.14159265358979323846;
      Cam& c = cams[n_nad + k];
      Stream rs(p.seed, 11, (uint64_t)k);
      bacam::from_angles(yaw, p.oblique_pitch + rs.uniform(-1, 1) * p.tilt_jitter_deg,
                         rs.uniform(-1, 1) * p.tilt_jitter_deg, c.R);
      c.C[0] = x;
      c.C[1] = y;
      c.C[2] = p.altitude + rs.uniform(-1, 1) * 0.02 * p.altitude;
    }
  }
  for (auto& c : cams) footprint(p, c);

  // True intrinsics.
  Stream ks(p.seed, 12, 0);
  const double K[5] = {p.f, p.cx, p.cy, ks.uniform(-p.k_range, p.k_range),
                       ks.uniform(-p.k_range, p.k_range)};

  // Ground area: nadir footprints.
  double ax0 = 1e300, ax1 = -1e300, ay0 = 1e300, ay1 = -1e300;
  for (int i = 0; i < n_nad; ++i) {
    const Cam& c = cams[i];
    ax0 = std::min(ax0, c.C[0] - 0.5 * foot_across);
    ax1 = std::max(ax1, c.C[0] + 0.5 * foot_across);
    ay0 = std::min(ay0, c.C[1] - 0.5 * foot_along);
    ay1 = std::max(ay1, c.C[1] + 0.5 * foot_along);
  }
  // Camera grid over the area.
  const double cell = std::max(5.0, 0.25 * std::min(foot_along, foot_across));
  const int gx = std::max(1, (int)std::ceil((ax1 - ax0) / cell));
  const int gy = std::max(1, (int)std::ceil((ay1 - ay0) / cell));
  std::vector<std::vector<uint32_t>> grid((size_t)gx * gy);
  for (int i = 0; i < nc; ++i) {
    const Cam& c = cams[i];
    const int i0 = std::max(0, (int)std::floor((c.bx0 - ax0) / cell));
    const int i1 = std::min(gx - 1, (int)std::floor((c.bx1 - ax0) / cell));
    const int j0 = std::max(0, (int)std::floor((c.by0 - ay0) / cell));
    const int j1 = std::min(gy - 1, (int)std::floor((c.by1 - ay0) / cell));
    for (int j = j0; j <= j1; ++j)
      for (int ii = i0; ii <= i1; ++ii) grid[(size_t)j * gx + ii].push_back((uint32_t)i);
  }

  // Candidate points in index order, in parallel chunks.
  const int64_t want = p.n_points;
  const int64_t max_cand = 200 * want + 1000;
  std::vector<double> pts;
  std::vector<uint32_t> ocam, opt;
  std::vector<double> ouv;
  std::vector<double> tpts;
  pts.reserve(3 * want);
  tpts.reserve(3 * want);
  int64_t kept = 0;
  const int64_t chunk = std::max<int64_t>(65536, want / 8);
  for (int64_t base = 0; base < max_cand && kept < want; base += chunk) {
    const int64_t n = std::min(chunk, max_cand - base);
    std::vector<std::vector<std::pair<uint32_t, std::array<double, 2>>>> views(n);
    std::vector<std::array<double, 3>> X(n);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t t = 0; t < n; ++t) {
      Stream s(p.seed, 1, (uint64_t)(base + t));
      const double x = s.uniform(ax0, ax1), y = s.uniform(ay0, ay1);
      X[t] = {x, y, terrain(p, x, y)};
      const int ci = std::min(gx - 1, std::max(0, (int)((x - ax0) / cell)));
      const int cj = std::min(gy - 1, std::max(0, (int)((y - ay0) / cell)));
      for (uint32_t c : grid[(size_t)cj * gx + ci]) {
        double u[2];
        if (!bacam::project(cams[c].R, cams[c].C, K, X[t].data(), u)) continue;
        if (u[0] > 0.0 && u[1] > 0.0 && u[0] < p.width && u[1] < p.height)
          views[t].push_back({c, {u[0], u[1]}});
      }
      std::sort(views[t].begin(), views[t].end(),
                [](const auto& a, const auto& b) { return a.first < b.first; });
    }
    std::vector<double> tuv;
    for (int64_t t = 0; t < n && kept < want; ++t) {
      if (views[t].size() < 2) continue;
      Stream s(p.seed, 2, (uint64_t)(base + t));
      double Xp[3];
      for (int a = 0; a < 3; ++a) Xp[a] = X[t][a] + p.point_perturb_m * s.normal();
      tuv.clear();
      int inliers = 0;
      for (auto& v : views[t]) {
        double u0 = v.second[0] + p.noise_px * s.normal();
        double u1 = v.second[1] + p.noise_px * s.normal();
        if (s.uniform() < p.outlier_frac) {
          u0 = s.uniform(0.0, (double)p.width);
          u1 = s.uniform(0.0, (double)p.height);
        } else {
          ++inliers;
        }
        tuv.push_back(u0);
        tuv.push_back(u1);
      }
      if (inliers < p.min_inlier_views) continue;  // gated out of the round
      const uint32_t pt = (uint32_t)kept++;
      for (int a = 0; a < 3; ++a) tpts.push_back(X[t][a]);
      for (int a = 0; a < 3; ++a) pts.push_back(Xp[a]);
      for (size_t i = 0; i < views[t].size(); ++i) {
        ocam.push_back(views[t][i].first);
        opt.push_back(pt);
        ouv.push_back(tuv[2 * i]);
        ouv.push_back(tuv[2 * i + 1]);
      }
    }
  }

  h->nc = nc;
  h->np = kept;
  h->no = (int64_t)ocam.size();
  h->obs_cam = std::move(ocam);
  h->obs_pt = std::move(opt);
  h->obs_uv = std::move(ouv);
  h->points = std::move(pts);
  h->true_points = std::move(tpts);
  h->rot.resize(9 * (size_t)nc);
  h->center.resize(3 * (size_t)nc);
  h->true_rot.resize(9 * (size_t)nc);
  h->true_center.resize(3 * (size_t)nc);
  h->prior.resize(6 * (size_t)nc);
  const double dr = 3.14159265358979323846 / 180.0;
  for (int i = 0; i < nc; ++i) {
    const Cam& c = cams[i];
    std::memcpy(&h->true_rot[9 * i], c.R, sizeof c.R);
    std::memcpy(&h->true_center[3 * i], c.C, sizeof c.C);
    Stream s(p.seed, 3, (uint64_t)i);
    // Random axis (uniform on the sphere), fixed angle; random direction.
    double a[3], n2;
    do {
      for (double& v : a) v = s.normal();
      n2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    } while (n2 < 1e-12);
    const double inv = 1.0 / std::sqrt(n2);
    const double w[3] = {a[0] * inv * p.rot_perturb_deg * dr, a[1] * inv * p.rot_perturb_deg * dr,
                         a[2] * inv * p.rot_perturb_deg * dr};
    double E[9];
    bacam::exp_so3(w, E);
    bacam::matmul3(E, c.R, &h->rot[9 * i]);
    do {
      for (double& v : a) v = s.normal();
      n2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    } while (n2 < 1e-12);
    const double inv2 = 1.0 / std::sqrt(n2);
    for (int k = 0; k < 3; ++k) h->center[3 * i + k] = c.C[k] + a[k] * inv2 * p.centre_perturb_m;
    const double sg[3] = {p.prior_sigma_h, p.prior_sigma_h, p.prior_sigma_v};
    for (int k = 0; k < 3; ++k) {
      h->prior[6 * i + k] = c.C[k] + sg[k] * s.normal();
      h->prior[6 * i + 3 + k] = sg[k];
    }
  }
  std::memcpy(h->true_intr, K, sizeof K);
  h->intr[0] = K[0] * p.f_scale_init;
  h->intr[1] = K[1];
  h->intr[2] = K[2];
  h->intr[3] = 0.0;
  h->intr[4] = 0.0;
  return h;
}

void survey_sizes(const survey_handle* h, int64_t* nc, int64_t* np, int64_t* no) {
  *nc = h->nc;
  *np = h->np;
  *no = h->no;
}

void survey_copy(const survey_handle* h, const survey_arrays* a) {
  const size_t nc = h->nc, np = h->np, no = h->no;
  std::memcpy(a->obs_cam, h->obs_cam.data(), 4 * no);
  std::memcpy(a->obs_pt, h->obs_pt.data(), 4 * no);
  std::memcpy(a->obs_uv, h->obs_uv.data(), 16 * no);
  for (size_t i = 0; i < nc; ++i) a->cam_group[i] = 0, a->prior_mask[i] = 1;
  std::memcpy(a->prior, h->prior.data(), 48 * nc);
  std::memcpy(a->rot, h->rot.data(), 72 * nc);
  std::memcpy(a->center, h->center.data(), 24 * nc);
  std::memcpy(a->intr, h->intr, 40);
  std::memcpy(a->points, h->points.data(), 24 * np);
  if (a->true_rot) std::memcpy(a->true_rot, h->true_rot.data(), 72 * nc);
  if (a->true_center) std::memcpy(a->true_center, h->true_center.data(), 24 * nc);
  if (a->true_intr) std::memcpy(a->true_intr, h->true_intr, 40);
  if (a->true_points) std::memcpy(a->true_points, h->true_points.data(), 24 * np);
}

void survey_free(survey_handle* h) { delete h; }

}  // extern "C"
