// ORACLE — test infrastructure only.
//
// A CPU, FP64 restatement of stitch-core's bundle adjustment
// (crates/stitch-core/src/recon/ba.rs:56-391) and of the camera model it uses
// (crates/stitch-core/src/recon/geometry.rs:15-112).  It is the checker that
// the CUDA solver is compared against, and the timed CPU baseline; it is never
// linked into, called by, or shipped with the product library.
//
// Parity pin: the reference cannot be built here (Rust toolchain absent), so
// this restatement is pinned by the reference's own known-answer test
// `recovers_perturbed_survey` (ba.rs:400-493), restated as
// `oracle_make_ref_survey` below, and by its geometry tests
// (geometry.rs:318-351).  Third-party arithmetic (nalgebra 0.33.3
// `try_inverse`, Cargo.lock) is restated with textbook algorithms: a 3x3
// adjugate inverse and a 6x6 LU with partial pivoting.
//
// Data structures follow the reference on purpose, because this file is also
// the CPU baseline: the reduced camera system is a row-wise hash map of 6x6
// blocks (ba.rs:130-153), assembled serially (ba.rs:270-331); the per-
// observation and per-point phases run in parallel with OpenMP where the
// reference uses rayon `par_iter` (ba.rs:107,145,224,235,352).
//
// Build: see oracle/Makefile (compiled with -ffp-contract=off so that, like
// Rust, no multiply-add is fused).

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// Flat SoA problem, the same field meaning as the product's C ABI.
typedef struct oracle_problem {
  int32_t n_cams, n_points, n_obs, n_groups;
  const uint32_t* obs_cam;    // [n_obs]
  const uint32_t* obs_pt;     // [n_obs], sorted ascending (ba.rs:36)
  const double* obs_uv;       // [2*n_obs]
  const uint32_t* cam_group;  // [n_cams]
  const uint8_t* prior_mask;  // [n_cams] or NULL (no priors)
  const double* prior;        // [6*n_cams]: centre xyz, sigma xyz
  int32_t refine_intrinsics;
} oracle_problem;

typedef struct oracle_state {
  double* rot;     // [9*n_cams] world->camera R, row-major
  double* center;  // [3*n_cams]
  double* intr;    // [5*n_groups]: f, cx, cy, k1, k2
  double* points;  // [3*n_points]
} oracle_state;

typedef struct oracle_stats {
  int64_t iterations;
  double initial_rms, final_rms;
  double initial_cost, final_cost;
  // Optional per-iteration log (caller-owned, log_cap entries each).
  int32_t log_cap;
  double* log_new_cost;  // cost of the trial state
  double* log_lambda;    // lambda used to build the system
  int32_t* log_pcg;      // PCG iterations
  int32_t* log_accept;   // 1 if accepted
  // Per-phase wall time, seconds.
  double t_linearise, t_point, t_assembly, t_schur, t_pcg, t_backsub, t_cost,
      t_total;
} oracle_stats;

}  // extern "C"

namespace {

enum { LOSS_CAUCHY = 0, LOSS_HUBER = 1 };

using M6 = std::array<double, 36>;  // row-major 6x6
using V6 = std::array<double, 6>;

double now_s() {
  return std::chrono::duration<double>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// ---- camera model (geometry.rs) -------------------------------------------

// R·(X − C)   (geometry.rs:57-59)
inline void to_cam(const double* R, const double* C, const double* X,
                   double* xc) {
  const double d0 = X[0] - C[0], d1 = X[1] - C[1], d2 = X[2] - C[2];
  xc[0] = R[0] * d0 + R[1] * d1 + R[2] * d2;
  xc[1] = R[3] * d0 + R[4] * d1 + R[5] * d2;
  xc[2] = R[6] * d0 + R[7] * d1 + R[8] * d2;
}

// Pose::project (geometry.rs:66-72) with Intrinsics::distort (:28-32).
inline bool project(const double* R, const double* C, const double* K,
                    const double* X, double* u) {
  double xc[3];
  to_cam(R, C, X, xc);
  if (xc[2] <= 1e-6) return false;
  const double px = xc[0] / xc[2], py = xc[1] / xc[2];
  const double r2 = px * px + py * py;
  const double d = 1.0 + K[3] * r2 + K[4] * r2 * r2;
  u[0] = K[0] * d * px + K[1];
  u[1] = K[0] * d * py + K[2];
  return true;
}

// skew (geometry.rs:95-97), row-major.
inline void skew(const double* v, double* S) {
  S[0] = 0.0;   S[1] = -v[2]; S[2] = v[1];
  S[3] = v[2];  S[4] = 0.0;   S[5] = -v[0];
  S[6] = -v[1]; S[7] = v[0];  S[8] = 0.0;
}

inline void matmul3(const double* A, const double* B, double* C) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] +
                     A[3 * i + 2] * B[6 + j];
}

// rot_axis (geometry.rs:100-103): I + K sin(a) + K² (1 − cos(a)).
void rot_axis(const double* axis, double angle, double* R) {
  double K[9], K2[9];
  skew(axis, K);
  matmul3(K, K, K2);
  const double s = std::sin(angle), c1 = 1.0 - std::cos(angle);
  for (int i = 0; i < 9; ++i)
    R[i] = ((i % 4 == 0) ? 1.0 : 0.0) + K[i] * s + K2[i] * c1;
}

// exp_so3 (geometry.rs:106-112).
void exp_so3(const double* w, double* R) {
  const double th = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  if (th < 1e-12) {
    double K[9];
    skew(w, K);
    for (int i = 0; i < 9; ++i) R[i] = ((i % 4 == 0) ? 1.0 : 0.0) + K[i];
    return;
  }
  const double a[3] = {w[0] / th, w[1] / th, w[2] / th};
  rot_axis(a, th, R);
}

// Pose::from_angles (geometry.rs:76-92): R (world->camera) and nothing else.
void from_angles(double yaw_deg, double pitch_deg, double roll_deg,
                 double* R) {
  const double dr = M_PI / 180.0;
  const double sy = std::sin(yaw_deg * dr), cy = std::cos(yaw_deg * dr);
  const double sp = std::sin(pitch_deg * dr), cp = std::cos(pitch_deg * dr);
  const double heading[3] = {sy, cy, 0.0};
  const double x[3] = {cy, -sy, 0.0};  // right
  double z[3] = {heading[0] * cp, heading[1] * cp, heading[2] * cp + sp};
  double y[3] = {z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2],
                 z[0] * x[1] - z[1] * x[0]};  // z × x
  double rwc[9] = {x[0], y[0], z[0], x[1], y[1], z[1], x[2], y[2], z[2]};
  if (std::fabs(roll_deg) > 1e-9) {
    const double ax[3] = {0.0, 0.0, 1.0};
    double Rr[9], T[9];
    rot_axis(ax, roll_deg * dr, Rr);
    matmul3(rwc, Rr, T);
    std::memcpy(rwc, T, sizeof T);
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = rwc[3 * j + i];
}

// ---- small dense algebra ----------------------------------------------------

// 3x3 inverse via the adjugate; false iff the determinant is exactly zero
// (the behaviour ba.rs:265 relies on: a singular point block is skipped).
bool inv3(const double* A, double* Ai) {
  const double c00 = A[4] * A[8] - A[5] * A[7];
  const double c01 = A[5] * A[6] - A[3] * A[8];
  const double c02 = A[3] * A[7] - A[4] * A[6];
  const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
  if (det == 0.0) return false;
  Ai[0] = c00 / det;
  Ai[1] = (A[2] * A[7] - A[1] * A[8]) / det;
  Ai[2] = (A[1] * A[5] - A[2] * A[4]) / det;
  Ai[3] = c01 / det;
  Ai[4] = (A[0] * A[8] - A[2] * A[6]) / det;
  Ai[5] = (A[2] * A[3] - A[0] * A[5]) / det;
  Ai[6] = c02 / det;
  Ai[7] = (A[1] * A[6] - A[0] * A[7]) / det;
  Ai[8] = (A[0] * A[4] - A[1] * A[3]) / det;
  return true;
}

// 6x6 inverse, LU with partial pivoting; false on an exactly zero pivot
// (ba.rs:160 then falls back to the identity).
bool inv6(const M6& A, M6& Ai) {
  double a[36];
  std::memcpy(a, A.data(), sizeof a);
  int perm[6] = {0, 1, 2, 3, 4, 5};
  for (int k = 0; k < 6; ++k) {
    int piv = k;
    double best = std::fabs(a[6 * k + k]);
    for (int i = k + 1; i < 6; ++i)
      if (std::fabs(a[6 * i + k]) > best) best = std::fabs(a[6 * i + k]), piv = i;
    if (best == 0.0) return false;
    if (piv != k) {
      for (int j = 0; j < 6; ++j) std::swap(a[6 * k + j], a[6 * piv + j]);
      std::swap(perm[k], perm[piv]);
    }
    for (int i = k + 1; i < 6; ++i) {
      const double l = a[6 * i + k] / a[6 * k + k];
      a[6 * i + k] = l;
      for (int j = k + 1; j < 6; ++j) a[6 * i + j] -= l * a[6 * k + j];
    }
  }
  // Solve L U x = P e_j for each column j.
  for (int j = 0; j < 6; ++j) {
    double x[6];
    for (int i = 0; i < 6; ++i) x[i] = (perm[i] == j) ? 1.0 : 0.0;
    for (int i = 0; i < 6; ++i)
      for (int k = 0; k < i; ++k) x[i] -= a[6 * i + k] * x[k];
    for (int i = 5; i >= 0; --i) {
      for (int k = i + 1; k < 6; ++k) x[i] -= a[6 * i + k] * x[k];
      x[i] /= a[6 * i + i];
    }
    for (int i = 0; i < 6; ++i) Ai[6 * i + j] = x[i];
  }
  return true;
}

// ---- linearisation (ba.rs:48-101) -----------------------------------------

struct Lin {
  double e[2];
  double jc[12];  // 2x6 row-major: [d/drot | d/dcentre]
  double jg[6];   // 2x3 row-major: d pred / d(f, k1, k2)
  double jp[6];   // 2x3 row-major
  double w;
};

inline double robust_weight(double e2, double sigma, int loss) {
  if (loss == LOSS_HUBER) {
    const double a = std::sqrt(e2);
    return a <= sigma ? 1.0 : sigma / a;
  }
  return 1.0 / (1.0 + e2 / (sigma * sigma));  // ba.rs:99
}

inline double robust_rho(double e2, double sigma, int loss) {
  if (loss == LOSS_HUBER) {
    const double a = std::sqrt(e2);
    return a <= sigma ? e2 : 2.0 * sigma * a - sigma * sigma;
  }
  const double s2 = sigma * sigma;
  return s2 * std::log(1.0 + e2 / s2);  // ba.rs:114
}

bool linearise(const oracle_problem& P, const oracle_state& S, int k,
               double sigma, int loss, Lin& l) {
  const uint32_t cam = P.obs_cam[k];
  const double* R = S.rot + 9 * cam;
  const double* C = S.center + 3 * cam;
  const double* K = S.intr + 5 * P.cam_group[cam];
  const double* X = S.points + 3 * (size_t)P.obs_pt[k];
  double xc[3];
  to_cam(R, C, X, xc);
  if (xc[2] <= 1e-6) return false;  // ba.rs:61
  const double f = K[0], k1 = K[3], k2 = K[4];
  const double iz = 1.0 / xc[2];
  const double px = xc[0] * iz, py = xc[1] * iz;
  const double r2 = px * px + py * py;
  const double d = 1.0 + k1 * r2 + k2 * r2 * r2;
  const double qx = px * d, qy = py * d;
  const double predx = f * qx + K[1], predy = f * qy + K[2];
  l.e[0] = P.obs_uv[2 * k] - predx;
  l.e[1] = P.obs_uv[2 * k + 1] - predy;
  // du/dp = f (d I + c p pᵀ), c = 2 (k1 + 2 k2 r2)   (ba.rs:71-78)
  const double c = 2.0 * (k1 + 2.0 * k2 * r2);
  const double a00 = (d + c * px * px) * f, a01 = (c * px * py) * f;
  const double a10 = (c * px * py) * f, a11 = (d + c * py * py) * f;
  // dp/dx (ba.rs:79)
  const double b02 = -xc[0] * iz * iz, b12 = -xc[1] * iz * iz;
  double dudx[6];
  dudx[0] = a00 * iz;
  dudx[1] = a01 * iz;
  dudx[2] = a00 * b02 + a01 * b12;
  dudx[3] = a10 * iz;
  dudx[4] = a11 * iz;
  dudx[5] = a10 * b02 + a11 * b12;
  double sk[9];
  skew(xc, sk);
  for (int r = 0; r < 2; ++r)
    for (int j = 0; j < 3; ++j) {
      double rot = 0.0, cc = 0.0, pp = 0.0;
      for (int t = 0; t < 3; ++t) {
        rot += dudx[3 * r + t] * (-sk[3 * t + j]);
        cc += dudx[3 * r + t] * (-R[3 * t + j]);
        pp += dudx[3 * r + t] * R[3 * t + j];
      }
      l.jc[6 * r + j] = rot;
      l.jc[6 * r + 3 + j] = cc;
      l.jp[3 * r + j] = pp;
    }
  if (P.refine_intrinsics) {  // ba.rs:87-98
    l.jg[0] = qx;
    l.jg[1] = f * px * r2;
    l.jg[2] = f * px * r2 * r2;
    l.jg[3] = qy;
    l.jg[4] = f * py * r2;
    l.jg[5] = f * py * r2 * r2;
  } else {
    for (int i = 0; i < 6; ++i) l.jg[i] = 0.0;
  }
  l.w = robust_weight(l.e[0] * l.e[0] + l.e[1] * l.e[1], sigma, loss);
  return true;
}

// ---- robust cost (ba.rs:103-128) -------------------------------------------

struct CostOut {
  double cost, rms;
  int64_t n;
};

CostOut robust_cost(const oracle_problem& P, const oracle_state& S,
                    double sigma, int loss) {
  double cost = 0.0, sq = 0.0;
  int64_t n = 0;
  const double behind = sigma * sigma * 10.0;  // ba.rs:116
#pragma omp parallel for reduction(+ : cost, sq, n) schedule(static)
  for (int k = 0; k < P.n_obs; ++k) {
    const uint32_t cam = P.obs_cam[k];
    double u[2];
    if (project(S.rot + 9 * cam, S.center + 3 * cam,
                S.intr + 5 * P.cam_group[cam],
                S.points + 3 * (size_t)P.obs_pt[k], u)) {
      const double ex = P.obs_uv[2 * k] - u[0], ey = P.obs_uv[2 * k + 1] - u[1];
      const double e2 = ex * ex + ey * ey;
      cost += robust_rho(e2, sigma, loss);
      sq += e2;
      n += 1;
    } else {
      cost += behind;
    }
  }
  double prior = 0.0;  // serial, ba.rs:120-126
  if (P.prior_mask) {
    for (int i = 0; i < P.n_cams; ++i) {
      if (!P.prior_mask[i]) continue;
      const double* pr = P.prior + 6 * i;
      const double dx = S.center[3 * i] - pr[0], dy = S.center[3 * i + 1] - pr[1],
                   dz = S.center[3 * i + 2] - pr[2];
      prior += (dx / pr[3]) * (dx / pr[3]) + (dy / pr[4]) * (dy / pr[4]) +
               (dz / pr[5]) * (dz / pr[5]);
    }
  }
  CostOut o;
  o.cost = cost + prior;
  o.rms = std::sqrt(sq / (double)std::max<int64_t>(n, 1));
  o.n = n;
  return o;
}

// ---- sparse block matrix (ba.rs:130-153) ------------------------------------

// Non-zero: visit each row's blocks in a seeded random order inside the
// matrix-vector product, the way the reference's HashMap (RandomState, a
// fresh hash key per map) orders them differently from run to run.  Used to
// measure the reference's own rounding sensitivity; 0 keeps one fixed order.
uint64_t g_spmv_seed = 0;
uint64_t g_sparse_instances = 0;

inline uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}

struct Sparse {
  std::vector<std::unordered_map<size_t, M6>> rows;
  uint64_t instance;
  explicit Sparse(size_t n) : rows(n), instance(++g_sparse_instances) {}
  M6& at(size_t i, size_t k) {
    auto it = rows[i].find(k);
    if (it == rows[i].end()) it = rows[i].emplace(k, M6{}).first;
    return it->second;
  }
  void add(size_t i, size_t k, const M6& m) {
    M6& d = at(i, k);
    for (int t = 0; t < 36; ++t) d[t] += m[t];
  }
  void mul(const std::vector<V6>& x, std::vector<V6>& out) const {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)rows.size(); ++i) {
      V6 s{};
      auto add = [&](size_t k, const M6& m) {
        const V6& xv = x[k];
        for (int r = 0; r < 6; ++r) {
          double acc = 0.0;
          for (int c = 0; c < 6; ++c) acc += m[6 * r + c] * xv[c];
          s[r] += acc;
        }
      };
      if (g_spmv_seed == 0) {
        for (const auto& kv : rows[i]) add(kv.first, kv.second);
      } else {
        std::vector<std::pair<size_t, const M6*>> e;
        e.reserve(rows[i].size());
        for (const auto& kv : rows[i]) e.emplace_back(kv.first, &kv.second);
        std::sort(e.begin(), e.end(),
                  [](const auto& a, const auto& b) { return a.first < b.first; });
        uint64_t h = mix64(g_spmv_seed ^ mix64(instance * 1315423911ULL + (uint64_t)i));
        for (size_t j = e.size(); j > 1; --j) {
          h = mix64(h);
          std::swap(e[j - 1], e[h % j]);
        }
        for (const auto& kv : e) add(kv.first, *kv.second);
      }
      out[i] = s;
    }
  }
};

double dot(const std::vector<V6>& a, const std::vector<V6>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) {
    double d = 0.0;
    for (int t = 0; t < 6; ++t) d += a[i][t] * b[i][t];
    s += d;
  }
  return s;
}

// Block-Jacobi PCG (ba.rs:155-196).
std::vector<V6> pcg(const Sparse& s, const std::vector<V6>& b, int max_iter,
                    int* iters_out) {
  const size_t n = b.size();
  std::vector<M6> pre(n);
  for (size_t i = 0; i < n; ++i) {
    M6 d{};
    auto it = s.rows[i].find(i);
    if (it != s.rows[i].end())
      d = it->second;
    else
      for (int t = 0; t < 6; ++t) d[7 * t] = 1.0;
    if (!inv6(d, pre[i])) {
      pre[i] = M6{};
      for (int t = 0; t < 6; ++t) pre[i][7 * t] = 1.0;
    }
  }
  auto apply = [&](const std::vector<V6>& r, std::vector<V6>& z) {
    for (size_t i = 0; i < n; ++i)
      for (int rr = 0; rr < 6; ++rr) {
        double acc = 0.0;
        for (int c = 0; c < 6; ++c) acc += pre[i][6 * rr + c] * r[i][c];
        z[i][rr] = acc;
      }
  };
  std::vector<V6> x(n, V6{}), r = b, z(n), p, q(n, V6{});
  apply(r, z);
  p = z;
  double rz = dot(r, z);
  const double b2 = std::max(dot(b, b), 1e-300);
  int spmv = 0;  // iterations = matrix-vector products performed
  for (int it = 0; it < max_iter; ++it) {
    s.mul(p, q);
    ++spmv;
    const double pq = dot(p, q);
    if (std::fabs(pq) < 1e-300) break;
    const double a = rz / pq;
    for (size_t i = 0; i < n; ++i)
      for (int t = 0; t < 6; ++t) {
        x[i][t] += p[i][t] * a;
        r[i][t] -= q[i][t] * a;
      }
    if (dot(r, r) < 1e-20 * b2) break;
    apply(r, z);
    const double rz2 = dot(r, z);
    const double beta = rz2 / rz;
    rz = rz2;
    for (size_t i = 0; i < n; ++i)
      for (int t = 0; t < 6; ++t) p[i][t] = z[i][t] + p[i][t] * beta;
  }
  if (iters_out) *iters_out = spmv;
  return x;
}

// ---- one reduced system (ba.rs:221-331) ------------------------------------

struct PointSys {
  double vinv[9];
  double v[3];
  std::vector<std::pair<size_t, std::array<double, 18>>> y;  // (block, 6x3)
};

struct System {
  std::vector<Lin> lins;
  std::vector<uint8_t> valid;
  std::vector<uint8_t> has_sys;
  std::vector<PointSys> point_sys;
  Sparse s;
  std::vector<V6> g;
  explicit System(size_t nb) : s(nb), g(nb, V6{}) {}
};

struct Timing {
  double lin = 0, point = 0, assembly = 0, schur = 0;
};

void build_system(const oracle_problem& P, const oracle_state& S,
                  const std::vector<std::pair<size_t, size_t>>& ranges,
                  double lambda, double sigma, int loss, System& sys,
                  Timing& tm) {
  const int nc = P.n_cams, np = P.n_points, no = P.n_obs;
  const bool refine = P.refine_intrinsics != 0;
  double t0 = now_s();
  // Linearise, parallel over observations (ba.rs:222-226).
  sys.lins.assign(no, Lin{});
  sys.valid.assign(no, 0);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < no; ++k)
    sys.valid[k] = linearise(P, S, k, sigma, loss, sys.lins[k]) ? 1 : 0;
  double t1 = now_s();
  tm.lin += t1 - t0;

  // Per-point blocks, parallel over points (ba.rs:229-268).
  sys.point_sys.assign(np, PointSys{});
  sys.has_sys.assign(np, 0);
#pragma omp parallel for schedule(dynamic, 256)
  for (int j = 0; j < np; ++j) {
    const size_t s0 = ranges[j].first, e0 = ranges[j].second;
    if (e0 - s0 < 2) continue;
    double vm[9] = {0}, v[3] = {0};
    PointSys ps;
    ps.y.reserve(e0 - s0 + 1);
    for (size_t k = s0; k < e0; ++k) {
      if (!sys.valid[k]) continue;
      const Lin& l = sys.lins[k];
      for (int a = 0; a < 3; ++a) {
        for (int b = 0; b < 3; ++b)
          vm[3 * a + b] += (l.jp[a] * l.jp[b] + l.jp[3 + a] * l.jp[3 + b]) * l.w;
        v[a] += (l.jp[a] * l.e[0] + l.jp[3 + a] * l.e[1]) * l.w;
      }
      std::array<double, 18> yc;
      for (int a = 0; a < 6; ++a)
        for (int b = 0; b < 3; ++b)
          yc[3 * a + b] =
              (l.jc[a] * l.jp[b] + l.jc[6 + a] * l.jp[3 + b]) * l.w;
      const uint32_t cam = P.obs_cam[k];
      ps.y.emplace_back((size_t)cam, yc);
      if (refine) {
        std::array<double, 18> yg{};
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b)
            yg[3 * a + b] =
                (l.jg[a] * l.jp[b] + l.jg[3 + a] * l.jp[3 + b]) * l.w;
        const size_t g = (size_t)nc + P.cam_group[cam];
        bool found = false;
        for (auto& ent : ps.y)
          if (ent.first == g) {
            for (int t = 0; t < 18; ++t) ent.second[t] += yg[t];
            found = true;
            break;
          }
        if (!found) ps.y.emplace_back(g, yg);
      }
    }
    for (int d = 0; d < 3; ++d) vm[4 * d] = vm[4 * d] * (1.0 + lambda) + 1e-9;
    if (!inv3(vm, ps.vinv)) continue;  // ba.rs:265
    std::memcpy(ps.v, v, sizeof v);
    sys.point_sys[j] = std::move(ps);
    sys.has_sys[j] = 1;
  }
  double t2 = now_s();
  tm.point += t2 - t1;

  // Reduced system, serial (ba.rs:270-319).
  for (int k = 0; k < no; ++k) {
    if (!sys.valid[k]) continue;
    if (!sys.has_sys[P.obs_pt[k]]) continue;
    const Lin& l = sys.lins[k];
    const size_t ci = P.obs_cam[k];
    M6 u;
    for (int a = 0; a < 6; ++a)
      for (int b = 0; b < 6; ++b)
        u[6 * a + b] = (l.jc[a] * l.jc[b] + l.jc[6 + a] * l.jc[6 + b]) * l.w;
    sys.s.add(ci, ci, u);
    for (int a = 0; a < 6; ++a)
      sys.g[ci][a] += (l.jc[a] * l.e[0] + l.jc[6 + a] * l.e[1]) * l.w;
    if (refine) {
      const size_t gi = (size_t)nc + P.cam_group[ci];
      // jg6 = [jg | 0]  (2x6)
      M6 gg{};
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
          gg[6 * a + b] = (l.jg[a] * l.jg[b] + l.jg[3 + a] * l.jg[3 + b]) * l.w;
      sys.s.add(gi, gi, gg);
      for (int a = 0; a < 3; ++a)
        sys.g[gi][a] += (l.jg[a] * l.e[0] + l.jg[3 + a] * l.e[1]) * l.w;
      M6 cg{}, gc{};
      for (int a = 0; a < 6; ++a)
        for (int b = 0; b < 3; ++b) {
          const double m = (l.jc[a] * l.jg[b] + l.jc[6 + a] * l.jg[3 + b]) * l.w;
          cg[6 * a + b] = m;
          gc[6 * b + a] = m;
        }
      sys.s.add(ci, gi, cg);
      sys.s.add(gi, ci, gc);
    }
  }
  if (P.prior_mask) {  // ba.rs:293-304
    for (int i = 0; i < nc; ++i) {
      if (!P.prior_mask[i]) continue;
      const double* pr = P.prior + 6 * i;
      M6 m{};
      for (int a = 0; a < 3; ++a) {
        const double w = 1.0 / (pr[3 + a] * pr[3 + a]);
        m[6 * (3 + a) + 3 + a] = w;
        sys.g[i][3 + a] += w * (pr[a] - S.center[3 * i + a]);
      }
      sys.s.add(i, i, m);
    }
  }
  const size_t nb = sys.g.size();
  for (size_t b = 0; b < nb; ++b) {  // ba.rs:305-319
    M6& d = sys.s.at(b, b);
    for (int k = 0; k < 6; ++k) d[7 * k] = d[7 * k] * (1.0 + lambda) + 1e-9;
    if (b >= (size_t)nc) {
      for (int k = 3; k < 6; ++k) d[7 * k] = 1.0;
      if (!refine) {
        d = M6{};
        for (int k = 0; k < 6; ++k) d[7 * k] = 1.0;
      }
    }
  }
  double t3 = now_s();
  tm.assembly += t3 - t2;

  // Schur subtraction, serial (ba.rs:320-331).
  for (int j = 0; j < np; ++j) {
    if (!sys.has_sys[j]) continue;
    const PointSys& ps = sys.point_sys[j];
    const size_t m = ps.y.size();
    // vy_b = vinv · y_bᵀ (3x6)
    std::vector<std::array<double, 18>> vy(m);
    for (size_t b = 0; b < m; ++b)
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 6; ++c)
          vy[b][6 * r + c] = ps.vinv[3 * r] * ps.y[b].second[3 * c] +
                             ps.vinv[3 * r + 1] * ps.y[b].second[3 * c + 1] +
                             ps.vinv[3 * r + 2] * ps.y[b].second[3 * c + 2];
    double vv[3];
    for (int r = 0; r < 3; ++r)
      vv[r] = ps.vinv[3 * r] * ps.v[0] + ps.vinv[3 * r + 1] * ps.v[1] +
              ps.vinv[3 * r + 2] * ps.v[2];
    for (size_t a = 0; a < m; ++a) {
      const auto& ya = ps.y[a].second;
      V6& ga = sys.g[ps.y[a].first];
      for (int r = 0; r < 6; ++r)
        ga[r] -= ya[3 * r] * vv[0] + ya[3 * r + 1] * vv[1] + ya[3 * r + 2] * vv[2];
      for (size_t b = 0; b < m; ++b) {
        M6 mm;
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 6; ++c)
            mm[6 * r + c] = -(ya[3 * r] * vy[b][c] + ya[3 * r + 1] * vy[b][6 + c] +
                              ya[3 * r + 2] * vy[b][12 + c]);
        sys.s.add(ps.y[a].first, ps.y[b].first, mm);
      }
    }
  }
  tm.schur += now_s() - t3;
}

// Apply dx to a copy of the state (ba.rs:338-366).
void apply_update(const oracle_problem& P, const System& sys,
                  const std::vector<V6>& dx, const oracle_state& cur,
                  oracle_state& out) {
  const int nc = P.n_cams, ng = P.n_groups, np = P.n_points;
  for (int i = 0; i < nc; ++i) {
    const double w[3] = {dx[i][0], dx[i][1], dx[i][2]};
    double E[9], Rn[9];
    exp_so3(w, E);
    matmul3(E, cur.rot + 9 * i, Rn);
    std::memcpy(out.rot + 9 * i, Rn, sizeof Rn);
    for (int a = 0; a < 3; ++a)
      out.center[3 * i + a] = cur.center[3 * i + a] + dx[i][3 + a];
  }
  std::memcpy(out.intr, cur.intr, sizeof(double) * 5 * ng);
  if (P.refine_intrinsics) {
    for (int g = 0; g < ng; ++g) {
      const V6& d = dx[nc + g];
      out.intr[5 * g + 0] += d[0];
      out.intr[5 * g + 3] += d[1];
      out.intr[5 * g + 4] += d[2];
    }
  }
#pragma omp parallel for schedule(dynamic, 256)
  for (int j = 0; j < np; ++j) {
    double* X = out.points + 3 * (size_t)j;
    const double* X0 = cur.points + 3 * (size_t)j;
    if (!sys.has_sys[j]) {
      X[0] = X0[0], X[1] = X0[1], X[2] = X0[2];
      continue;
    }
    const PointSys& ps = sys.point_sys[j];
    double rhs[3] = {ps.v[0], ps.v[1], ps.v[2]};
    for (const auto& ent : ps.y) {
      const V6& d = dx[ent.first];
      for (int r = 0; r < 3; ++r) {
        double acc = 0.0;
        for (int c = 0; c < 6; ++c) acc += ent.second[3 * c + r] * d[c];
        rhs[r] -= acc;
      }
    }
    for (int r = 0; r < 3; ++r)
      X[r] = X0[r] + (ps.vinv[3 * r] * rhs[0] + ps.vinv[3 * r + 1] * rhs[1] +
                      ps.vinv[3 * r + 2] * rhs[2]);
  }
}

std::vector<std::pair<size_t, size_t>> point_ranges(const oracle_problem& P) {
  // ba.rs:203-214
  std::vector<std::pair<size_t, size_t>> ranges(P.n_points, {0, 0});
  size_t i = 0;
  const size_t no = P.n_obs;
  while (i < no) {
    const uint32_t pt = P.obs_pt[i];
    const size_t s = i;
    while (i < no && P.obs_pt[i] == pt) ++i;
    ranges[pt] = {s, i};
  }
  return ranges;
}

struct OwnedState {
  std::vector<double> rot, center, intr, points;
  OwnedState(const oracle_problem& P)
      : rot(9 * (size_t)P.n_cams), center(3 * (size_t)P.n_cams),
        intr(5 * (size_t)P.n_groups), points(3 * (size_t)P.n_points) {}
  oracle_state view() {
    return oracle_state{rot.data(), center.data(), intr.data(), points.data()};
  }
};

void copy_state(const oracle_problem& P, const oracle_state& a,
                oracle_state& b) {
  std::memcpy(b.rot, a.rot, sizeof(double) * 9 * P.n_cams);
  std::memcpy(b.center, a.center, sizeof(double) * 3 * P.n_cams);
  std::memcpy(b.intr, a.intr, sizeof(double) * 5 * P.n_groups);
  std::memcpy(b.points, a.points, sizeof(double) * 3 * (size_t)P.n_points);
}

struct ThreadScope {
#ifdef _OPENMP
  int saved;
  explicit ThreadScope(int n) : saved(omp_get_max_threads()) {
    if (n > 0) omp_set_num_threads(n);
  }
  ~ThreadScope() { omp_set_num_threads(saved); }
#else
  explicit ThreadScope(int) {}
#endif
};

}  // namespace

extern "C" {

int oracle_version(void) { return 1; }

void oracle_set_spmv_shuffle(uint64_t seed) { g_spmv_seed = seed; }

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// bundle_adjust (ba.rs:198-391).  Mutates `st` in place.
int oracle_bundle_adjust(const oracle_problem* P, oracle_state* st,
                         int32_t max_iter, double sigma_px, int32_t loss,
                         int32_t pcg_max_iter, int32_t n_threads,
                         oracle_stats* out) {
  ThreadScope ts(n_threads);
  const double T0 = now_s();
  const int nc = P->n_cams, ng = P->n_groups;
  const size_t nb = (size_t)nc + ng;
  const auto ranges = point_ranges(*P);
  Timing tm;
  double t_pcg = 0, t_back = 0, t_cost = 0;
  double tc = now_s();
  CostOut c0 = robust_cost(*P, *st, sigma_px, loss);
  t_cost += now_s() - tc;
  double cost = c0.cost;
  double lambda = 1e-4;
  int64_t iterations = 0;
  OwnedState old(*P);
  oracle_state oldv = old.view();
  for (int it = 0; it < max_iter; ++it) {
    ++iterations;
    System sys(nb);
    build_system(*P, *st, ranges, lambda, sigma_px, loss, sys, tm);
    double tp = now_s();
    int pcg_iters = 0;
    std::vector<V6> dx = pcg(sys.s, sys.g, pcg_max_iter, &pcg_iters);
    t_pcg += now_s() - tp;
    double tb = now_s();
    copy_state(*P, *st, oldv);  // snapshot (ba.rs:335-337)
    apply_update(*P, sys, dx, oldv, *st);
    t_back += now_s() - tb;
    tc = now_s();
    const double new_cost = robust_cost(*P, *st, sigma_px, loss).cost;
    t_cost += now_s() - tc;
    bool accepted = false;
    bool stop = false;
    const double lambda_used = lambda;
    if (new_cost < cost) {  // ba.rs:368-383
      accepted = true;
      const double rel = (cost - new_cost) / std::max(cost, 1e-12);
      cost = new_cost;
      lambda = std::max(lambda / 3.0, 1e-9);
      if (rel < 1e-6) stop = true;
    } else {
      copy_state(*P, oldv, *st);
      lambda *= 5.0;
      if (lambda > 1e6) stop = true;
    }
    if (out && out->log_cap > it) {
      if (out->log_new_cost) out->log_new_cost[it] = new_cost;
      if (out->log_lambda) out->log_lambda[it] = lambda_used;
      if (out->log_pcg) out->log_pcg[it] = pcg_iters;
      if (out->log_accept) out->log_accept[it] = accepted ? 1 : 0;
    }
    if (stop) break;
  }
  tc = now_s();
  CostOut c1 = robust_cost(*P, *st, sigma_px, loss);
  t_cost += now_s() - tc;
  if (out) {
    out->iterations = iterations;
    out->initial_rms = c0.rms;
    out->final_rms = c1.rms;
    out->initial_cost = c0.cost;
    out->final_cost = c1.cost;
    out->t_linearise = tm.lin;
    out->t_point = tm.point;
    out->t_assembly = tm.assembly;
    out->t_schur = tm.schur;
    out->t_pcg = t_pcg;
    out->t_backsub = t_back;
    out->t_cost = t_cost;
    out->t_total = now_s() - T0;
  }
  return 0;
}

// robust_cost (ba.rs:103-128): writes cost, rms, count.
int oracle_robust_cost(const oracle_problem* P, const oracle_state* st,
                       double sigma_px, int32_t loss, double* cost,
                       double* rms, int64_t* n) {
  CostOut c = robust_cost(*P, *st, sigma_px, loss);
  *cost = c.cost;
  *rms = c.rms;
  *n = c.n;
  return 0;
}

// linearise (ba.rs:56-101) for every observation.  e[2n], jc[12n], jg[6n],
// jp[6n], w[n], valid[n]; invalid rows are zero.
int oracle_linearise(const oracle_problem* P, const oracle_state* st,
                     double sigma_px, int32_t loss, double* e, double* jc,
                     double* jg, double* jp, double* w, uint8_t* valid) {
  for (int k = 0; k < P->n_obs; ++k) {
    Lin l{};
    const bool ok = linearise(*P, *st, k, sigma_px, loss, l);
    if (!ok) l = Lin{};
    valid[k] = ok ? 1 : 0;
    std::memcpy(e + 2 * (size_t)k, l.e, sizeof l.e);
    std::memcpy(jc + 12 * (size_t)k, l.jc, sizeof l.jc);
    std::memcpy(jg + 6 * (size_t)k, l.jg, sizeof l.jg);
    std::memcpy(jp + 6 * (size_t)k, l.jp, sizeof l.jp);
    w[k] = l.w;
  }
  return 0;
}

// One LM system at damping `lambda` (ba.rs:221-366) without the accept step:
// the dense reduced matrix S[(6 nb)^2] (row-major; may be NULL), g[6 nb], the
// PCG solution dx[6 nb], per-point flag `has_sys`, the trial state `trial`
// and its cost.  For small problems (tests).
int oracle_lm_step(const oracle_problem* P, const oracle_state* st,
                   double lambda, double sigma_px, int32_t loss,
                   int32_t pcg_max_iter, double* S_dense, double* g_out,
                   double* dx_out, uint8_t* has_sys, int32_t* pcg_iters,
                   oracle_state* trial, double* trial_cost) {
  const size_t nb = (size_t)P->n_cams + P->n_groups;
  const auto ranges = point_ranges(*P);
  System sys(nb);
  Timing tm;
  build_system(*P, *st, ranges, lambda, sigma_px, loss, sys, tm);
  if (S_dense) {
    std::memset(S_dense, 0, sizeof(double) * 36 * nb * nb);
    for (size_t i = 0; i < nb; ++i)
      for (const auto& kv : sys.s.rows[i])
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 6; ++c)
            S_dense[(6 * i + r) * 6 * nb + 6 * kv.first + c] = kv.second[6 * r + c];
  }
  for (size_t i = 0; i < nb; ++i)
    for (int t = 0; t < 6; ++t) g_out[6 * i + t] = sys.g[i][t];
  int it = 0;
  std::vector<V6> dx = pcg(sys.s, sys.g, pcg_max_iter, &it);
  if (pcg_iters) *pcg_iters = it;
  for (size_t i = 0; i < nb; ++i)
    for (int t = 0; t < 6; ++t) dx_out[6 * i + t] = dx[i][t];
  for (int j = 0; j < P->n_points; ++j) has_sys[j] = sys.has_sys[j];
  apply_update(*P, sys, dx, *st, *trial);
  *trial_cost = robust_cost(*P, *trial, sigma_px, loss).cost;
  return 0;
}

// exp_so3 / from_angles / project exposed for the geometry pins.
void oracle_exp_so3(const double* w, double* R) { exp_so3(w, R); }
void oracle_from_angles(double yaw, double pitch, double roll, double* R) {
  from_angles(yaw, pitch, roll, R);
}
int oracle_project(const double* R, const double* C, const double* K,
                   const double* X, double* u) {
  return project(R, C, K, X, u) ? 1 : 0;
}
// Intrinsics::undistort (geometry.rs:35-44), 8 fixed-point steps.
void oracle_undistort(const double* K, const double* u, double* p) {
  const double qx = (u[0] - K[1]) / K[0], qy = (u[1] - K[2]) / K[0];
  double px = qx, py = qy;
  for (int i = 0; i < 8; ++i) {
    const double r2 = px * px + py * py;
    const double d = 1.0 + K[3] * r2 + K[4] * r2 * r2;
    px = qx / d;
    py = qy / d;
  }
  p[0] = px;
  p[1] = py;
}

// Symmetric 4x4 eigen-decomposition by cyclic Jacobi rotations (the
// reference calls nalgebra's symmetric_eigen, a third-party routine not in
// the reference tree; any accurate symmetric solver gives the same
// eigenvector of a simple eigenvalue up to sign and rounding).
static void jacobi4(double A[4][4], double V[4][4]) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) V[i][j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < 4; ++i) {
      diag += A[i][i] * A[i][i];
      for (int j = i + 1; j < 4; ++j) off += A[i][j] * A[i][j];
    }
    if (off <= 1e-34 * diag || off == 0.0) break;
    for (int p = 0; p < 3; ++p)
      for (int q = p + 1; q < 4; ++q) {
        if (A[p][q] == 0.0) continue;
        const double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) /
                         (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < 4; ++k) {  // A <- J^T A J
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - sn * akq;
          A[k][q] = sn * akp + c * akq;
        }
        for (int k = 0; k < 4; ++k) {
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - sn * aqk;
          A[q][k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < 4; ++k) {
          const double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - sn * vkq;
          V[k][q] = sn * vkp + c * vkq;
        }
      }
  }
}

// triangulate (geometry.rs:115-144): linear multi-view triangulation from
// undistorted normalised coordinates via the smallest eigenvector of A^T A.
static bool triangulate_track(int n, const double* const* R, const double* const* C,
                              const double* p, double* X) {
  if (n < 2) return false;
  double ata[4][4] = {};
  for (int i = 0; i < n; ++i) {
    const double* Ri = R[i];
    double t[3];
    for (int k = 0; k < 3; ++k)
      t[k] = -(Ri[3 * k] * C[i][0] + Ri[3 * k + 1] * C[i][1] + Ri[3 * k + 2] * C[i][2]);
    const double row0[4] = {Ri[0], Ri[1], Ri[2], t[0]};
    const double row1[4] = {Ri[3], Ri[4], Ri[5], t[1]};
    const double row2[4] = {Ri[6], Ri[7], Ri[8], t[2]};
    double a0[4], a1[4];
    for (int c = 0; c < 4; ++c) {
      a0[c] = p[2 * i] * row2[c] - row0[c];
      a1[c] = p[2 * i + 1] * row2[c] - row1[c];
    }
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) ata[r][c] += a0[r] * a0[c] + a1[r] * a1[c];
  }
  double V[4][4];
  jacobi4(ata, V);
  int best = 0;
  for (int i = 1; i < 4; ++i)
    if (ata[i][i] < ata[best][best]) best = i;
  const double v3 = V[3][best];
  if (std::fabs(v3) < 1e-12) return false;
  for (int k = 0; k < 3; ++k) X[k] = V[k][best] / v3;
  return true;
}

// One round's triangulation and reprojection gating of every track
// (sparse.rs:389-421): triangulate from undistorted observations, keep the
// observations that reproject within thr pixels, keep the track if at least
// two remain and their rays span more than 2 degrees (3+ views) or 6 degrees
// (2 views; geometry.rs:146-156 max_ray_angle).  Tracks in CSR form
// (track_ptr[n_tracks + 1], obs_cam, obs_uv); cameras: rot (row-major),
// center, intr per group, cam_group.  Outputs kept[n_tracks],
// points[3 * n_tracks], good[n_obs].  Returns the number of kept tracks.
int64_t oracle_triangulate(int64_t n_tracks, const uint32_t* track_ptr, const uint32_t* obs_cam,
                           const double* obs_uv, const double* rot, const double* center,
                           const double* intr, const uint32_t* cam_group, double thr,
                           uint8_t* kept, double* points, uint8_t* good, int n_threads) {
  int64_t nk = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : nk) num_threads(n_threads)
  for (int64_t t = 0; t < n_tracks; ++t) {
    const uint32_t b = track_ptr[t], e = track_ptr[t + 1];
    const int n = (int)(e - b);
    std::vector<const double*> Rs(n), Cs(n);
    std::vector<double> pn(2 * (size_t)n);
    for (int i = 0; i < n; ++i) {
      const uint32_t c = obs_cam[b + i];
      Rs[i] = rot + 9 * (size_t)c;
      Cs[i] = center + 3 * (size_t)c;
      oracle_undistort(intr + 5 * (size_t)cam_group[c], obs_uv + 2 * (size_t)(b + i), &pn[2 * i]);
      good[b + i] = 0;
    }
    double X[3] = {0, 0, 0};
    kept[t] = 0;
    points[3 * t] = points[3 * t + 1] = points[3 * t + 2] = 0.0;
    if (!triangulate_track(n, Rs.data(), Cs.data(), pn.data(), X)) continue;
    int ng = 0;
    for (int i = 0; i < n; ++i) {
      const uint32_t c = obs_cam[b + i];
      double u[2];
      if (!project(Rs[i], Cs[i], intr + 5 * (size_t)cam_group[c], X, u)) continue;
      const double dx = u[0] - obs_uv[2 * (size_t)(b + i)], dy = u[1] - obs_uv[2 * (size_t)(b + i) + 1];
      if (std::sqrt(dx * dx + dy * dy) < thr) good[b + i] = 1, ++ng;
    }
    if (ng < 2) {
      for (int i = 0; i < n; ++i) good[b + i] = 0;
      continue;
    }
    // max_ray_angle over the kept observations' unit rays (geometry.rs:146-156)
    std::vector<double> ray(3 * (size_t)n);
    for (int i = 0; i < n; ++i) {
      double r[3];
      for (int k = 0; k < 3; ++k) r[k] = X[k] - Cs[i][k];
      const double l = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
      for (int k = 0; k < 3; ++k) ray[3 * i + k] = r[k] / l;
    }
    double best = 0.0;
    for (int i = 0; i < n; ++i) {
      if (!good[b + i]) continue;
      for (int j = i + 1; j < n; ++j) {
        if (!good[b + j]) continue;
        double d = ray[3 * i] * ray[3 * j] + ray[3 * i + 1] * ray[3 * j + 1] +
                   ray[3 * i + 2] * ray[3 * j + 2];
        d = std::min(1.0, std::max(-1.0, d));
        best = std::max(best, std::acos(d));
      }
    }
    const double deg = best * 180.0 / M_PI;
    const bool ok = ng >= 3 ? deg > 2.0 : deg > 6.0;
    if (!ok) {
      for (int i = 0; i < n; ++i) good[b + i] = 0;
      continue;
    }
    kept[t] = 1;
    for (int k = 0; k < 3; ++k) points[3 * t + k] = X[k];
    ++nk;
  }
  return nk;
}

// ---- epipolar geometry: pair pruning and fundamental-matrix RANSAC --------

// Symmetric NxN eigen-decomposition by cyclic Jacobi rotations (as jacobi4;
// stands in for nalgebra's symmetric_eigen, geometry.rs:209 and :131).
extern "C++" {
template <int N>
static void jacobi_sym(double A[N][N], double V[N][N]) {
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) V[i][j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < N; ++i) {
      diag += A[i][i] * A[i][i];
      for (int j = i + 1; j < N; ++j) off += A[i][j] * A[i][j];
    }
    if (off <= 1e-34 * diag || off == 0.0) break;
    for (int p = 0; p < N - 1; ++p)
      for (int q = p + 1; q < N; ++q) {
        if (A[p][q] == 0.0) continue;
        const double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) /
                         (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < N; ++k) {
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - sn * akq;
          A[k][q] = sn * akp + c * akq;
        }
        for (int k = 0; k < N; ++k) {
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - sn * aqk;
          A[q][k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < N; ++k) {
          const double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - sn * vkq;
          V[k][q] = sn * vkp + c * vkq;
        }
      }
  }
}
}  // extern "C++"

// normalise (geometry.rs:161-183) of one side (side 0: a, 1: b) of the
// correspondences idx[0..n) of uv (4 values per correspondence: a then b):
// centroid as a running sum of p/n, mean distance to it, scale sqrt(2)/d.
static void ep_normalise(const double* uv, const uint32_t* idx, int n, int side,
                         double* out, double T[9]) {
  const double nn = (double)n;
  double mx = 0.0, my = 0.0;
  for (int i = 0; i < n; ++i) {
    const double* p = uv + 4 * (size_t)idx[i] + 2 * side;
    mx = mx + p[0] / nn;
    my = my + p[1] / nn;
  }
  double d = 0.0;
  for (int i = 0; i < n; ++i) {
    const double* p = uv + 4 * (size_t)idx[i] + 2 * side;
    const double dx = p[0] - mx, dy = p[1] - my;
    d += std::sqrt(dx * dx + dy * dy);
  }
  d /= nn;
  const double s = d > 1e-12 ? M_SQRT2 / d : 1.0;
  const double t[9] = {s, 0.0, -s * mx, 0.0, s, -s * my, 0.0, 0.0, 1.0};
  std::memcpy(T, t, sizeof t);
  for (int i = 0; i < n; ++i) {
    const double* p = uv + 4 * (size_t)idx[i] + 2 * side;
    out[2 * i] = (p[0] - mx) * s;
    out[2 * i + 1] = (p[1] - my) * s;
  }
}

// fundamental (geometry.rs:186-230): normalised 8-point F from the
// correspondences idx[0..n), smallest eigenvector of the 9x9 normal matrix,
// rank 2 by removing the smallest singular value (F - (F v) v^T, v the right
// singular vector of the smallest singular value, from the eigenvectors of
// F^T F), denormalised T_b^T F T_a and scaled to unit Frobenius norm.
static bool ep_fundamental(const double* uv, const uint32_t* idx, int n, double F[9]) {
  if (n < 8) return false;
  std::vector<double> na(2 * (size_t)n), nb(2 * (size_t)n);
  double ta[9], tb[9];
  ep_normalise(uv, idx, n, 0, na.data(), ta);
  ep_normalise(uv, idx, n, 1, nb.data(), tb);
  double m[9][9] = {};
  for (int i = 0; i < n; ++i) {
    const double p0 = na[2 * i], p1 = na[2 * i + 1], q0 = nb[2 * i], q1 = nb[2 * i + 1];
    const double row[9] = {q0 * p0, q0 * p1, q0, q1 * p0, q1 * p1, q1, p0, p1, 1.0};
    for (int r = 0; r < 9; ++r)
      for (int c = 0; c < 9; ++c) m[r][c] += row[r] * row[c];
  }
  double V[9][9];
  jacobi_sym<9>(m, V);
  int k = 0;
  for (int i = 1; i < 9; ++i)
    if (m[i][i] < m[k][k]) k = i;
  double fm[9];
  for (int i = 0; i < 9; ++i) fm[i] = V[i][k];
  double ftf[3][3], W[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      ftf[r][c] = fm[r] * fm[c] + fm[3 + r] * fm[3 + c] + fm[6 + r] * fm[6 + c];
  jacobi_sym<3>(ftf, W);
  int j = 0;
  for (int i = 1; i < 3; ++i)
    if (ftf[i][i] < ftf[j][j]) j = i;
  const double v[3] = {W[0][j], W[1][j], W[2][j]};
  double f2[9];
  for (int r = 0; r < 3; ++r) {
    const double fv = fm[3 * r] * v[0] + fm[3 * r + 1] * v[1] + fm[3 * r + 2] * v[2];
    for (int c = 0; c < 3; ++c) f2[3 * r + c] = fm[3 * r + c] - fv * v[c];
  }
  double tbt[9], tmp[9], full[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) tbt[3 * r + c] = tb[3 * c + r];
  matmul3(tbt, f2, tmp);
  matmul3(tmp, ta, full);
  double nrm = 0.0;
  for (int i = 0; i < 9; ++i) nrm += full[i] * full[i];
  nrm = std::sqrt(nrm);
  if (!(nrm > 1e-15)) return false;
  for (int i = 0; i < 9; ++i) F[i] = full[i] / nrm;
  return true;
}

// sampson (geometry.rs:233-246): squared Sampson distance, f64::MAX when the
// gradient norm is below 1e-18.
static double ep_sampson(const double* F, double ax, double ay, double bx, double by) {
  const double f0 = F[0] * ax + F[1] * ay + F[2];
  const double f1 = F[3] * ax + F[4] * ay + F[5];
  const double f2 = F[6] * ax + F[7] * ay + F[8];
  const double g0 = F[0] * bx + F[3] * by + F[6];
  const double g1 = F[1] * bx + F[4] * by + F[7];
  const double e = bx * f0 + by * f1 + f2;
  const double d = f0 * f0 + f1 * f1 + g0 * g0 + g1 * g1;
  return d < 1e-18 ? 1.7976931348623157e308 : e * e / d;
}

// ransac_fundamental (geometry.rs:248-300) per pair: pairs p own the
// correspondences match_ptr[p]..match_ptr[p+1] of uv (u_a, v_a, u_b, v_b).
// xorshift64 (13, 7, 17) from seed | 1, index = state % n, eight distinct
// indices per hypothesis (repeats redrawn); the first hypothesis with the
// most inliers (Sampson^2 < thresh^2) wins; one refit on its inliers is
// kept when it has at least as many.  Fewer than 12 correspondences: none.
// Outputs: inlier u8[n_matches], n_inliers, best hypothesis (-1: none),
// refit taken (0/1).
void oracle_ransac_fundamental(int64_t n_pairs, const uint32_t* match_ptr, const double* uv,
                               const uint64_t* seed, double thresh, int iters, uint8_t* inlier,
                               int32_t* n_inl, int32_t* best_hyp, uint8_t* refit,
                               int n_threads) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads)
  for (int64_t p = 0; p < n_pairs; ++p) {
    const uint32_t b = match_ptr[p];
    const int n = (int)(match_ptr[p + 1] - b);
    const double* U = uv + 4 * (size_t)b;
    for (int i = 0; i < n; ++i) inlier[b + i] = 0;
    n_inl[p] = 0, best_hyp[p] = -1, refit[p] = 0;
    if (n < 12) continue;
    const double t2 = thresh * thresh;
    uint64_t s = seed[p] | 1;
    auto rnd = [&](uint64_t m) {
      s ^= s << 13;
      s ^= s >> 7;
      s ^= s << 17;
      return (uint32_t)(s % m);
    };
    std::vector<uint32_t> best, cur;
    uint32_t idx[8];
    double F[9];
    for (int it = 0; it < iters; ++it) {
      int k = 0;
      while (k < 8) {
        const uint32_t c = rnd((uint64_t)n);
        bool dup = false;
        for (int q = 0; q < k; ++q) dup |= idx[q] == c;
        if (!dup) idx[k++] = c;
      }
      if (!ep_fundamental(U, idx, 8, F)) continue;
      cur.clear();
      for (int i = 0; i < n; ++i)
        if (ep_sampson(F, U[4 * i], U[4 * i + 1], U[4 * i + 2], U[4 * i + 3]) < t2)
          cur.push_back((uint32_t)i);
      if (cur.size() > best.size()) best.swap(cur), best_hyp[p] = it;
    }
    if (best.size() >= 8 && ep_fundamental(U, best.data(), (int)best.size(), F)) {
      cur.clear();
      for (int i = 0; i < n; ++i)
        if (ep_sampson(F, U[4 * i], U[4 * i + 1], U[4 * i + 2], U[4 * i + 3]) < t2)
          cur.push_back((uint32_t)i);
      if (cur.size() >= best.size()) best.swap(cur), refit[p] = 1;
    }
    for (uint32_t i : best) inlier[b + i] = 1;
    n_inl[p] = (int32_t)best.size();
  }
}

// pair_fits (sparse.rs:620-645): median Sampson error in pixels (times the
// first camera's focal length) of a pair's matches under the current poses,
// E = [t]x R with R = R_b R_a^T, t = R_b (C_a - C_b), on undistorted
// normalised coordinates; f64::MAX for a pair without matches.
void oracle_pair_fits(int64_t n_pairs, const uint32_t* pair_cam, const uint32_t* match_ptr,
                      const double* uv, const double* rot, const double* center,
                      const double* intr, const uint32_t* cam_group, double* median,
                      int n_threads) {
#pragma omp parallel for schedule(dynamic, 4) num_threads(n_threads)
  for (int64_t p = 0; p < n_pairs; ++p) {
    const uint32_t ca = pair_cam[2 * p], cb = pair_cam[2 * p + 1];
    const double* Ra = rot + 9 * (size_t)ca;
    const double* Rb = rot + 9 * (size_t)cb;
    const double* Ka = intr + 5 * (size_t)cam_group[ca];
    const double* Kb = intr + 5 * (size_t)cam_group[cb];
    double RaT[9], R[9], t[3], S[9], E[9];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) RaT[3 * r + c] = Ra[3 * c + r];
    matmul3(Rb, RaT, R);
    const double d[3] = {center[3 * ca] - center[3 * cb], center[3 * ca + 1] - center[3 * cb + 1],
                         center[3 * ca + 2] - center[3 * cb + 2]};
    for (int r = 0; r < 3; ++r) t[r] = Rb[3 * r] * d[0] + Rb[3 * r + 1] * d[1] + Rb[3 * r + 2] * d[2];
    skew(t, S);
    matmul3(S, R, E);
    const uint32_t b = match_ptr[p], e = match_ptr[p + 1];
    if (e == b) {
      median[p] = 1.7976931348623157e308;
      continue;
    }
    std::vector<double> errs(e - b);
    for (uint32_t i = b; i < e; ++i) {
      double x1[2], x2[2];
      oracle_undistort(Ka, uv + 4 * (size_t)i, x1);
      oracle_undistort(Kb, uv + 4 * (size_t)i + 2, x2);
      errs[i - b] = std::sqrt(ep_sampson(E, x1[0], x1[1], x2[0], x2[1])) * Ka[0];
    }
    auto key = [](double z) {  // f64::total_cmp
      uint64_t u;
      std::memcpy(&u, &z, 8);
      return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
    };
    std::sort(errs.begin(), errs.end(), [&](double x, double y) { return key(x) < key(y); });
    median[p] = errs[errs.size() / 2];
  }
}

// Per-camera summary of a finished sparse reconstruction (sparse.rs:470-483,
// 515-533) and the f32 points of sparse.ply (mod.rs:31-35).  Shared-point
// counts per ordered pair of distinct cameras of each point and each
// camera's observed depths, as the reference's loops over `kept` collect
// them; neighbours sorted by count, best first (equal counts by ascending
// camera index: the reference takes them in HashMap order), at most max_nb;
// depth range (d[n/20] * 0.8, d[19n/20] * 1.25) of the depths in total order
// when n >= 10, else (0.3 agl, 3 agl).  Observations sorted by point.
void oracle_sparse_summary(int64_t nc, int64_t np, int64_t no, const uint32_t* obs_cam,
                           const uint32_t* obs_pt, const double* rot, const double* center,
                           const double* points, int max_nb, double agl, uint32_t* nb,
                           uint32_t* shared, int32_t* n_nb, double* range, float* pts32) {
  std::vector<std::unordered_map<uint32_t, uint32_t>> sh(nc);
  std::vector<std::vector<double>> depths(nc);
  for (int64_t b = 0, e; b < no; b = e) {
    for (e = b + 1; e < no && obs_pt[e] == obs_pt[b]; ++e) {
    }
    const double* X = points + 3 * (size_t)obs_pt[b];
    for (int64_t i = b; i < e; ++i) {
      const uint32_t a = obs_cam[i];
      double xc[3];
      to_cam(rot + 9 * (size_t)a, center + 3 * (size_t)a, X, xc);
      depths[a].push_back(xc[2]);
      for (int64_t j = b; j < e; ++j)
        if (obs_cam[j] != a) ++sh[a][obs_cam[j]];
    }
  }
  auto key = [](double z) {
    uint64_t u;
    std::memcpy(&u, &z, 8);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
  };
  for (int64_t a = 0; a < nc; ++a) {
    std::vector<std::pair<uint32_t, uint32_t>> v(sh[a].begin(), sh[a].end());
    std::sort(v.begin(), v.end(), [](const auto& x, const auto& y) {
      return x.second != y.second ? x.second > y.second : x.first < y.first;
    });
    const int k = (int)std::min<size_t>(v.size(), (size_t)max_nb);
    n_nb[a] = k;
    for (int q = 0; q < max_nb; ++q) {
      nb[a * max_nb + q] = q < k ? v[q].first : 0xffffffffu;
      shared[a * max_nb + q] = q < k ? v[q].second : 0u;
    }
    auto& d = depths[a];
    std::sort(d.begin(), d.end(), [&](double x, double y) { return key(x) < key(y); });
    const size_t n = d.size();
    if (n >= 10) {
      range[2 * a] = d[n / 20] * 0.8;
      range[2 * a + 1] = d[n * 19 / 20] * 1.25;
    } else {
      range[2 * a] = agl * 0.3;
      range[2 * a + 1] = agl * 3.0;
    }
  }
  for (int64_t i = 0; i < 3 * np; ++i) pts32[i] = (float)points[i];
}

// The reference's own known-answer problem, `recovers_perturbed_survey`
// (ba.rs:400-481): 3x4 nadir cameras at 80 m, 1500 candidate ground points,
// LCG seeded 99 drawing U(−0.5, 0.5) from the top 53 bits (ba.rs:422-428).
// Capacities: cams 12, points 1500, obs 18000.  Returns the counts through
// n_points/n_obs; the initial (perturbed) state goes to `st`, the true focal
// length to *f_true.
int oracle_make_ref_survey(uint32_t* obs_cam, uint32_t* obs_pt, double* obs_uv,
                           uint8_t* prior_mask, double* prior,
                           oracle_state* st, int32_t* n_points,
                           int32_t* n_obs, double* f_true) {
  const double K[5] = {3000.0, 2000.0, 1500.0, -0.03, 0.0};
  double truthR[12][9], truthC[12][3];
  int nc = 0;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) {
      const double yaw = (r % 2 == 0) ? 90.0 : 270.0;
      from_angles(yaw, -90.0, 0.0, truthR[nc]);
      truthC[nc][0] = c * 25.0;
      truthC[nc][1] = r * 35.0;
      truthC[nc][2] = 80.0;
      ++nc;
    }
  uint64_t s = 99;
  auto rnd = [&s]() {
    s = s * 6364136223846793005ULL + 1442695040888963407ULL;
    return ((double)(s >> 11) / (double)(1ULL << 53)) - 0.5;
  };
  int npt = 0, nobs = 0;
  for (int it = 0; it < 1500; ++it) {
    // Rust evaluates constructor arguments left to right.
    const double x0 = rnd() * 120.0 + 37.0;
    const double x1 = rnd() * 110.0 + 35.0;
    const double x2 = rnd() * 8.0;
    const double X[3] = {x0, x1, x2};
    int vi[12];
    double vu[12][2];
    int nv = 0;
    for (int i = 0; i < nc; ++i) {
      double u[2];
      if (!project(truthR[i], truthC[i], K, X, u)) continue;
      if (u[0] > 0.0 && u[1] > 0.0 && u[0] < 4000.0 && u[1] < 3000.0) {
        vi[nv] = i;
        vu[nv][0] = u[0];
        vu[nv][1] = u[1];
        ++nv;
      }
    }
    if (nv < 2) continue;
    const int pt = npt++;
    const double p0 = rnd(), p1 = rnd(), p2 = rnd();
    st->points[3 * pt] = X[0] + p0 * 2.0;
    st->points[3 * pt + 1] = X[1] + p1 * 2.0;
    st->points[3 * pt + 2] = X[2] + p2 * 2.0;
    for (int v = 0; v < nv; ++v) {
      const double n0 = rnd(), n1 = rnd();
      obs_cam[nobs] = (uint32_t)vi[v];
      obs_pt[nobs] = (uint32_t)pt;
      obs_uv[2 * nobs] = vu[v][0] + n0 * 0.5;
      obs_uv[2 * nobs + 1] = vu[v][1] + n1 * 0.5;
      ++nobs;
    }
  }
  for (int i = 0; i < nc; ++i) {  // ba.rs:454-460
    const double w[3] = {rnd() * 0.02, rnd() * 0.02, rnd() * 0.02};
    double E[9];
    exp_so3(w, E);
    matmul3(E, truthR[i], st->rot + 9 * i);
    const double c0 = rnd(), c1 = rnd(), c2 = rnd();
    st->center[3 * i] = truthC[i][0] + c0 * 3.0;
    st->center[3 * i + 1] = truthC[i][1] + c1 * 3.0;
    st->center[3 * i + 2] = truthC[i][2] + c2 * 3.0;
  }
  for (int i = 0; i < nc; ++i) {  // ba.rs:461-469
    const double c0 = rnd(), c1 = rnd(), c2 = rnd();
    prior_mask[i] = 1;
    prior[6 * i] = truthC[i][0] + c0 * 1.0;
    prior[6 * i + 1] = truthC[i][1] + c1 * 1.0;
    prior[6 * i + 2] = truthC[i][2] + c2 * 1.0;
    prior[6 * i + 3] = 2.0;
    prior[6 * i + 4] = 2.0;
    prior[6 * i + 5] = 3.0;
  }
  st->intr[0] = K[0] * 1.03;  // ba.rs:470-472
  st->intr[1] = K[1];
  st->intr[2] = K[2];
  st->intr[3] = 0.0;
  st->intr[4] = K[4];
  *n_points = npt;
  *n_obs = nobs;
  *f_true = K[0];
  return 0;
}

}  // extern "C"
