// Kernels of one Levenberg–Marquardt iteration (ba.rs:219-383), templated on
// the storage type R of Jacobians, Schur blocks and PCG vectors (double for
// the plain form, float for the mixed form).  Costs, PCG inner products and
// the 3x3 / 6x6 block inversions are always FP64.
#pragma once

#include "solver.cuh"
#include "structure.cuh"

namespace ba {

constexpr int kLinW = 28;  // per-observation record: jc 12, jp 6, jg 6, e 2, w, valid

enum { LOSS_CAUCHY = 0, LOSS_HUBER = 1 };

template <typename R>
struct IterBufs {
  R* lin;      // [no][kLinW]
  // [no][9]: FP64 form: Y_k V^-1 v (6) | w Jg^T Jp V^-1 v (3).  Mixed form:
  // the observation's whole share of the reduced gradient, Jc^T r' (6) |
  // Jg^T r' (3) with r' = w (e - Jp V^-1 v), computed from FP64 values.
  R* gsub;
  R* Z;        // [no][18]: Y_k L (L L^T = V^-1)
  R* Zl;       // [nl][9]: lens entry, top 3x3
  double* ptL;   // [np][6]: l00 l10 l11 l20 l21 l22
  double* ptzv;  // [np][3]: L^T v
  uint8_t* kept;  // [np]: 0 skipped, 1 kept, 2 kept and ill-conditioned (mixed form)
  double* camU;   // [nc][21] upper triangle of sum w Jc^T Jc
  double* camgj;  // [nc][6] sum w Jc^T e
  double* camgs;  // [nc][6] sum Y V^-1 v
  double* camX;   // [nc][18] sum w Jc^T Jg (6x3)
  double* caml;   // [nc][12]: lens U upper (6) | sum w Jg^T e (3) | lens Schur g (3)
  double* grpU;   // [ng][6]
  double* grpg;   // [ng][3]
  double* part;   // [nsub][36] Schur sub-segment sums
  R* S;           // [nz][36] full symmetric BSR
  R* pre;         // [nb][36] block-Jacobi inverses (computed in FP64)
  R* g;           // [nb][6]
  R* x;           // [nb][6] (dx)
  double* cost_part;  // [ncost][3]
  float* ptf;         // [np][9] mixed form: L (6) | t = V^-1 v (3) in FP32 for the Z pass
  // Mixed form with a pair list: observation k's Schur factor is stored at
  // Z[zpos[k]], its position in the camera ordering, so that the factors a
  // destination block (a, b) gathers lie in the segments of cameras a and b
  // in increasing order; null: at Z[k].
  const uint32_t* zpos = nullptr;
  // Values per Schur factor record: 18, or 24 with zpos (96 bytes, three
  // whole 32-byte sectors: the scattered stores of the camera-major layout
  // then write whole sectors, and a gather is three 32-byte-aligned loads).
  int32_t zpitch = 18;
};

// Store an 18-value FP32 Schur factor as a 24-value record (96-byte aligned).
// Values 18..20 carry what the camera pass needs of the observation, read
// in camera order from the same record: its weighted point-step residual
// r' = (r0, r1) (its gradient shares are Jc^T r' and Jg^T r', formed there
// by gshare as the factor pass would), or mode 1: the shares are in gsub
// (points on the FP64 ill-conditioned path).  Values 21..23 are zero.
__device__ __forceinline__ void store_Z24(float* dst, const float (&z)[18], float r0 = 0.0f,
                                          float r1 = 0.0f, float mode = 0.0f) {
  float4* d = reinterpret_cast<float4*>(dst);
  d[0] = make_float4(z[0], z[1], z[2], z[3]);
  d[1] = make_float4(z[4], z[5], z[6], z[7]);
  d[2] = make_float4(z[8], z[9], z[10], z[11]);
  d[3] = make_float4(z[12], z[13], z[14], z[15]);
  d[4] = make_float4(z[16], z[17], r0, r1);
  d[5] = make_float4(mode, 0.0f, 0.0f, 0.0f);
}
// Value offsets of r' and the mode in a 24-value factor record.
constexpr int kZ24R = 18, kZ24Mode = 20;

// An observation's share of the reduced gradient, a Jc^T r' or Jg^T r'
// component: the same expression in the factor pass and the camera pass, so
// that the two give the same FP32 value.
__device__ __forceinline__ float gshare(float a, float b, float r0, float r1) {
  return a * r0 + b * r1;
}

__device__ __forceinline__ size_t z_index(const uint32_t* zpos, int64_t k) {
  return zpos ? (size_t)zpos[k] : (size_t)k;
}

__device__ __forceinline__ double robust_weight(double e2, double sigma, int loss) {
  if (loss == LOSS_HUBER) {
    const double a = sqrt(e2);
    return a <= sigma ? 1.0 : sigma / a;
  }
  return __drcp_rn(1.0 + e2 / (sigma * sigma));  // ba.rs:99 (IEEE 1 / x)
}

__device__ __forceinline__ double robust_rho(double e2, double sigma, int loss) {
  if (loss == LOSS_HUBER) {
    const double a = sqrt(e2);
    return a <= sigma ? e2 : 2.0 * sigma * a - sigma * sigma;
  }
  const double s2 = sigma * sigma;
  return s2 * log(1.0 + e2 / s2);  // ba.rs:114
}

// Bits of 1e300 as a signed 64-bit integer: for the Cauchy factors q >= 1 (or
// NaN) of the cost kernels, q < 1e300 exactly when their bit patterns
// compare so (an integer compare instead of an FP64 one).
constexpr long long kQMaxBits = 0x7e37e43c8800759cLL;

// linearise (ba.rs:56-101) of observation k into out[kLinW]; false if the
// point is not in front of the camera (z <= 1e-6).
template <typename R>
__device__ __forceinline__ bool linearise(const Prob& P, const StateView& st, int64_t k,
                                          double sigma, bool refine, R* out) {
  const uint32_t cam = P.obs_cam[k];
  const double* Rm = st.rot + 9 * (size_t)cam;
  const double* C = st.center + 3 * (size_t)cam;
  const double* K = st.intr + 5 * (size_t)P.cam_group[cam];
  const double* X = st.points + 3 * (size_t)P.obs_pt[k];
  double xc[3];
  bacam::to_cam(Rm, C, X, xc);
  if (xc[2] <= 1e-6) return false;
  const double f = K[0], k1 = K[3], k2 = K[4];
  const double iz = __drcp_rn(xc[2]);  // IEEE 1 / z, as a reciprocal
  const double px = xc[0] * iz, py = xc[1] * iz;
  const double r2 = px * px + py * py;
  const double d = 1.0 + k1 * r2 + k2 * r2 * r2;
  const double qx = px * d, qy = py * d;
  const double ex = P.obs_uv[2 * k] - (f * qx + K[1]);
  const double ey = P.obs_uv[2 * k + 1] - (f * qy + K[2]);
  // Jacobians in the storage precision R (FP32 in the mixed form; the
  // residual above stays FP64).
  const R fR = (R)f, iz_ = (R)iz, px_ = (R)px, py_ = (R)py, r2_ = (R)r2, d_ = (R)d;
  const R x0 = (R)xc[0], x1 = (R)xc[1], x2 = (R)xc[2];
  const R c = (R)2 * ((R)k1 + (R)2 * (R)k2 * r2_);
  const R a00 = (d_ + c * px_ * px_) * fR, a01 = (c * px_ * py_) * fR;
  const R a11 = (d_ + c * py_ * py_) * fR;
  const R b02 = -x0 * iz_ * iz_, b12 = -x1 * iz_ * iz_;
  R du[6];
  du[0] = a00 * iz_;
  du[1] = a01 * iz_;
  du[2] = a00 * b02 + a01 * b12;
  du[3] = a01 * iz_;
  du[4] = a11 * iz_;
  du[5] = a01 * b02 + a11 * b12;
  // Jc = [dudx · (−[xc]x) | dudx · (−R)], Jp = dudx · R.
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const R u0 = du[3 * r], u1 = du[3 * r + 1], u2 = du[3 * r + 2];
    out[6 * r + 0] = u2 * x1 - u1 * x2;
    out[6 * r + 1] = u0 * x2 - u2 * x0;
    out[6 * r + 2] = u1 * x0 - u0 * x1;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const R pp = u0 * (R)Rm[j] + u1 * (R)Rm[3 + j] + u2 * (R)Rm[6 + j];
      out[6 * r + 3 + j] = -pp;
      out[12 + 3 * r + j] = pp;
    }
  }
  if (refine) {  // ba.rs:87-95
    out[18] = (R)qx;
    out[19] = fR * px_ * r2_;
    out[20] = fR * px_ * r2_ * r2_;
    out[21] = (R)qy;
    out[22] = fR * py_ * r2_;
    out[23] = fR * py_ * r2_ * r2_;
  } else {
#pragma unroll
    for (int i = 18; i < 24; ++i) out[i] = (R)0;
  }
  out[24] = (R)ex;
  out[25] = (R)ey;
  out[26] = (R)robust_weight(ex * ex + ey * ey, sigma, P.loss);
  out[27] = (R)1;
  return true;
}

// Lower Cholesky factor of a symmetric positive definite 3x3 (row-major);
// a non-positive pivot (rounding on a near-singular block) is clamped to 0.
__device__ __forceinline__ void chol3(const double* A, double* L) {
  const double a00 = A[0], a10 = A[3], a11 = A[4], a20 = A[6], a21 = A[7], a22 = A[8];
  const double l00 = a00 > 0.0 ? sqrt(a00) : 0.0;
  const double l10 = l00 > 0.0 ? a10 / l00 : 0.0;
  const double l20 = l00 > 0.0 ? a20 / l00 : 0.0;
  const double t11 = a11 - l10 * l10;
  const double l11 = t11 > 0.0 ? sqrt(t11) : 0.0;
  const double l21 = l11 > 0.0 ? (a21 - l20 * l10) / l11 : 0.0;
  const double t22 = a22 - l20 * l20 - l21 * l21;
  const double l22 = t22 > 0.0 ? sqrt(t22) : 0.0;
  L[0] = l00, L[1] = l10, L[2] = l11, L[3] = l20, L[4] = l21, L[5] = l22;
}

// ---- per point: linearise its observations, V, v, V^-1, Z (ba.rs:222-268) ----

template <typename R>
__device__ __forceinline__ void point_system(const Prob& P, const StateView& st,
                                             const StructView& S, const IterBufs<R>& B,
                                             int64_t p, bool refine, double sg, double lam) {
  const uint32_t s = S.pt_ptr[p], e = S.pt_ptr[p + 1];
  if (e - s < 2) {  // ba.rs:238
    B.kept[p] = 0;
    for (uint32_t k = s; k < e; ++k) {
      R* o = B.lin + (size_t)k * kLinW;
      if (!linearise<R>(P, st, k, sg, refine, o))
        for (int i = 0; i < kLinW; ++i) o[i] = (R)0;
      for (int i = 0; i < 18; ++i) B.Z[(size_t)k * 18 + i] = (R)0;
      for (int i = 0; i < 9; ++i) B.gsub[(size_t)k * 9 + i] = (R)0;
    }
    for (uint32_t j = S.lens_ptr[p]; j < S.lens_ptr[p + 1]; ++j)
      for (int i = 0; i < 9; ++i) B.Zl[(size_t)j * 9 + i] = (R)0;
    return;
  }
  // V, v and the Y / Z products accumulate in the storage precision R; the 3x3
  // inversion and its Cholesky factor are FP64.
  R V[6] = {0, 0, 0, 0, 0, 0}, v[3] = {0, 0, 0};
  for (uint32_t k = s; k < e; ++k) {
    R* o = B.lin + (size_t)k * kLinW;
    if (!linearise<R>(P, st, k, sg, refine, o)) {
      for (int i = 0; i < kLinW; ++i) o[i] = (R)0;
      continue;
    }
    const R w = o[26];
    const R j0 = o[12], j1 = o[13], j2 = o[14], j3 = o[15], j4 = o[16], j5 = o[17];
    const R e0 = o[24], e1 = o[25];
    V[0] += (j0 * j0 + j3 * j3) * w;
    V[1] += (j0 * j1 + j3 * j4) * w;
    V[2] += (j0 * j2 + j3 * j5) * w;
    V[3] += (j1 * j1 + j4 * j4) * w;
    V[4] += (j1 * j2 + j4 * j5) * w;
    V[5] += (j2 * j2 + j5 * j5) * w;
    v[0] += (j0 * e0 + j3 * e1) * w;
    v[1] += (j1 * e0 + j4 * e1) * w;
    v[2] += (j2 * e0 + j5 * e1) * w;
  }
  double A[9], Ai[9], Vd[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) Vd[i] = (double)V[i];
  sym3_full(Vd, A);
  A[0] = A[0] * (1.0 + lam) + 1e-9;  // ba.rs:262-264
  A[4] = A[4] * (1.0 + lam) + 1e-9;
  A[8] = A[8] * (1.0 + lam) + 1e-9;
  const bool ok = inv3(A, Ai);  // ba.rs:265
  B.kept[p] = ok ? 1 : 0;
  double L[6] = {0, 0, 0, 0, 0, 0};
  if (ok) chol3(Ai, L);
  const double zv0d = L[0] * (double)v[0] + L[1] * (double)v[1] + L[3] * (double)v[2];
  const double zv1d = L[2] * (double)v[1] + L[4] * (double)v[2];
  const double zv2d = L[5] * (double)v[2];
  // t = V^-1 v = L zv
  const R l00 = (R)L[0], l10 = (R)L[1], l11 = (R)L[2], l20 = (R)L[3], l21 = (R)L[4], l22 = (R)L[5];
  const R t0 = (R)(L[0] * zv0d), t1 = (R)(L[1] * zv0d + L[2] * zv1d),
          t2 = (R)(L[3] * zv0d + L[4] * zv1d + L[5] * zv2d);
  double* pl = B.ptL + 6 * (size_t)p;
#pragma unroll
  for (int i = 0; i < 6; ++i) pl[i] = L[i];
  B.ptzv[3 * p] = zv0d, B.ptzv[3 * p + 1] = zv1d, B.ptzv[3 * p + 2] = zv2d;
  for (uint32_t k = s; k < e; ++k) {
    const R* o = B.lin + (size_t)k * kLinW;
    R* Z = B.Z + (size_t)k * 18;
    R* gs = B.gsub + (size_t)k * 9;
    if (!ok || o[27] == (R)0) {
#pragma unroll
      for (int i = 0; i < 18; ++i) Z[i] = (R)0;
#pragma unroll
      for (int i = 0; i < 9; ++i) gs[i] = (R)0;
      continue;
    }
    const R w = o[26];
    const R j0 = o[12], j1 = o[13], j2 = o[14], j3 = o[15], j4 = o[16], j5 = o[17];
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      const R ca = o[r], cb = o[6 + r];
      // Y = (Jc^T Jp) w   (ba.rs:249)
      const R y0 = (ca * j0 + cb * j3) * w;
      const R y1 = (ca * j1 + cb * j4) * w;
      const R y2 = (ca * j2 + cb * j5) * w;
      Z[3 * r + 0] = y0 * l00 + y1 * l10 + y2 * l20;
      Z[3 * r + 1] = y1 * l11 + y2 * l21;
      Z[3 * r + 2] = y2 * l22;
      gs[r] = y0 * t0 + y1 * t1 + y2 * t2;
    }
    // w Jg^T (Jp t)
    const R pt0 = j0 * t0 + j1 * t1 + j2 * t2, pt1 = j3 * t0 + j4 * t1 + j5 * t2;
#pragma unroll
    for (int a = 0; a < 3; ++a) gs[6 + a] = (o[18 + a] * pt0 + o[21 + a] * pt1) * w;
  }
  // Lens entries: Y_g = sum over the point's observations in group g (ba.rs:251-259).
  const uint32_t l0 = S.lens_ptr[p], l1 = S.lens_ptr[p + 1];
  for (uint32_t j = l0; j < l1; ++j) {
    R Y[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t k = s; k < e; ++k) {
      if (S.obs_lens[k] != j) continue;
      const R* o = B.lin + (size_t)k * kLinW;
      if (o[27] == (R)0) continue;
      const R w = o[26];
      const R j0 = o[12], j1 = o[13], j2 = o[14], j3 = o[15], j4 = o[16], j5 = o[17];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const R ga = o[18 + a], gb = o[21 + a];
        Y[3 * a + 0] += (ga * j0 + gb * j3) * w;
        Y[3 * a + 1] += (ga * j1 + gb * j4) * w;
        Y[3 * a + 2] += (ga * j2 + gb * j5) * w;
      }
    }
    R* Zl = B.Zl + (size_t)j * 9;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const R y0 = Y[3 * a], y1 = Y[3 * a + 1], y2 = Y[3 * a + 2];
      Zl[3 * a + 0] = ok ? y0 * l00 + y1 * l10 + y2 * l20 : (R)0;
      Zl[3 * a + 1] = ok ? y1 * l11 + y2 * l21 : (R)0;
      Zl[3 * a + 2] = ok ? y2 * l22 : (R)0;
    }
  }
}

// Exact float -> double in integer instructions (the FP64 pipe, which also
// executes the hardware conversion, is the bound of the FP64 sums here).
// Zero, subnormal, infinite and NaN inputs take the hardware conversion.
__device__ __forceinline__ double f2d_exact(float x) {
  const uint32_t u = __float_as_uint(x);
  const uint32_t ex = (u >> 23) & 0xffu;
  if (ex == 0u || ex == 0xffu) return (double)x;
  const uint32_t hi = (u & 0x80000000u) | (((u & 0x7fffffffu) >> 3) + (896u << 20));
  return __hiloint2double((int)hi, (int)(u << 29));
}

// Mixed form, FP32 copy of each camera's rotation (row-major), focal length
// and radial terms k1, k2: the per-observation pass reads them instead of
// converting FP64 state per observation.
constexpr int kCamF = 12;

static __global__ void cam_f32_kernel(Prob P, StateView st, float* camf, const int32_t* active) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= P.nc || (active && !active[P.cam_model[c]])) return;
  const double* R = st.rot + 9 * (size_t)c;
  const double* K = st.intr + 5 * (size_t)P.cam_group[c];
  float* o = camf + kCamF * (size_t)c;
#pragma unroll
  for (int i = 0; i < 9; ++i) o[i] = (float)R[i];
  o[9] = (float)K[0], o[10] = (float)K[3], o[11] = (float)K[4];
}

// 1/x for x > 0 to about 1e-14 relative: an FP32 reciprocal refined by one
// FP64 Newton step (two FP64 instructions and two conversions instead of an
// IEEE division).  The mixed form's residual needs this accuracy only far
// below the FP32 rounding of the stored residual.
__device__ __forceinline__ double rcp_newton(double x) {
  const double r = (double)(1.0f / (float)x);
  return fma(r, fma(-x, r, 1.0), r);
}

// Mixed form, record of an observation with extreme Jacobians, all in FP64:
// an observation of a point barely in front of its camera has |J| up to
// ~1e19 (w ~ 1e-24), and FP32 J^T J would overflow.  Such a record is stored
// whitened, sqrt(w) J and sqrt(w) e with weight 1: every use of the record is
// bilinear in (J, e) times w, so the sums are unchanged.  On return `ev` is
// the (whitened) FP64 residual that goes with the stored record.
static __device__ __noinline__ void linearise_mixed_extreme(const Prob& P, const StateView& st,
                                                            int64_t k, double sigma, bool refine,
                                                            const double (&xc)[3], float* out,
                                                            double (&ev)[2]) {
  const uint32_t cam = P.obs_cam[k];
  const double* Rm = st.rot + 9 * (size_t)cam;
  const double* K = st.intr + 5 * (size_t)P.cam_group[cam];
  const double f = K[0], k1 = K[3], k2 = K[4];
  const double iz = __drcp_rn(xc[2]);  // IEEE 1 / z, as a reciprocal
  const double px = xc[0] * iz, py = xc[1] * iz;
  const double r2 = px * px + py * py;
  const double d = 1.0 + k1 * r2 + k2 * r2 * r2;
  const double qx = px * d, qy = py * d;
  ev[0] = P.obs_uv[2 * k] - (f * qx + K[1]);
  ev[1] = P.obs_uv[2 * k + 1] - (f * qy + K[2]);
  const double c = 2.0 * (k1 + 2.0 * k2 * r2);
  const double a00 = (d + c * px * px) * f, a01 = (c * px * py) * f;
  const double a11 = (d + c * py * py) * f;
  const double b02 = -xc[0] * iz * iz, b12 = -xc[1] * iz * iz;
  double du[6];
  du[0] = a00 * iz;
  du[1] = a01 * iz;
  du[2] = a00 * b02 + a01 * b12;
  du[3] = a01 * iz;
  du[4] = a11 * iz;
  du[5] = a01 * b02 + a11 * b12;
  const double w = robust_weight(ev[0] * ev[0] + ev[1] * ev[1], sigma, P.loss);
  const double sw = sqrt(w);
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const double u0 = du[3 * r], u1 = du[3 * r + 1], u2 = du[3 * r + 2];
    const float f0 = (float)(u0 * sw), f1 = (float)(u1 * sw), f2 = (float)(u2 * sw);
    const float x0 = (float)xc[0], x1 = (float)xc[1], x2 = (float)xc[2];
    out[6 * r + 0] = f2 * x1 - f1 * x2;
    out[6 * r + 1] = f0 * x2 - f2 * x0;
    out[6 * r + 2] = f1 * x0 - f0 * x1;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double jp = u0 * Rm[j] + u1 * Rm[3 + j] + u2 * Rm[6 + j];
      out[6 * r + 3 + j] = -(float)(jp * sw);
      out[12 + 3 * r + j] = (float)(jp * sw);
    }
  }
  if (refine) {  // ba.rs:87-95
    out[18] = (float)(qx * sw);
    out[19] = (float)(f * px * r2 * sw);
    out[20] = (float)(f * px * r2 * r2 * sw);
    out[21] = (float)(qy * sw);
    out[22] = (float)(f * py * r2 * sw);
    out[23] = (float)(f * py * r2 * r2 * sw);
  } else {
#pragma unroll
    for (int i = 18; i < 24; ++i) out[i] = 0.0f;
  }
  ev[0] *= sw;
  ev[1] *= sw;
  out[24] = (float)ev[0];
  out[25] = (float)ev[1];
  out[26] = 1.0f;
  out[27] = 1.0f;
}

// Mixed form, first pass over an observation.  The residual is FP64 (it
// decides the gradient near convergence); dudx, Jc, Jp, Jg and the robust
// weight are FP32 and stored as the record.  The point system V, v is summed
// in FP64 from exactly these stored values (`jp`, `w`; products of FP32
// numbers are exact in FP64), so V^-1 v is the exact least-squares point
// step of the stored Jacobians: a point whose rays are nearly parallel has a
// nearly singular V, and any rounding between V, v and the records would be
// amplified by V^-1.  On return `ev` is the FP64 residual matching the
// record (whitened for an extreme record).
// The FP32 part of a mixed record, from the point in camera coordinates xc
// (FP64, in front of the camera) and the FP64 residual ev of observation k.
__device__ __forceinline__ void mixed_record_from(const Prob& P, const StateView& st,
                                                  const float* camf, int64_t k, double sigma,
                                                  float sigma_f, float inv_s2, bool refine,
                                                  const double (&xc)[3], double (&ev)[2],
                                                  float* out, float (&jp)[6], float& w) {
  const uint32_t cam = P.obs_cam[k];
  const float* cf = camf + kCamF * (size_t)cam;
  const float x0 = (float)xc[0], x1 = (float)xc[1], x2 = (float)xc[2];
  const float f = cf[9], k1 = cf[10], k2 = cf[11];
  const float iz = 1.0f / x2;
  const float px = x0 * iz, py = x1 * iz;
  const float r2 = px * px + py * py;
  const float d = 1.0f + k1 * r2 + k2 * r2 * r2;
  const float c = 2.0f * (k1 + 2.0f * k2 * r2);
  const float a00 = (d + c * px * px) * f, a01 = (c * px * py) * f;
  const float a11 = (d + c * py * py) * f;
  const float b02 = -x0 * iz * iz, b12 = -x1 * iz * iz;
  float du[6];
  du[0] = a00 * iz;
  du[1] = a01 * iz;
  du[2] = a00 * b02 + a01 * b12;
  du[3] = a01 * iz;
  du[4] = a11 * iz;
  du[5] = a01 * b02 + a11 * b12;
  const float e0 = (float)ev[0], e1 = (float)ev[1];
  const float e2 = e0 * e0 + e1 * e1;
  float jmax = 0.0f;
#pragma unroll
  for (int i = 0; i < 6; ++i) jmax = fmaxf(jmax, fabsf(du[i]));
  jmax *= fmaxf(1.0f, fmaxf(fabsf(x0), fmaxf(fabsf(x1), fabsf(x2))));
  // NaN or inf in the FP32 chain fails the test as well.
  if (!(jmax < 1e12f) || !(e2 < 1e30f)) {
    linearise_mixed_extreme(P, st, k, sigma, refine, xc, out, ev);
#pragma unroll
    for (int i = 0; i < 6; ++i) jp[i] = out[12 + i];
    w = 1.0f;
    return;
  }
  if (P.loss == LOSS_HUBER) {
    const float a = sqrtf(e2);
    w = a <= sigma_f ? 1.0f : sigma_f / a;
  } else {
    w = 1.0f / (1.0f + e2 * inv_s2);  // ba.rs:99
  }
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const float u0 = du[3 * r], u1 = du[3 * r + 1], u2 = du[3 * r + 2];
    out[6 * r + 0] = u2 * x1 - u1 * x2;
    out[6 * r + 1] = u0 * x2 - u2 * x0;
    out[6 * r + 2] = u1 * x0 - u0 * x1;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float pp = u0 * cf[j] + u1 * cf[3 + j] + u2 * cf[6 + j];
      jp[3 * r + j] = pp;
      out[6 * r + 3 + j] = -pp;
      out[12 + 3 * r + j] = pp;
    }
  }
  if (refine) {  // ba.rs:87-95
    out[18] = px * d;
    out[19] = f * px * r2;
    out[20] = f * px * r2 * r2;
    out[21] = py * d;
    out[22] = f * py * r2;
    out[23] = f * py * r2 * r2;
  } else {
#pragma unroll
    for (int i = 18; i < 24; ++i) out[i] = 0.0f;
  }
  out[24] = e0;
  out[25] = e1;
  out[26] = w;
  out[27] = 1.0f;
}

__device__ __forceinline__ bool linearise_mixed(const Prob& P, const StateView& st,
                                                const float* camf, int64_t k, double sigma,
                                                float sigma_f, float inv_s2, bool refine,
                                                float* out, float (&jp)[6], double (&ev)[2],
                                                float& w) {
  const uint32_t cam = P.obs_cam[k];
  const double* Rm = st.rot + 9 * (size_t)cam;
  const double* C = st.center + 3 * (size_t)cam;
  const double* K = st.intr + 5 * (size_t)P.cam_group[cam];
  const double* X = st.points + 3 * (size_t)P.obs_pt[k];
  double xc[3];
  bacam::to_cam(Rm, C, X, xc);
  if (xc[2] <= 1e-6) return false;
  {
    const double iz = rcp_newton(xc[2]);
    const double px = xc[0] * iz, py = xc[1] * iz;
    const double r2 = px * px + py * py;
    const double d = 1.0 + K[3] * r2 + K[4] * r2 * r2;
    ev[0] = P.obs_uv[2 * k] - (K[0] * (px * d) + K[1]);
    ev[1] = P.obs_uv[2 * k + 1] - (K[0] * (py * d) + K[2]);
  }
  mixed_record_from(P, st, camf, k, sigma, sigma_f, inv_s2, refine, xc, ev, out, jp, w);
  return true;
}

// Above this bound on cond(V) a point's second pass runs in FP64 (its V^-1
// would amplify FP32 rounding of Jc, Jp beyond the accuracy the reduced
// system needs).  cond(V) <= tr^3 / (4 det) for a 3x3 SPD matrix.
constexpr double kMixedCondLimit = 1e4;

// Mixed form, a point with cond(V) above kMixedCondLimit: V, v, V^-1 and the
// second pass all from an FP64 re-linearisation, so that V^-1 v stays the
// exact point step of the Jacobians the Schur factors are formed from (FP32
// rounding of the records would be amplified by V^-1).  Z and the gradient
// shares are rounded to FP32 once.  About 0.4 % of the points of a converging
// survey take this path.  kZ false: the Schur factors are not stored (the
// matrix-free PCG recomputes them where it uses them).
template <bool kZ>
static __device__ __noinline__ void point_system_mixed_ill(const Prob& P, const StateView& st,
                                                           const StructView& S,
                                                           const IterBufs<float>& B, int64_t p,
                                                           bool refine, double sg, double lam) {
  const uint32_t s = S.pt_ptr[p], e = S.pt_ptr[p + 1];
  double V[6] = {0, 0, 0, 0, 0, 0}, v[3] = {0, 0, 0};
  for (uint32_t k = s; k < e; ++k) {
    double o[kLinW];
    if (!linearise<double>(P, st, k, sg, refine, o)) continue;
    const double w = o[26];
    const double j0 = o[12], j1 = o[13], j2 = o[14], j3 = o[15], j4 = o[16], j5 = o[17];
    V[0] += (j0 * j0 + j3 * j3) * w;
    V[1] += (j0 * j1 + j3 * j4) * w;
    V[2] += (j0 * j2 + j3 * j5) * w;
    V[3] += (j1 * j1 + j4 * j4) * w;
    V[4] += (j1 * j2 + j4 * j5) * w;
    V[5] += (j2 * j2 + j5 * j5) * w;
    v[0] += (j0 * o[24] + j3 * o[25]) * w;
    v[1] += (j1 * o[24] + j4 * o[25]) * w;
    v[2] += (j2 * o[24] + j5 * o[25]) * w;
  }
  double A[9], Ai[9];
  sym3_full(V, A);
  A[0] = A[0] * (1.0 + lam) + 1e-9;  // ba.rs:262-264
  A[4] = A[4] * (1.0 + lam) + 1e-9;
  A[8] = A[8] * (1.0 + lam) + 1e-9;
  const bool ok = inv3(A, Ai);  // ba.rs:265
  double L[6] = {0, 0, 0, 0, 0, 0};
  if (ok) chol3(Ai, L);
  B.kept[p] = ok ? 2 : 0;
  if (!ok) {
    for (uint32_t k = s; k < e; ++k) {
      if constexpr (kZ)
        for (int i = 0; i < 18; ++i) B.Z[z_index(B.zpos, k) * B.zpitch + i] = 0.0f;
      for (int i = 0; i < 9; ++i) B.gsub[(size_t)k * 9 + i] = 0.0f;
    }
    for (uint32_t j = S.lens_ptr[p]; j < S.lens_ptr[p + 1]; ++j)
      for (int i = 0; i < 9; ++i) B.Zl[(size_t)j * 9 + i] = 0.0f;
    return;
  }
  const double zv0 = L[0] * v[0] + L[1] * v[1] + L[3] * v[2];
  const double zv1 = L[2] * v[1] + L[4] * v[2];
  const double zv2 = L[5] * v[2];
  const double t0 = L[0] * zv0, t1 = L[1] * zv0 + L[2] * zv1, t2 = L[3] * zv0 + L[4] * zv1 + L[5] * zv2;
  double* pl = B.ptL + 6 * (size_t)p;
#pragma unroll
  for (int i = 0; i < 6; ++i) pl[i] = L[i];
  B.ptzv[3 * p] = zv0, B.ptzv[3 * p + 1] = zv1, B.ptzv[3 * p + 2] = zv2;
  const uint32_t l0 = S.lens_ptr[p], l1 = S.lens_ptr[p + 1];
  for (uint32_t k = s; k < e; ++k) {
    float* Z = kZ ? B.Z + z_index(B.zpos, k) * B.zpitch : nullptr;
    float* gs = B.gsub + (size_t)k * 9;
    if constexpr (kZ) {
      if (B.zpitch == 24) {  // the camera pass takes this observation's shares from gsub
#pragma unroll
        for (int i = kZ24R; i < 24; ++i) Z[i] = i == kZ24Mode ? 1.0f : 0.0f;
      }
    }
    double o[kLinW];
    if (!linearise<double>(P, st, k, sg, refine, o)) {
      if constexpr (kZ)
#pragma unroll
        for (int i = 0; i < 18; ++i) Z[i] = 0.0f;
#pragma unroll
      for (int i = 0; i < 9; ++i) gs[i] = 0.0f;
      continue;
    }
    const double w = o[26];
    const double j0 = o[12], j1 = o[13], j2 = o[14], j3 = o[15], j4 = o[16], j5 = o[17];
    const double r0 = (o[24] - (j0 * t0 + j1 * t1 + j2 * t2)) * w;
    const double r1 = (o[25] - (j3 * t0 + j4 * t1 + j5 * t2)) * w;
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      const double ca = o[r], cb = o[6 + r];
      const double y0 = (ca * j0 + cb * j3) * w;
      const double y1 = (ca * j1 + cb * j4) * w;
      const double y2 = (ca * j2 + cb * j5) * w;
      if constexpr (kZ) {
        Z[3 * r + 0] = (float)(y0 * L[0] + y1 * L[1] + y2 * L[3]);
        Z[3 * r + 1] = (float)(y1 * L[2] + y2 * L[4]);
        Z[3 * r + 2] = (float)(y2 * L[5]);
      }
      gs[r] = (float)(ca * r0 + cb * r1);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) gs[6 + a] = (float)(o[18 + a] * r0 + o[21 + a] * r1);
  }
  for (uint32_t j = l0; j < l1; ++j) {
    double Y[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t k = s; k < e; ++k) {
      if (S.obs_lens[k] != j) continue;
      double o[kLinW];
      if (!linearise<double>(P, st, k, sg, refine, o)) continue;
      const double w = o[26];
      const double j0 = o[12], j1 = o[13], j2 = o[14], j3 = o[15], j4 = o[16], j5 = o[17];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const double ga = o[18 + a], gb = o[21 + a];
        Y[3 * a + 0] += (ga * j0 + gb * j3) * w;
        Y[3 * a + 1] += (ga * j1 + gb * j4) * w;
        Y[3 * a + 2] += (ga * j2 + gb * j5) * w;
      }
    }
    float* Zl = B.Zl + (size_t)j * 9;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double y0 = Y[3 * a], y1 = Y[3 * a + 1], y2 = Y[3 * a + 2];
      Zl[3 * a + 0] = (float)(y0 * L[0] + y1 * L[1] + y2 * L[3]);
      Zl[3 * a + 1] = (float)(y1 * L[2] + y2 * L[4]);
      Zl[3 * a + 2] = (float)(y2 * L[5]);
    }
  }
}

// FP64 form: a thread per point (in order of observation count).
template <typename R>
__global__ void __launch_bounds__(128)
    point_kernel(Prob P, StateView st, StructView S, IterBufs<R> B, const int32_t* active,
                 const double* lambda, const double* sigma) {
  static_assert(sizeof(R) == 8, "the mixed form runs obs_record / point_solve_mixed / obs_factor");
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= P.np) return;
  const int64_t p = S.pt_order ? S.pt_order[tid] : tid;
  const uint32_t m = P.pt_model[p];
  if (!active[m]) return;
  const bool refine = P.model_refine[m] != 0;
  point_system<R>(P, st, S, B, p, refine, sigma[m], lambda[m]);
}

// ---- mixed form in three passes: records, point systems, Schur factors -------
//
// The point system of the mixed form is split by what each step is indexed by.
// Observations are sorted by point, so passes over observations read the
// problem and write the per-observation arrays coalesced (a warp stages its 32
// records in shared memory and stores them as contiguous runs); only the FP64
// point-system sums run a thread per point.

constexpr int kObsThreads = 256;
constexpr int kObsWarps = kObsThreads / 32;
// Odd pitches: lanes writing the same field of their records hit distinct banks.
constexpr int kLinPitch = kLinW + 1;
constexpr int kZPitch = 19;
constexpr int kGPitch = 9;

// Store a warp's n (<= 32) consecutive records of W floats, staged in shared
// memory at `pitch`, to dst[0 .. n*W): contiguous 128-byte runs per
// instruction.  Records whose bit in `mask` is clear are left as they are.
template <int W>
__device__ __forceinline__ void warp_store_records(const float* sm, int pitch, float* dst, int n,
                                                   uint32_t mask, int lane) {
  for (int i = lane; i < n * W; i += 32) {
    const int r = i / W;
    if ((mask >> r) & 1u) dst[i] = sm[r * pitch + (i - r * W)];
  }
}

// Pass 1, a thread per observation: the FP32 record (linearise_mixed: FP64
// residual, FP32 Jacobians and weight).
// stale: null, or per model whether its records must be formed here (else
// the trial cost of its accepted step left them, at this state).
static __global__ void __launch_bounds__(kObsThreads, 4)
    obs_record_kernel(Prob P, StateView st, IterBufs<float> B, const float* camf,
                      const int32_t* active, const double* sigma, const int32_t* stale) {
  __shared__ float sm[kObsWarps][32 * kLinPitch];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t k0 = (int64_t)blockIdx.x * kObsThreads + warp * 32;
  if (k0 >= P.no) return;
  const int64_t k = k0 + lane;
  float* rec = &sm[warp][lane * kLinPitch];
  bool mine = false;
  if (k < P.no) {
    const uint32_t m = P.pt_model[P.obs_pt[k]];
    if (active[m] && (!stale || stale[m])) {
      mine = true;
      const double sg = sigma[m];
      const float sg_f = (float)sg, inv_s2 = 1.0f / (sg_f * sg_f);
      float jpf[6], wf;
      double ev[2];
      if (!linearise_mixed(P, st, camf, k, sg, sg_f, inv_s2, P.model_refine[m] != 0, rec, jpf,
                           ev, wf)) {
#pragma unroll
        for (int i = 0; i < kLinW; ++i) rec[i] = 0.0f;
      }
    }
  }
  const uint32_t mask = __ballot_sync(0xffffffffu, mine);
  __syncwarp();
  const int n = P.no - k0 < 32 ? (int)(P.no - k0) : 32;
  warp_store_records<kLinW>(sm[warp], kLinPitch, B.lin + k0 * kLinW, n, mask, lane);
}

// Double-float accumulation: hi + lo += w a b for FP32 w, a, b, where
// (p, q) = w a exactly (p = w a rounded, q = fma(w, a, -p)).  The products are
// split exactly with FMAs and added by Knuth's two-sum, so hi + lo carries
// about 48 bits — close to FP64 — from FP32 instructions, which on this GPU
// run 64 times faster than FP64 ones.
__device__ __forceinline__ void df_add_prod(float& hi, float& lo, float p, float q, float b) {
  const float a = p * b;
  const float c = fmaf(p, b, -a) + q * b;  // the rest of (p + q) b
  const float s = hi + a;
  const float bb = s - hi;
  lo += ((hi - (s - bb)) + (a - bb)) + c;
  hi = s;
}

// Double-float accumulation hi + lo += x (Knuth's two-sum).
__device__ __forceinline__ void df_add(float& hi, float& lo, float x) {
  const float s = hi + x;
  const float bb = s - hi;
  lo += (hi - (s - bb)) + (x - bb);
  hi = s;
}

// Lower Cholesky factor of a symmetric positive definite 3x3 (row-major) by
// reciprocal square roots (mixed form); a non-positive pivot gives zeros.
__device__ __forceinline__ void chol3_rsqrt(const double* A, double* L) {
  const double a00 = A[0], a10 = A[3], a11 = A[4], a20 = A[6], a21 = A[7], a22 = A[8];
  const double r0 = a00 > 0.0 ? rsqrt(a00) : 0.0;
  const double l00 = a00 * r0, l10 = a10 * r0, l20 = a20 * r0;
  const double t11 = a11 - l10 * l10;
  const double r1 = t11 > 0.0 ? rsqrt(t11) : 0.0;
  const double l11 = t11 * r1, l21 = (a21 - l20 * l10) * r1;
  const double t22 = a22 - l20 * l20 - l21 * l21;
  const double l22 = t22 > 0.0 ? t22 * rsqrt(t22) : 0.0;
  L[0] = l00, L[1] = l10, L[2] = l11, L[3] = l20, L[4] = l21, L[5] = l22;
}

// The end of a point's mixed-form system once its sums are done (both point
// kernels): FP64 V and v from the double-float sums, damping, the
// conditioning test (an ill-conditioned point takes the FP64 path), V^-1 and
// its Cholesky factor, the point's outputs and its lens entries (ba.rs:238-268).
// rec(k): observation k's record (shared or global memory); pf_local: null, or
// where the point's FP32 factor and step (9 floats) go besides B.ptf.
template <typename Rec>
__device__ __forceinline__ void point_mixed_finish(
    const Prob& P, const StateView& st, const StructView& S, const IterBufs<float>& B, int64_t p,
    uint32_t m, uint32_t s, uint32_t e, uint32_t l0, uint32_t l1, bool sum, const float (&Vh)[6],
    const float (&Vl)[6], const float (&vh)[3], const float (&vl)[3], float (&Y)[9],
    const double* lambda, const double* sigma, Rec&& rec, float* pf_local) {
  const bool refine = P.model_refine[m] != 0;
  if (!sum) {  // fewer than two observations (ba.rs:238)
    B.kept[p] = 0;
    for (uint32_t j = l0; j < l1; ++j)
      for (int i = 0; i < 9; ++i) B.Zl[(size_t)j * 9 + i] = 0.0f;
    return;
  }
  double V[6], v[3];
#pragma unroll
  for (int t = 0; t < 6; ++t) V[t] = f2d_exact(Vh[t]) + f2d_exact(Vl[t]);
#pragma unroll
  for (int i = 0; i < 3; ++i) v[i] = f2d_exact(vh[i]) + f2d_exact(vl[i]);
  const double lam = lambda[m];
  double A[9];
  sym3_full(V, A);
  A[0] = A[0] * (1.0 + lam) + 1e-9;  // ba.rs:262-264
  A[4] = A[4] * (1.0 + lam) + 1e-9;
  A[8] = A[8] * (1.0 + lam) + 1e-9;
  // Cofactors of the first row: the determinant serves the conditioning
  // test and the inverse (ba.rs:265; exactly-singular V is skipped).
  const double c00 = A[4] * A[8] - A[5] * A[7];
  const double c01 = A[5] * A[6] - A[3] * A[8];
  const double c02 = A[3] * A[7] - A[4] * A[6];
  const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
  const double tr = A[0] + A[4] + A[8];
  if (!(det > 0.0) || tr * tr * tr > 4.0 * kMixedCondLimit * det) {
    if (B.Z)
      point_system_mixed_ill<true>(P, st, S, B, p, refine, sigma[m], lam);
    else
      point_system_mixed_ill<false>(P, st, S, B, p, refine, sigma[m], lam);
    return;
  }
  double Ai[9];
  {
    const double id = __drcp_rn(det);  // IEEE 1 / det
    Ai[0] = c00 * id;
    Ai[1] = (A[2] * A[7] - A[1] * A[8]) * id;
    Ai[2] = (A[1] * A[5] - A[2] * A[4]) * id;
    Ai[3] = c01 * id;
    Ai[4] = (A[0] * A[8] - A[2] * A[6]) * id;
    Ai[5] = (A[2] * A[3] - A[0] * A[5]) * id;
    Ai[6] = c02 * id;
    Ai[7] = (A[1] * A[6] - A[0] * A[7]) * id;
    Ai[8] = (A[0] * A[4] - A[1] * A[3]) * id;
  }
  double L[6];
  chol3_rsqrt(Ai, L);
  B.kept[p] = 1;
  const double zv0 = L[0] * v[0] + L[1] * v[1] + L[3] * v[2];
  const double zv1 = L[2] * v[1] + L[4] * v[2];
  const double zv2 = L[5] * v[2];
  double* pl = B.ptL + 6 * (size_t)p;
#pragma unroll
  for (int i = 0; i < 6; ++i) pl[i] = L[i];
  B.ptzv[3 * p] = zv0, B.ptzv[3 * p + 1] = zv1, B.ptzv[3 * p + 2] = zv2;
  float pfv[9];
#pragma unroll
  for (int i = 0; i < 6; ++i) pfv[i] = (float)L[i];
  pfv[6] = (float)(L[0] * zv0);
  pfv[7] = (float)(L[1] * zv0 + L[2] * zv1);
  pfv[8] = (float)(L[3] * zv0 + L[4] * zv1 + L[5] * zv2);
  float* pf = B.ptf + 9 * (size_t)p;
#pragma unroll
  for (int i = 0; i < 9; ++i) pf[i] = pfv[i];
  if (pf_local)
#pragma unroll
    for (int i = 0; i < 9; ++i) pf_local[i] = pfv[i];
  const float l00 = pfv[0], l10 = pfv[1], l11 = pfv[2], l20 = pfv[3], l21 = pfv[4], l22 = pfv[5];
  for (uint32_t j = l0; j < l1; ++j) {  // lens entries (ba.rs:251-259)
    if (j > l0) {
#pragma unroll
      for (int i = 0; i < 9; ++i) Y[i] = 0.0f;
    }
    for (uint32_t k = s; k < e && j > l0; ++k) {
      if (S.obs_lens[k] != j) continue;
      const float* o = rec(k);
      if (o[27] == 0.0f) continue;
      const float w = o[26];
      const float j0 = o[12], j1 = o[13], j2 = o[14], j3 = o[15], j4 = o[16], j5 = o[17];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float ga = o[18 + a], gb = o[21 + a];
        Y[3 * a + 0] += (ga * j0 + gb * j3) * w;
        Y[3 * a + 1] += (ga * j1 + gb * j4) * w;
        Y[3 * a + 2] += (ga * j2 + gb * j5) * w;
      }
    }
    float* Zl = B.Zl + (size_t)j * 9;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float y0 = Y[3 * a], y1 = Y[3 * a + 1], y2 = Y[3 * a + 2];
      Zl[3 * a + 0] = y0 * l00 + y1 * l10 + y2 * l20;
      Zl[3 * a + 1] = y1 * l11 + y2 * l21;
      Zl[3 * a + 2] = y2 * l22;
    }
  }
}

// Pass 2, a thread per point: V and v summed in FP64 from the stored FP32
// records (products of FP32 numbers are exact in FP64, so V^-1 v is the
// exact least-squares step of the stored Jacobians and residuals), the
// damped inverse, its Cholesky factor, and the point's lens entries.  Points
// with cond(V) above kMixedCondLimit take the FP64 path of
// point_system_mixed_ill, which also writes their Z and gradient shares.
//
// A CTA takes kPtSolveThreads consecutive points, whose records are one
// contiguous range (observations are sorted by point).  The CTA stages the
// part of each record the sums read (Jp, Jg, e, w, valid: floats 12..27, one
// 16-byte-aligned 64-byte run) and its lens entry in shared memory, in rounds
// of kPtStageRecs records read with coalesced 16-byte loads; each thread then
// adds its own point's records in observation order, as a thread reading
// them from global memory would.
constexpr int kPtSolveThreads = 128;
constexpr int kPtStageRecs = 512;
constexpr int kPtStagePitch = 17;  // staged floats per record: lin[12..27], lens entry

static __global__ void __launch_bounds__(kPtSolveThreads, 6)
    point_solve_mixed_kernel(Prob P, StateView st, StructView S, IterBufs<float> B,
                             const int32_t* active, const double* lambda, const double* sigma) {
  __shared__ float srec[kPtStageRecs * kPtStagePitch];
  const int64_t pb = (int64_t)blockIdx.x * kPtSolveThreads;
  if (pb >= P.np) return;  // uniform over the CTA
  const int64_t pe = pb + kPtSolveThreads < P.np ? pb + kPtSolveThreads : P.np;
  const int64_t p = pb + threadIdx.x;
  const bool in = p < pe;
  const uint32_t m = in ? P.pt_model[p] : 0u;
  const bool act = in && active[m] != 0;
  if (!__syncthreads_or(act)) return;  // every point of the CTA in a finished model
  const uint32_t s = in ? S.pt_ptr[p] : 0u, e = in ? S.pt_ptr[p + 1] : 0u;
  const uint32_t l0 = in ? S.lens_ptr[p] : 0u, l1 = in ? S.lens_ptr[p + 1] : 0u;
  const bool sum = act && e - s >= 2;  // ba.rs:238
  // V and v as double-float sums of the stored FP32 values (about 48 bits:
  // V^-1 v stays the exact point step of the stored records to ~1e-10
  // relative for the well-conditioned points that use it), then FP64.
  float Vh[6] = {0, 0, 0, 0, 0, 0}, Vl[6] = {0, 0, 0, 0, 0, 0};
  float vh[3] = {0, 0, 0}, vl[3] = {0, 0, 0};
  // The point's first lens entry (usually its only one) sums Y = w Jg^T Jp in
  // the same pass (ba.rs:251-259); further entries take a second pass below.
  float Y[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const uint32_t rb = S.pt_ptr[pb], re = S.pt_ptr[pe];
  for (uint32_t c0 = rb; c0 < re; c0 += kPtStageRecs) {
    const uint32_t c1 = re - c0 < (uint32_t)kPtStageRecs ? re : c0 + kPtStageRecs;
    const uint32_t n = c1 - c0;
    for (uint32_t t = threadIdx.x; t < 4 * n; t += kPtSolveThreads) {
      const uint32_t r = t >> 2, q = t & 3;
      const float4 v = reinterpret_cast<const float4*>(B.lin + (size_t)(c0 + r) * kLinW + 12)[q];
      float* d = srec + r * kPtStagePitch + 4 * q;
      d[0] = v.x, d[1] = v.y, d[2] = v.z, d[3] = v.w;
    }
    for (uint32_t r = threadIdx.x; r < n; r += kPtSolveThreads)
      srec[r * kPtStagePitch + 16] = __uint_as_float(S.obs_lens[c0 + r]);
    __syncthreads();
    const uint32_t k0 = s > c0 ? s : c0, k1 = e < c1 ? e : c1;
    for (uint32_t k = sum ? k0 : k1; k < k1; ++k) {
      const float* o = srec + (k - c0) * kPtStagePitch;  // o[i] = lin[12 + i]
      if (o[15] == 0.0f) continue;                       // valid
      const float w = o[14];
      const float jp[6] = {o[0], o[1], o[2], o[3], o[4], o[5]};
      if (l1 > l0 && __float_as_uint(o[16]) == l0) {
        const float jg[6] = {o[6], o[7], o[8], o[9], o[10], o[11]};
#pragma unroll
        for (int t = 0; t < 3; ++t) {
          const float ga = jg[t], gb = jg[3 + t];
          Y[3 * t + 0] += (ga * jp[0] + gb * jp[3]) * w;
          Y[3 * t + 1] += (ga * jp[1] + gb * jp[4]) * w;
          Y[3 * t + 2] += (ga * jp[2] + gb * jp[5]) * w;
        }
      }
      float ph[6], pq[6];  // w jp = ph + pq exactly
#pragma unroll
      for (int i = 0; i < 6; ++i) ph[i] = w * jp[i], pq[i] = fmaf(w, jp[i], -ph[i]);
      // V (upper triangle 00 01 02 11 12 22) += w (jp_i jp_j + jp_{3+i} jp_{3+j})
      constexpr int VI[6] = {0, 0, 0, 1, 1, 2}, VJ[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
      for (int t = 0; t < 6; ++t) {
        df_add_prod(Vh[t], Vl[t], ph[VI[t]], pq[VI[t]], jp[VJ[t]]);
        df_add_prod(Vh[t], Vl[t], ph[3 + VI[t]], pq[3 + VI[t]], jp[3 + VJ[t]]);
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        df_add_prod(vh[i], vl[i], ph[i], pq[i], o[12]);
        df_add_prod(vh[i], vl[i], ph[3 + i], pq[3 + i], o[13]);
      }
    }
    __syncthreads();
  }
  if (!act) return;
  point_mixed_finish(P, st, S, B, p, m, s, e, l0, l1, sum, Vh, Vl, vh, vl, Y, lambda, sigma,
                     [&](uint32_t k) { return B.lin + (size_t)k * kLinW; }, nullptr);
}

// Pass 3, a thread per observation: Z = Y L (Y = w Jc^T Jp) and the
// observation's share of the reduced gradient, Jc^T r' and Jg^T r' with
// r' = w (e - Jp t), in FP32 from the record and the point's FP32 L and t.
// Observations of ill-conditioned points were written by pass 2.
static __global__ void __launch_bounds__(kObsThreads)
    obs_factor_kernel(Prob P, IterBufs<float> B, const int32_t* active) {
  __shared__ float smz[kObsWarps][32 * kZPitch];
  __shared__ float smg[kObsWarps][32 * kGPitch];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t k0 = (int64_t)blockIdx.x * kObsThreads + warp * 32;
  if (k0 >= P.no) return;
  const int64_t k = k0 + lane;
  float* Z = &smz[warp][lane * kZPitch];
  float* gs = &smg[warp][lane * kGPitch];
  bool mine = false;
  float fr0 = 0.0f, fr1 = 0.0f;  // r' for the camera-major record's tail
  if (k < P.no) {
    const uint32_t p = P.obs_pt[k];
    const uint8_t kp = B.kept[p];
    if (active[P.pt_model[p]] && kp != 2) {
      mine = true;
      const float4* o4 = reinterpret_cast<const float4*>(B.lin + (size_t)k * kLinW);
      float o[kLinW];
#pragma unroll
      for (int i = 0; i < kLinW / 4; ++i) {
        const float4 q = o4[i];
        o[4 * i] = q.x, o[4 * i + 1] = q.y, o[4 * i + 2] = q.z, o[4 * i + 3] = q.w;
      }
      if (kp == 0 || o[27] == 0.0f) {
#pragma unroll
        for (int i = 0; i < 18; ++i) Z[i] = 0.0f;
#pragma unroll
        for (int i = 0; i < 9; ++i) gs[i] = 0.0f;
        // a skipped point's observations leave the camera sums (ba.rs:274-277):
        // marked invalid in the record, which the camera pass then reads alone
        if (kp == 0 && o[27] != 0.0f) B.lin[(size_t)k * kLinW + 27] = 0.0f;
      } else {
        const float* pf = B.ptf + 9 * (size_t)p;
        const float l00 = pf[0], l10 = pf[1], l11 = pf[2], l20 = pf[3], l21 = pf[4], l22 = pf[5];
        const float t0 = pf[6], t1 = pf[7], t2 = pf[8];
        const float w = o[26];
        const float j0 = o[12], j1 = o[13], j2 = o[14], j3 = o[15], j4 = o[16], j5 = o[17];
        const float r0 = (o[24] - (j0 * t0 + j1 * t1 + j2 * t2)) * w;
        const float r1 = (o[25] - (j3 * t0 + j4 * t1 + j5 * t2)) * w;
        fr0 = r0, fr1 = r1;
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          const float ca = o[r], cb = o[6 + r];
          const float y0 = (ca * j0 + cb * j3) * w;
          const float y1 = (ca * j1 + cb * j4) * w;
          const float y2 = (ca * j2 + cb * j5) * w;
          Z[3 * r + 0] = y0 * l00 + y1 * l10 + y2 * l20;
          Z[3 * r + 1] = y1 * l11 + y2 * l21;
          Z[3 * r + 2] = y2 * l22;
          gs[r] = gshare(ca, cb, r0, r1);
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) gs[6 + a] = gshare(o[18 + a], o[21 + a], r0, r1);
      }
    }
  }
  const uint32_t mask = __ballot_sync(0xffffffffu, mine);
  __syncwarp();
  const int n = P.no - k0 < 32 ? (int)(P.no - k0) : 32;
  if (B.zpos) {
    // camera-major factors: each lane stores its own 96-byte record at its
    // camera-order position, with r' for the camera pass (which then needs
    // no gradient shares from here)
    if (mine) {
      float z[18];
#pragma unroll
      for (int i = 0; i < 18; ++i) z[i] = Z[i];
      store_Z24(B.Z + (size_t)B.zpos[k] * B.zpitch, z, fr0, fr1, 0.0f);
    }
  } else {
    if (B.Z) warp_store_records<18>(smz[warp], kZPitch, B.Z + k0 * 18, n, mask, lane);
    warp_store_records<9>(smg[warp], kGPitch, B.gsub + k0 * 9, n, mask, lane);
  }
}

// ---- mixed form: the three passes fused per chunk of observations ---------
//
// One CTA per chunk of kChunk consecutive observations.  Its points are those
// whose first observation lies in the chunk (fu_p0[b] .. fu_p0[b + 1], built
// by chunk_points_kernel), so its observations are one contiguous run of
// records: the chunk plus the rest of its last point's track.  The CTA
//   1. forms each record (a thread per observation) in shared memory and
//      copies the run to global memory, for the camera sums, with coalesced
//      stores;
//   2. sums each point's system from the shared records (a thread per point,
//      its observations in order) and keeps the point's FP32 factor and step
//      in shared memory;
//   3. forms each observation's Schur factor and gradient share (a thread per
//      observation) from its shared record and its point's shared factor,
//      staged for coalesced stores in the record slots the warp has read.
// The records cross HBM once (written) instead of three times (written, then
// read by the point and factor passes).  Every value comes from the same
// arithmetic in the same order as obs_record_kernel, point_solve_mixed_kernel
// and obs_factor_kernel, so the results are bit-identical to theirs.  Records
// beyond kCap of a run (a track longer than half a chunk at its end) are
// read back from global memory.
template <int kChunk>
struct FusedPoint {
  static constexpr int kThreads = kChunk;  // a thread per observation of the chunk
  static constexpr int kCap = kChunk * 3 / 2;
  static constexpr int kPtF = 10;  // per point slot: ptf (9) | kept
  static constexpr size_t kSmem =
      (size_t)kCap * kLinPitch * 4 + (size_t)kChunk * kPtF * 4 + (size_t)kCap * 4;
  static constexpr int kMinBlocks = 768 / kChunk;
};

// fu_p0[b] = the first point whose first observation is at or after b kChunk
// (b = 0 .. nchunks); the last entry is np.
static __global__ void chunk_points_kernel(int64_t np, const uint32_t* pt_ptr, uint32_t chunk,
                                           int64_t nchunks, uint32_t* fu_p0) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p == 0) fu_p0[0] = 0, fu_p0[nchunks] = (uint32_t)np;
  if (p >= np) return;
  const uint32_t lo = pt_ptr[p], hi = pt_ptr[p + 1];
  // chunk starts b kChunk in (lo, hi]: point p + 1 is the first at or after them
  for (int64_t b = lo / chunk + 1; b <= (int64_t)(hi / chunk) && b < nchunks; ++b)
    fu_p0[b] = (uint32_t)(p + 1);
}

template <int kChunk>
static __global__ void __launch_bounds__(FusedPoint<kChunk>::kThreads,
                                         FusedPoint<kChunk>::kMinBlocks)
    point_fused_mixed_kernel(Prob P, StateView st, StructView S, IterBufs<float> B,
                             const float* camf, const uint32_t* fu_p0, const int32_t* active,
                             const double* lambda, const double* sigma, const int32_t* stale) {
  using F = FusedPoint<kChunk>;
  constexpr int kCap = F::kCap, kThreads = F::kThreads;
  extern __shared__ __align__(16) float fu_sm[];
  float* srec = fu_sm;                                // [kCap][kLinPitch]
  float* spt = srec + (size_t)kCap * kLinPitch;       // [kChunk][kPtF]
  // per staged record: 1 if its model is active | 2 if formed here (else
  // loaded: the trial cost of an accepted step left it) | point slot << 2
  uint32_t* sslot = reinterpret_cast<uint32_t*>(spt + (size_t)kChunk * F::kPtF);
  const uint32_t p0 = fu_p0[blockIdx.x], p1 = fu_p0[blockIdx.x + 1];
  if (p0 >= p1) return;  // uniform over the CTA
  const uint32_t o_lo = S.pt_ptr[p0], n = S.pt_ptr[p1] - o_lo;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  auto rec = [&](uint32_t k) -> float* {
    const uint32_t j = k - o_lo;
    return j < (uint32_t)kCap ? srec + (size_t)j * kLinPitch : B.lin + (size_t)k * kLinW;
  };
  // 1. Records (as obs_record_kernel).
  for (uint32_t j = threadIdx.x; j < n; j += kThreads) {
    const uint32_t k = o_lo + j;
    const uint32_t m = P.pt_model[P.obs_pt[k]];
    const bool act = active[m] != 0;
    const bool form = act && (!stale || stale[m]);
    if (j < (uint32_t)kCap) sslot[j] = (act ? 1u : 0u) | (form ? 2u : 0u);
    if (!act) continue;
    float* out = rec(k);
    if (!form) {  // stage the stored record
      if (j < (uint32_t)kCap) {
        const float* src = B.lin + (size_t)k * kLinW;
#pragma unroll
        for (int i = 0; i < kLinW; ++i) out[i] = src[i];
      }
      continue;
    }
    const double sg = sigma[m];
    const float sg_f = (float)sg, inv_s2 = 1.0f / (sg_f * sg_f);
    float jpf[6], wf;
    double ev[2];
    if (!linearise_mixed(P, st, camf, k, sg, sg_f, inv_s2, P.model_refine[m] != 0, out, jpf, ev,
                         wf)) {
#pragma unroll
      for (int i = 0; i < kLinW; ++i) out[i] = 0.0f;
    }
  }
  __syncthreads();
  {  // staged records of active models out to global memory, contiguous
    const uint32_t ns = n < (uint32_t)kCap ? n : (uint32_t)kCap;
    float* dst = B.lin + (size_t)o_lo * kLinW;
    for (uint32_t i = threadIdx.x; i < ns * kLinW; i += kThreads) {
      const uint32_t j = i / kLinW;
      if (sslot[j] & 2u) dst[i] = srec[(size_t)j * kLinPitch + (i - j * kLinW)];
    }
  }
  // 2. Point systems (as point_solve_mixed_kernel).
  for (uint32_t p = p0 + threadIdx.x; p < p1; p += kThreads) {
    const uint32_t m = P.pt_model[p];
    const bool act = active[m] != 0;
    if (!act) continue;
    const uint32_t s = S.pt_ptr[p], e = S.pt_ptr[p + 1];
    const uint32_t l0 = S.lens_ptr[p], l1 = S.lens_ptr[p + 1];
    const uint32_t slot = s - o_lo;  // < kChunk for a point with observations
    for (uint32_t k = s; k < e; ++k)
      if (k - o_lo < (uint32_t)kCap) sslot[k - o_lo] |= slot << 2;
    const bool sum = e - s >= 2;  // ba.rs:238
    float Vh[6] = {0, 0, 0, 0, 0, 0}, Vl[6] = {0, 0, 0, 0, 0, 0};
    float vh[3] = {0, 0, 0}, vl[3] = {0, 0, 0};
    float Y[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t k = sum ? s : e; k < e; ++k) {
      const float* o = rec(k) + 12;  // o[i] = lin[12 + i]
      if (o[15] == 0.0f) continue;   // valid
      const float w = o[14];
      const float jp[6] = {o[0], o[1], o[2], o[3], o[4], o[5]};
      if (l1 > l0 && S.obs_lens[k] == l0) {
        const float jg[6] = {o[6], o[7], o[8], o[9], o[10], o[11]};
#pragma unroll
        for (int t = 0; t < 3; ++t) {
          const float ga = jg[t], gb = jg[3 + t];
          Y[3 * t + 0] += (ga * jp[0] + gb * jp[3]) * w;
          Y[3 * t + 1] += (ga * jp[1] + gb * jp[4]) * w;
          Y[3 * t + 2] += (ga * jp[2] + gb * jp[5]) * w;
        }
      }
      float ph[6], pq[6];  // w jp = ph + pq exactly
#pragma unroll
      for (int i = 0; i < 6; ++i) ph[i] = w * jp[i], pq[i] = fmaf(w, jp[i], -ph[i]);
      constexpr int VI[6] = {0, 0, 0, 1, 1, 2}, VJ[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
      for (int t = 0; t < 6; ++t) {
        df_add_prod(Vh[t], Vl[t], ph[VI[t]], pq[VI[t]], jp[VJ[t]]);
        df_add_prod(Vh[t], Vl[t], ph[3 + VI[t]], pq[3 + VI[t]], jp[3 + VJ[t]]);
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        df_add_prod(vh[i], vl[i], ph[i], pq[i], o[12]);
        df_add_prod(vh[i], vl[i], ph[3 + i], pq[3 + i], o[13]);
      }
    }
    float* pt_sm = e > s ? spt + (size_t)slot * F::kPtF : nullptr;
    point_mixed_finish(P, st, S, B, p, m, s, e, l0, l1, sum, Vh, Vl, vh, vl, Y, lambda, sigma,
                       rec, pt_sm);
    if (pt_sm) pt_sm[9] = __uint_as_float((uint32_t)B.kept[p]);
  }
  __syncthreads();
  // 3. Schur factors and gradient shares (as obs_factor_kernel).
  for (uint32_t j0 = (uint32_t)warp * 32; j0 < n; j0 += kThreads) {
    const uint32_t j = j0 + lane, k = o_lo + j;
    bool mine = false;
    float Z[18], gs[9];
    float fr0 = 0.0f, fr1 = 0.0f;  // r' for the camera-major record's tail
    if (j < n) {
      const uint32_t p = P.obs_pt[k];
      bool act;
      uint32_t slot;
      if (j < (uint32_t)kCap) {
        const uint32_t sl = sslot[j];
        act = (sl & 1u) != 0, slot = sl >> 2;
      } else {
        act = active[P.pt_model[p]] != 0, slot = S.pt_ptr[p] - o_lo;
      }
      const float* pf = spt + (size_t)slot * F::kPtF;
      const uint32_t kp = act ? __float_as_uint(pf[9]) : 0u;
      if (act && kp != 2) {
        mine = true;
        const float* o = rec(k);
        if (kp == 0 || o[27] == 0.0f) {
#pragma unroll
          for (int i = 0; i < 18; ++i) Z[i] = 0.0f;
#pragma unroll
          for (int i = 0; i < 9; ++i) gs[i] = 0.0f;
          // as obs_factor_kernel: a skipped point's observation is marked
          // invalid in the stored record for the camera pass
          if (kp == 0 && o[27] != 0.0f) B.lin[(size_t)k * kLinW + 27] = 0.0f;
        } else {
          const float l00 = pf[0], l10 = pf[1], l11 = pf[2], l20 = pf[3], l21 = pf[4],
                      l22 = pf[5];
          const float t0 = pf[6], t1 = pf[7], t2 = pf[8];
          const float w = o[26];
          const float j0v = o[12], j1 = o[13], j2 = o[14], j3 = o[15], j4 = o[16], j5 = o[17];
          const float r0 = (o[24] - (j0v * t0 + j1 * t1 + j2 * t2)) * w;
          const float r1 = (o[25] - (j3 * t0 + j4 * t1 + j5 * t2)) * w;
          fr0 = r0, fr1 = r1;
#pragma unroll
          for (int r = 0; r < 6; ++r) {
            const float ca = o[r], cb = o[6 + r];
            const float y0 = (ca * j0v + cb * j3) * w;
            const float y1 = (ca * j1 + cb * j4) * w;
            const float y2 = (ca * j2 + cb * j5) * w;
            Z[3 * r + 0] = y0 * l00 + y1 * l10 + y2 * l20;
            Z[3 * r + 1] = y1 * l11 + y2 * l21;
            Z[3 * r + 2] = y2 * l22;
            gs[r] = gshare(ca, cb, r0, r1);
          }
#pragma unroll
          for (int a = 0; a < 3; ++a) gs[6 + a] = gshare(o[18 + a], o[21 + a], r0, r1);
        }
      }
    }
    const uint32_t mask = __ballot_sync(0xffffffffu, mine);
    const int nw = n - j0 < 32u ? (int)(n - j0) : 32;
    if (B.zpos) {  // camera-major factors: each lane stores its own record, with r'
      if (mine) store_Z24(B.Z + (size_t)B.zpos[k] * B.zpitch, Z, fr0, fr1, 0.0f);
    }
    if (j0 + 32 <= (uint32_t)kCap) {
      // the warp's 32 record slots (read above) stage its stores
      __syncwarp();
      float* stg = srec + (size_t)j0 * kLinPitch;  // 32 x 29 floats
      float* stz = stg;                            // [32][kZPitch]
      float* stgs = stg + 32 * kZPitch;            // [32][kGPitch]
      if (mine) {
#pragma unroll
        for (int i = 0; i < 18; ++i) stz[lane * kZPitch + i] = Z[i];
#pragma unroll
        for (int i = 0; i < 9; ++i) stgs[lane * kGPitch + i] = gs[i];
      }
      __syncwarp();
      if (!B.zpos) {  // camera-major records carry r' instead of the shares
        if (B.Z)
          warp_store_records<18>(stz, kZPitch, B.Z + (size_t)(o_lo + j0) * 18, nw, mask, lane);
        warp_store_records<9>(stgs, kGPitch, B.gsub + (size_t)(o_lo + j0) * 9, nw, mask, lane);
      }
    } else if (mine && !B.zpos) {
      if (B.Z)
#pragma unroll
        for (int i = 0; i < 18; ++i) B.Z[(size_t)k * 18 + i] = Z[i];
#pragma unroll
      for (int i = 0; i < 9; ++i) B.gsub[(size_t)k * 9 + i] = gs[i];
    }
  }
}

// ---- per camera: U, g, lens terms (ba.rs:273-292) ----------------------------

constexpr int kCamThreads = 128;
constexpr int kCamN = 45;  // 21 U | 18 X | 6 lens U     (storage precision)
constexpr int kCamG = 18;  // 6 gj | 6 gs | 3 lg | 3 ls  (FP64)

// FP64 form, per camera (ba.rs:273-292): every sum in FP64; a CTA per camera,
// its observations gathered through the camera ordering.  (The mixed form
// runs camera_mixed_kernel.)
template <typename R>
__global__ void __launch_bounds__(kCamThreads)
    camera_kernel(Prob P, StructView S, IterBufs<R> B, const int32_t* active) {
  static_assert(sizeof(R) == 8, "the mixed form runs camera_mixed_kernel");
  __shared__ double scratch[kCamN * 32];
  __shared__ double gscratch[kCamG * 32];
  const int64_t c = blockIdx.x;
  if (c >= P.nc) return;
  const uint32_t m = P.cam_model[c];
  if (!active[m]) return;
  const bool refine = P.model_refine[m] != 0;
  double accd[kCamN];
  double gacc[kCamG];
#pragma unroll
  for (int i = 0; i < kCamN; ++i) accd[i] = 0.0;
#pragma unroll
  for (int i = 0; i < kCamG; ++i) gacc[i] = 0.0;
  const uint32_t b = S.cam_ptr[c], e = S.cam_ptr[c + 1];
  for (uint32_t i = b + threadIdx.x; i < e; i += blockDim.x) {
    const uint32_t k = S.cam_obs[i];
    const double* o = B.lin + (size_t)k * kLinW;
    if (o[27] == 0.0 || !B.kept[P.obs_pt[k]]) continue;  // ba.rs:274-277
    const double w = o[26];
    double jc[12];
#pragma unroll
    for (int t = 0; t < 12; ++t) jc[t] = o[t];
    int u = 0;
#pragma unroll
    for (int a = 0; a < 6; ++a)
#pragma unroll
      for (int bb = a; bb < 6; ++bb) accd[u++] += (jc[a] * jc[bb] + jc[6 + a] * jc[6 + bb]) * w;
    const double* gs = B.gsub + (size_t)k * 9;
    const double e0 = o[24], e1 = o[25];
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      gacc[a] += (jc[a] * e0 + jc[6 + a] * e1) * w;
      gacc[6 + a] += gs[a];
    }
    if (refine) {
      const double jg[6] = {o[18], o[19], o[20], o[21], o[22], o[23]};
#pragma unroll
      for (int a = 0; a < 6; ++a)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb)
          accd[21 + 3 * a + bb] += (jc[a] * jg[bb] + jc[6 + a] * jg[3 + bb]) * w;
      int v = 0;
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int bb = a; bb < 3; ++bb) accd[39 + v++] += (jg[a] * jg[bb] + jg[3 + a] * jg[3 + bb]) * w;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        gacc[12 + a] += (jg[a] * e0 + jg[3 + a] * e1) * w;
        gacc[15 + a] += gs[6 + a];
      }
    }
  }
  block_sum<kCamN>(accd, scratch);
  block_sum<kCamG>(gacc, gscratch);
  if (threadIdx.x == 0) {
    double* U = B.camU + 21 * c;
    for (int i = 0; i < 21; ++i) U[i] = accd[i];
    for (int i = 0; i < 6; ++i) B.camgj[6 * c + i] = gacc[i], B.camgs[6 * c + i] = gacc[6 + i];
    for (int i = 0; i < 18; ++i) B.camX[18 * c + i] = accd[21 + i];
    for (int i = 0; i < 6; ++i) B.caml[12 * c + i] = accd[39 + i];
    for (int i = 0; i < 6; ++i) B.caml[12 * c + 6 + i] = gacc[12 + i];
  }
}

// Mixed form, per camera (ba.rs:273-292): U = sum w Jc^T Jc (21), X = sum w
// Jc^T Jg (18), the lens block (6), and the sums of the observations' reduced-
// gradient shares.  Products are FP32; every lane sums runs of kCamRun
// observations in FP32, the warp adds its lanes' runs by a fixed butterfly and
// folds the result into FP64 sums spread over its lanes (lane l holds entries
// l and l + 32); the gradient shares are summed per lane as double-float
// pairs (about 48 bits) and then in FP64.  The
// warps' FP64 sums are added in warp order: the result does not depend on
// timing.  A camera sees thousands of observations: plain FP32 accumulation
// would bury the weak, prior-only directions of the reduced system.
constexpr int kCamMixThreads = 256;
constexpr int kCamMixWarps = kCamMixThreads / 32;
constexpr int kCamRun = 8;

static __global__ void __launch_bounds__(kCamMixThreads)
    camera_mixed_kernel(Prob P, StructView S, IterBufs<float> B, const int32_t* active) {
  __shared__ double part[kCamMixWarps][kCamN + 9];
  const int64_t c = blockIdx.x;
  if (c >= P.nc) return;
  const uint32_t m = P.cam_model[c];
  if (!active[m]) return;
  const bool refine = P.model_refine[m] != 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float acc[kCamN];
#pragma unroll
  for (int i = 0; i < kCamN; ++i) acc[i] = 0.0f;
  double lo = 0.0, hi = 0.0;  // this lane's FP64 sums of entries lane, lane + 32
  float gh[9], gl[9];         // gradient shares, double-float
#pragma unroll
  for (int i = 0; i < 9; ++i) gh[i] = 0.0f, gl[i] = 0.0f;
  const uint32_t b = S.cam_ptr[c], e = S.cam_ptr[c + 1];
  // camera-major factor records (zpitch 24) carry each observation's r'
  const bool tail = B.zpos != nullptr && B.Z != nullptr && B.zpitch == 24;
  for (uint32_t base = b; base < e; base += kCamMixThreads * kCamRun) {
    // The next observation's index is loaded one step ahead, and a record is
    // read whole before its validity is tested: two dependent loads per step.
    uint32_t i = base + threadIdx.x;
    uint32_t k = i < e ? S.cam_obs[i] : 0u;
#pragma unroll 1
    for (int j = 0; j < kCamRun; ++j) {
      if (i >= e) break;
      const uint32_t in = i + kCamMixThreads;
      const uint32_t kn = (j + 1 < kCamRun && in < e) ? S.cam_obs[in] : 0u;
      const float4* o4 = reinterpret_cast<const float4*>(B.lin + (size_t)k * kLinW);
      const float4 q6 = o4[6];  // e 24..25, w 26, valid 27
      const float4 q0 = o4[0], q1 = o4[1], q2 = o4[2];
      // Gradient shares: with camera-major factor records, from r' in the
      // record at this camera-order position (mode 1: from gsub); else gsub.
      const float* gs = B.gsub + (size_t)k * 9;
      float4 tl = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // z16 z17 r0 r1
      float md = 1.0f;
      float gv[6];
      if (tail) {
        const float* zr = B.Z + (size_t)i * 24;
        tl = *reinterpret_cast<const float4*>(zr + 16);
        md = zr[kZ24Mode];
      } else {
#pragma unroll
        for (int a = 0; a < 6; ++a) gv[a] = gs[a];
      }
      i = in, k = kn;
      // ba.rs:274-277: the factor pass marked the observations of skipped
      // points (kept 0) invalid, so the record's flag is the whole test
      if (q6.w == 0.0f) continue;
      const float jc[12] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x, q2.y, q2.z, q2.w};
      const float w = q6.z;
      const bool from_r = tail && md == 0.0f;
      if (from_r) {
#pragma unroll
        for (int a = 0; a < 6; ++a) gv[a] = gshare(jc[a], jc[6 + a], tl.z, tl.w);
      } else if (tail) {
#pragma unroll
        for (int a = 0; a < 6; ++a) gv[a] = gs[a];
      }
      int u = 0;
#pragma unroll
      for (int a = 0; a < 6; ++a)
#pragma unroll
        for (int bb = a; bb < 6; ++bb) acc[u++] += (jc[a] * jc[bb] + jc[6 + a] * jc[6 + bb]) * w;
#pragma unroll
      for (int a = 0; a < 6; ++a) df_add(gh[a], gl[a], gv[a]);
      if (refine) {
        const float4 q4 = o4[4], q5 = o4[5];
        const float jg[6] = {q4.z, q4.w, q5.x, q5.y, q5.z, q5.w};
#pragma unroll
        for (int a = 0; a < 6; ++a)
#pragma unroll
          for (int bb = 0; bb < 3; ++bb)
            acc[21 + 3 * a + bb] += (jc[a] * jg[bb] + jc[6 + a] * jg[3 + bb]) * w;
        int v = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int bb = a; bb < 3; ++bb)
            acc[39 + v++] += (jg[a] * jg[bb] + jg[3 + a] * jg[3 + bb]) * w;
#pragma unroll
        for (int a = 0; a < 3; ++a)
          df_add(gh[6 + a], gl[6 + a], from_r ? gshare(jg[a], jg[3 + a], tl.z, tl.w) : gs[6 + a]);
      }
    }
    // Warp-uniform: fold these runs' FP32 sums into the lanes' FP64 sums.
    float mlo = 0.0f, mhi = 0.0f;
#pragma unroll
    for (int t = 0; t < kCamN; ++t) {
      const float sum = warp_sum(acc[t]);
      acc[t] = 0.0f;
      if (t < 32) mlo = lane == t ? sum : mlo;
      else mhi = lane == t - 32 ? sum : mhi;
    }
    lo += f2d_exact(mlo);
    hi += f2d_exact(mhi);
  }
  double gacc[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) gacc[i] = warp_sum(f2d_exact(gh[i]) + f2d_exact(gl[i]));
  part[warp][lane] = lo;
  if (lane + 32 < kCamN) part[warp][lane + 32] = hi;
  if (lane < 9) {
    double g = gacc[0];
#pragma unroll
    for (int i = 1; i < 9; ++i) g = lane == i ? gacc[i] : g;
    part[warp][kCamN + lane] = g;
  }
  __syncthreads();
  const int t = threadIdx.x;
  if (t < kCamN + 9) {
    double v = 0.0;
#pragma unroll
    for (int w = 0; w < kCamMixWarps; ++w) v += part[w][t];
    if (t < 21) B.camU[21 * c + t] = v;
    else if (t < 39) B.camX[18 * c + (t - 21)] = v;
    else if (t < kCamN) B.caml[12 * c + (t - 39)] = v;
    else if (t < kCamN + 6) B.camgj[6 * c + (t - kCamN)] = v, B.camgs[6 * c + (t - kCamN)] = 0.0;
    else B.caml[12 * c + 6 + (t - kCamN - 6)] = v, B.caml[12 * c + 9 + (t - kCamN - 6)] = 0.0;
  }
}

// ---- per lens group: sum of its cameras' lens terms, in camera order ---------

static __global__ void __launch_bounds__(128)
    group_kernel(Prob P, StructView S, const double* caml, double* grpU, double* grpg,
                 const int32_t* active) {
  const int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (g >= P.ng) return;
  if (!active[P.blk_model[P.grp_blk[g]]]) return;
  double acc[12];
#pragma unroll
  for (int i = 0; i < 12; ++i) acc[i] = 0.0;
  for (uint32_t i = S.grp_ptr[g] + lane; i < S.grp_ptr[g + 1]; i += 32) {
    const double* l = caml + 12 * (size_t)S.grp_cams[i];
#pragma unroll
    for (int t = 0; t < 12; ++t) acc[t] += l[t];
  }
#pragma unroll
  for (int i = 0; i < 12; ++i) acc[i] = warp_sum(acc[i]);
  if (lane == 0) {
    for (int i = 0; i < 6; ++i) grpU[6 * g + i] = acc[i];
    for (int i = 0; i < 3; ++i) grpg[3 * g + i] = acc[6 + i] - acc[9 + i];
  }
}

// ---- robust cost (ba.rs:103-128), per model ---------------------------------

constexpr int kCostThreads = 256;

static __global__ void __launch_bounds__(kCostThreads)
    cost_chunk_kernel(Prob P, StateView st, StructView S, double* part, const int32_t* active,
                      const double* sigma) {
  __shared__ double scratch[3 * 32];
  const int64_t ch = blockIdx.x;
  if (ch >= S.ncost) return;
  const uint32_t m = S.cost_chunk_model[ch];
  if (active && !active[m]) return;
  const double sg = sigma[m];
  const double s2 = sg * sg, inv_s2 = 1.0 / s2;
  const double behind = s2 * 10.0;  // ba.rs:116
  const bool cauchy = P.loss == LOSS_CAUCHY;
  // Cauchy: sum_k s^2 ln(1 + e_k^2/s^2) = s^2 ln(prod_k (1 + e_k^2/s^2)).  The
  // factors (each >= 1) are multiplied into `prod`, kept in [1, 2) by moving
  // its binary exponent into `expo` after every product, and one logarithm
  // per thread closes the sum: FP64 throughout, one rounding per product
  // instead of one logarithm per observation.
  double prod = 1.0;
  int64_t expo = 0;
  double acc[3] = {0.0, 0.0, 0.0};
  uint32_t nfront = 0;  // in-front count (acc[2], exact in FP64 at the end)
  for (uint32_t k = S.cost_chunk_begin[ch] + threadIdx.x; k < S.cost_chunk_end[ch];
       k += blockDim.x) {
    const uint32_t cam = P.obs_cam[k];
    const double* K = st.intr + 5 * (size_t)P.cam_group[cam];
    double xc[3];
    bacam::to_cam(st.rot + 9 * (size_t)cam, st.center + 3 * (size_t)cam,
                  st.points + 3 * (size_t)P.obs_pt[k], xc);
    if (xc[2] > 1e-6) {  // Pose::project (geometry.rs:28-32, 66-72)
      const double iz = __drcp_rn(xc[2]);  // IEEE 1 / z, as a reciprocal
      const double px = xc[0] * iz, py = xc[1] * iz;
      const double r2 = px * px + py * py;
      const double d = 1.0 + K[3] * r2 + K[4] * r2 * r2;
      const double ex = P.obs_uv[2 * (size_t)k] - (K[0] * d * px + K[1]);
      const double ey = P.obs_uv[2 * (size_t)k + 1] - (K[0] * d * py + K[2]);
      const double e2 = ex * ex + ey * ey;
      if (cauchy) {
        const double q = 1.0 + e2 * inv_s2;  // ba.rs:114
        if (__double_as_longlong(q) < kQMaxBits) {  // q < 1e300 (q >= 1 or NaN)
          prod *= q;
          const int hi = __double2hiint(prod);
          expo += (hi >> 20) - 1023;
          prod = __hiloint2double((hi & 0x800FFFFF) | (1023 << 20), __double2loint(prod));
        } else {
          acc[0] += s2 * log(q);
        }
      } else {
        acc[0] += robust_rho(e2, sg, P.loss);
      }
      acc[1] += e2;
      ++nfront;
    } else {
      acc[0] += behind;
    }
  }
  if (cauchy) acc[0] += s2 * (log(prod) + (double)expo * 0.69314718055994530942);
  acc[2] = (double)nfront;
  block_sum<3>(acc, scratch);
  if (threadIdx.x == 0) {
    part[3 * ch] = acc[0];
    part[3 * ch + 1] = acc[1];
    part[3 * ch + 2] = acc[2];
  }
}

// Mixed form: the robust cost of a state (as cost_chunk_kernel, bit for bit)
// and, for the models in `active`, every observation's FP32 record at that
// state, formed from the same FP64 point in camera coordinates and the same
// FP64 residual the cost uses (the residual's FP64 projection is the costly
// part of a record on this GPU).  Called on the trial state of every LM
// iteration: when the step is accepted those records are the next
// iteration's, and the record pass skips the model (rec_stale); when it is
// rejected the record pass forms them again at the restored state.
static __global__ void __launch_bounds__(kCostThreads)
    cost_record_kernel(Prob P, StateView st, StructView S, IterBufs<float> B, const float* camf,
                       double* part, const int32_t* active, const double* sigma) {
  __shared__ double scratch[3 * 32];
  __shared__ float sm[kCostThreads / 32][32 * kLinPitch];
  const int64_t ch = blockIdx.x;
  if (ch >= S.ncost) return;
  const uint32_t m = S.cost_chunk_model[ch];
  if (active && !active[m]) return;
  const double sg = sigma[m];
  const double s2 = sg * sg, inv_s2 = 1.0 / s2;
  const double behind = s2 * 10.0;  // ba.rs:116
  const bool cauchy = P.loss == LOSS_CAUCHY;
  const float sg_f = (float)sg, inv_s2f = 1.0f / (sg_f * sg_f);
  const bool refine = P.model_refine[m] != 0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double prod = 1.0;  // as cost_chunk_kernel
  int64_t expo = 0;
  double acc[3] = {0.0, 0.0, 0.0};
  uint32_t nfront = 0;  // in-front count (acc[2], exact in FP64 at the end)
  const uint32_t c1 = S.cost_chunk_end[ch];
  // thread t takes observations begin + t, begin + t + blockDim, ... (the
  // order of cost_chunk_kernel); a warp's 32 records are staged and stored
  // as contiguous runs
  for (uint32_t kb = S.cost_chunk_begin[ch] + warp * 32; kb < c1; kb += blockDim.x) {
    const uint32_t k = kb + lane;
    float* rec = &sm[warp][lane * kLinPitch];
    if (k < c1) {
      const uint32_t cam = P.obs_cam[k];
      const double* K = st.intr + 5 * (size_t)P.cam_group[cam];
      double xc[3];
      bacam::to_cam(st.rot + 9 * (size_t)cam, st.center + 3 * (size_t)cam,
                    st.points + 3 * (size_t)P.obs_pt[k], xc);
      if (xc[2] > 1e-6) {  // Pose::project (geometry.rs:28-32, 66-72)
        const double iz = __drcp_rn(xc[2]);  // IEEE 1 / z, as a reciprocal
        const double px = xc[0] * iz, py = xc[1] * iz;
        const double r2 = px * px + py * py;
        const double d = 1.0 + K[3] * r2 + K[4] * r2 * r2;
        double ev[2];
        ev[0] = P.obs_uv[2 * (size_t)k] - (K[0] * d * px + K[1]);
        ev[1] = P.obs_uv[2 * (size_t)k + 1] - (K[0] * d * py + K[2]);
        const double e2 = ev[0] * ev[0] + ev[1] * ev[1];
        if (cauchy) {
          const double q = 1.0 + e2 * inv_s2;  // ba.rs:114
          if (__double_as_longlong(q) < kQMaxBits) {  // q < 1e300 (q >= 1 or NaN)
            prod *= q;
            const int hi = __double2hiint(prod);
            expo += (hi >> 20) - 1023;
            prod = __hiloint2double((hi & 0x800FFFFF) | (1023 << 20), __double2loint(prod));
          } else {
            acc[0] += s2 * log(q);
          }
        } else {
          acc[0] += robust_rho(e2, sg, P.loss);
        }
        acc[1] += e2;
        ++nfront;
        float jpf[6], wf;
        mixed_record_from(P, st, camf, k, sg, sg_f, inv_s2f, refine, xc, ev, rec, jpf, wf);
      } else {
        acc[0] += behind;
#pragma unroll
        for (int i = 0; i < kLinW; ++i) rec[i] = 0.0f;
      }
    }
    __syncwarp();
    const int n = c1 - kb < 32u ? (int)(c1 - kb) : 32;
    warp_store_records<kLinW>(sm[warp], kLinPitch, B.lin + (size_t)kb * kLinW, n, 0xffffffffu,
                              lane);
    __syncwarp();
  }
  if (cauchy) acc[0] += s2 * (log(prod) + (double)expo * 0.69314718055994530942);
  acc[2] = (double)nfront;
  block_sum<3>(acc, scratch);
  if (threadIdx.x == 0) {
    part[3 * ch] = acc[0];
    part[3 * ch + 1] = acc[1];
    part[3 * ch + 2] = acc[2];
  }
}

// CTA per model: the chunk partials and the GPS prior term over the model's
// cameras (ba.rs:103-128), summed in a fixed order (strided per thread, then
// the block's fixed tree).
constexpr int kCostFinalThreads = 256;

static __global__ void __launch_bounds__(kCostFinalThreads)
    cost_final_kernel(Prob P, StateView st, StructView S, const double* part,
                      const int32_t* active, double* cost, double* sq, int64_t* n_front) {
  __shared__ double scratch[4 * 32];
  const int64_t m = blockIdx.x;
  if (m >= P.nm) return;
  if (active && !active[m]) return;
  double a[4] = {0.0, 0.0, 0.0, 0.0};  // robust cost, squared residuals, count, prior
  for (uint32_t c = S.model_chunk0[m] + threadIdx.x; c < S.model_chunk0[m + 1]; c += blockDim.x)
    for (int i = 0; i < 3; ++i) a[i] += part[3 * (size_t)c + i];
  if (P.prior_mask) {
    for (uint32_t c = P.model_cam0[m] + threadIdx.x; c < P.model_cam0[m + 1]; c += blockDim.x) {
      if (!P.prior_mask[c]) continue;
      const double* q = P.prior + 6 * (size_t)c;
      const double dx = st.center[3 * (size_t)c] - q[0];
      const double dy = st.center[3 * (size_t)c + 1] - q[1];
      const double dz = st.center[3 * (size_t)c + 2] - q[2];
      a[3] += (dx / q[3]) * (dx / q[3]) + (dy / q[4]) * (dy / q[4]) + (dz / q[5]) * (dz / q[5]);
    }
  }
  block_sum<4>(a, scratch);
  if (threadIdx.x == 0) {
    cost[m] = a[0] + a[3];
    sq[m] = a[1];
    n_front[m] = (int64_t)a[2];
  }
}

// ---- LM accept / reject (ba.rs:367-383), thread per model --------------------

static __global__ void control_kernel(int64_t nm, Control C) {
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nm) return;
  if (!C.active[m]) {
    C.accepted[m] = 0;
    return;
  }
  const int32_t it = C.iters[m];
  C.iters[m] = it + 1;
  C.pcg_total[m] += C.pcg_iters[m];
  const double nc = C.new_cost[m], c = C.cost[m], lam = C.lambda[m];
  int32_t act = 1, acc = 0;
  if (nc < c) {
    acc = 1;
    const double rel = (c - nc) / fmax(c, 1e-12);
    C.cost[m] = nc;
    C.lambda[m] = fmax(lam / 3.0, 1e-9);
    // ba.rs:372-374 stops on the first such step (patience 1, the default);
    // a larger patience waits for that many consecutive ones, for inexact
    // inner solves that can give one small decrease before the minimum.
    if (rel < 1e-6) {
      if (++C.small[m] >= C.patience) act = 0;
    } else {
      C.small[m] = 0;
    }
    // Inexact-Newton forcing (Eisenstat and Walker, SIAM J. Sci. Comput. 17,
    // 1996): the inner solves tighten as the outer iteration converges.
    if (C.end_cap > 0 && rel < C.end_rel) C.pcg_cap[m] = C.end_cap;
  } else {
    C.lambda[m] = lam * 5.0;
    if (C.lambda[m] > 1e6) act = 0;
  }
  if (it + 1 >= C.max_iter) act = 0;
  C.accepted[m] = acc;
  C.active[m] = act;
  // mixed form: the trial cost left the records of the trial state; they are
  // the current state's only if the step was accepted
  if (C.rec_stale) C.rec_stale[m] = acc ? 0 : 1;
  if (act) atomicOr(C.any_active, 1);
  if (m == 0 && it < C.log_cap) {
    C.log_new_cost[it] = nc;
    C.log_lambda[it] = lam;
    C.log_pcg[it] = C.pcg_iters[m];
    C.log_accept[it] = acc;
  }
}

// Copy the trial state of accepted models over the current state.
static __global__ void commit_kernel(Prob P, const uint32_t* grp_model, StateView cur, StateView trial,
                              const int32_t* accepted) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < P.np && accepted[P.pt_model[i]])
    for (int a = 0; a < 3; ++a) cur.points[3 * i + a] = trial.points[3 * i + a];
  if (i < P.nc && accepted[P.cam_model[i]]) {
    for (int a = 0; a < 9; ++a) cur.rot[9 * i + a] = trial.rot[9 * i + a];
    for (int a = 0; a < 3; ++a) cur.center[3 * i + a] = trial.center[3 * i + a];
  }
  if (i < P.ng && accepted[grp_model[i]])
    for (int a = 0; a < 5; ++a) cur.intr[5 * i + a] = trial.intr[5 * i + a];
}

// ---- Schur sums: warp per sub-segment of one destination block ---------------

// An observation's Z (18 values) with vector loads: 144-byte records are
// 16-byte aligned (FP64: 9 x 16 B), 72-byte records 8-byte aligned (FP32:
// 9 x 8 B).
__device__ __forceinline__ void load_Z18(const double* s, double* z) {
  const double2* v = reinterpret_cast<const double2*>(s);
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const double2 t = __ldg(v + i);
    z[2 * i] = t.x, z[2 * i + 1] = t.y;
  }
}
// An FP32 record of 72 bytes starts on an 8-byte boundary: read the 80 bytes
// from the 16-byte boundary at or below it as five 16-byte loads (Z is
// allocated with 16 bytes of padding after its last record).
__device__ __forceinline__ void load_Z18(const float* s, float* z) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(s);
  const float4* v = reinterpret_cast<const float4*>(a & ~(uintptr_t)15);
  const bool off = (a & 15) != 0;
  float f[20];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    const float4 t = __ldg(v + i);
    f[4 * i] = t.x, f[4 * i + 1] = t.y, f[4 * i + 2] = t.z, f[4 * i + 3] = t.w;
  }
#pragma unroll
  for (int i = 0; i < 18; ++i) z[i] = off ? f[i + 2] : f[i];
}

// A 96-byte-aligned FP32 record of the camera-major layout: two 32-byte
// loads and one 8-byte load (three sectors, three L1 requests per lane where
// five 16-byte loads of a 72-byte record make five).
__device__ __forceinline__ void load_Z24(const float* s, float* z) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(z[0]), "=f"(z[1]), "=f"(z[2]), "=f"(z[3]), "=f"(z[4]), "=f"(z[5]), "=f"(z[6]),
        "=f"(z[7])
      : "l"(s));
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(z[8]), "=f"(z[9]), "=f"(z[10]), "=f"(z[11]), "=f"(z[12]), "=f"(z[13]), "=f"(z[14]),
        "=f"(z[15])
      : "l"(s + 8));
  const float2 t = __ldg(reinterpret_cast<const float2*>(s + 16));
  z[16] = t.x, z[17] = t.y;
}
__device__ __forceinline__ void load_Z24(const double*, double*) {}  // FP32 layout only

template <typename R>
__device__ __forceinline__ void load_Z(const IterBufs<R>& B, int64_t no, uint32_t eid, R* z) {
  if ((int64_t)eid < no) {
    if (sizeof(R) == 4 && B.zpitch == 24)
      load_Z24(B.Z + (size_t)eid * 24, z);
    else
      load_Z18(B.Z + (size_t)eid * B.zpitch, z);
  } else {
    const R* s = B.Zl + (size_t)(eid - no) * 9;
#pragma unroll
    for (int i = 0; i < 9; ++i) z[i] = s[i];
#pragma unroll
    for (int i = 9; i < 18; ++i) z[i] = (R)0;
  }
}

template <typename R>
// FP32 form: 3 CTAs per SM (80 registers; the kernel is bound by the latency
// of its gathers, and the extra resident warps hide more of it).
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 3 : 1)
    schur_kernel(Prob P, StructView S, IterBufs<R> B, const int32_t* active) {
  const int64_t sub = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (sub >= S.nsub) return;
  const uint32_t slot = S.sub_slot[sub];
  if (!active[P.blk_model[S.slot_row[slot]]]) return;
  R acc[36];
#pragma unroll
  for (int i = 0; i < 36; ++i) acc[i] = (R)0;
  const uint32_t b = S.sub_begin[sub], e = S.sub_end[sub];
  // The next pair's entry is loaded while this pair's factors are gathered
  // and multiplied (one dependent load less per pair on the critical path).
  uint64_t nxt = b + lane < e ? S.pairs[b + lane] : kSentinel;
  for (uint32_t i = b + lane; i < e; i += 32) {
    const uint64_t pr = nxt;
    nxt = i + 32 < e ? S.pairs[i + 32] : kSentinel;
    if (pr == kSentinel) continue;
    if ((int64_t)(pr & 0xffffffffu) >= P.no + S.nl || (int64_t)(pr >> 32) >= P.no + S.nl) continue;
    R za[18], zb[18];
    load_Z(B, P.no, (uint32_t)(pr & 0xffffffffu), za);
    load_Z(B, P.no, (uint32_t)(pr >> 32), zb);
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int c = 0; c < 6; ++c)
        acc[6 * r + c] += za[3 * r] * zb[3 * c] + za[3 * r + 1] * zb[3 * c + 1] +
                          za[3 * r + 2] * zb[3 * c + 2];
  }
  // Warp sum of the 36 entries, halving twice (36 -> 18 -> 9 values per lane)
  // before a butterfly on the last 9: 54 adds per lane instead of 180 (the
  // adds are FP64 warp instructions in the plain form).  Lanes 0, 8, 16, 24
  // then hold entries 0-8, 9-17, 18-26, 27-35.
  R a[18];
  {
    const bool up = lane & 16;
#pragma unroll
    for (int i = 0; i < 18; ++i) {
      const R recv = __shfl_xor_sync(kFull, up ? acc[i] : acc[18 + i], 16);
      a[i] = (up ? acc[18 + i] : acc[i]) + recv;
    }
  }
  R v[9];
  {
    const bool up = lane & 8;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      const R recv = __shfl_xor_sync(kFull, up ? a[i] : a[9 + i], 8);
      v[i] = (up ? a[9 + i] : a[i]) + recv;
    }
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    v[i] += __shfl_xor_sync(kFull, v[i], 4);
    v[i] += __shfl_xor_sync(kFull, v[i], 2);
    v[i] += __shfl_xor_sync(kFull, v[i], 1);
  }
  if ((lane & 7) == 0) {
    double* o = B.part + (size_t)sub * 36 + ((lane & 16) ? 18 : 0) + ((lane & 8) ? 9 : 0);
#pragma unroll
    for (int i = 0; i < 9; ++i) o[i] = (double)v[i];
  }
}

// ---- assemble S and g (ba.rs:293-331) ----------------------------------------

// Destination blocks with more than kFoldMin sub-segments (the lens block of
// a model gets a pair from every point) are summed first by a CTA each: warp
// w takes entries w, w + 8, ...; lane l adds sub-segments l, l + 32, ... in
// order, then a fixed butterfly; the total replaces the block's first
// partial, and assemble_kernel reads that one alone (sub_end[s] = first + 1).
constexpr uint32_t kFoldMin = 64;
constexpr int kFoldThreads = 256;

static __global__ void __launch_bounds__(kFoldThreads)
    schur_fold_kernel(Prob P, StructView S, double* part, const uint32_t* fold_slots,
                      const int32_t* active) {
  const uint32_t s = fold_slots[blockIdx.x];
  if (!active[P.blk_model[S.slot_row[s]]]) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t u0 = S.slot_sub_ptr[s], u1 = S.slot_sub_ptr[s + 1];
  double tot[5];
  int n = 0;
  for (int el = warp; el < 36; el += kFoldThreads / 32, ++n) {
    double v = 0.0;
    for (uint32_t u = u0 + lane; u < u1; u += 32) v += part[(size_t)u * 36 + el];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    tot[n] = v;
  }
  __syncthreads();  // every partial read before the first is replaced
  n = 0;
  for (int el = warp; el < 36; el += kFoldThreads / 32, ++n)
    if (lane == 0) part[(size_t)u0 * 36 + el] = tot[n];
}

template <typename R>
__global__ void assemble_kernel(Prob P, StateView st, StructView S, IterBufs<R> B,
                                const int32_t* active, const double* lambda, double* S64,
                                const uint32_t* sub_end) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.ns * 36) return;
  const int64_t s = t / 36;
  const int el = (int)(t % 36), r = el / 6, c = el % 6;
  const uint32_t a = S.slot_row[s], bcol = S.slot_col[s];
  const uint32_t m = P.blk_model[a];
  if (!active[m]) return;
  // Sub-segment sums in FP64 in both forms, in sub-segment order (a folded
  // block: its one folded total).
  double sum = 0.0;
  const uint32_t u1 = sub_end ? sub_end[s] : S.slot_sub_ptr[s + 1];
  const double* pp = B.part + el;
  uint32_t u = S.slot_sub_ptr[s];
  for (; u + 8 <= u1; u += 8) {
    double v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = pp[(size_t)(u + q) * 36];
#pragma unroll
    for (int q = 0; q < 8; ++q) sum += v[q];
  }
  for (; u < u1; ++u) sum += pp[(size_t)u * 36];
  double val;
  const bool lens_a = P.blk_is_lens[a] != 0;
  if (a == bcol) {
    const double lam = lambda[m];
    double u = 0.0;
    const uint32_t id = P.blk_id[a];
    const int i0 = r < c ? r : c, i1 = r < c ? c : r;
    if (!lens_a) {
      const int idx = i0 * 6 - (i0 * (i0 - 1)) / 2 + (i1 - i0);
      u = B.camU[21 * (size_t)id + idx];
      if (r == c && r >= 3 && P.prior_mask && P.prior_mask[id]) {
        const double sd = P.prior[6 * (size_t)id + r];
        u += 1.0 / (sd * sd);  // ba.rs:297-302
      }
      if (r == c) u = u * (1.0 + lam) + 1e-9;  // ba.rs:306-309
    } else {
      if (i1 < 3) u = B.grpU[6 * (size_t)id + (i0 * 3 - (i0 * (i0 - 1)) / 2 + (i1 - i0))];
      if (r == c) u = u * (1.0 + lam) + 1e-9;
      if (r == c && r >= 3) u = 1.0;  // ba.rs:310-314
      if (!P.model_refine[m]) u = (r == c) ? 1.0 : 0.0;  // ba.rs:315-317
    }
    val = u - (double)sum;
  } else {
    double x = 0.0;
    if (!lens_a && P.blk_is_lens[bcol] && c < 3) {
      const uint32_t cam = P.blk_id[a];
      if (P.grp_blk[P.cam_group[cam]] == bcol) x = B.camX[18 * (size_t)cam + 3 * r + c];
    }
    val = x - (double)sum;
  }
  const uint32_t pab = S.slot_pos_ab[s], pba = S.slot_pos_ba[s];
  if (pab < S.nz) B.S[(size_t)pab * 36 + 6 * r + c] = (R)val;
  if (a != bcol && pba < S.nz) B.S[(size_t)pba * 36 + 6 * c + r] = (R)val;
  // Mixed form with the two-level PCG: S before its rounding to FP32, for the
  // coarse matrix W^T S W (the gauge motions nearly annihilate S, and FP32
  // rounding of S is as large as what is left).
  if (S64) {
    if (pab < S.nz) S64[(size_t)pab * 36 + 6 * r + c] = val;
    if (a != bcol && pba < S.nz) S64[(size_t)pba * 36 + 6 * c + r] = val;
  }
}

template <typename R>
__global__ void rhs_kernel(Prob P, StateView st, IterBufs<R> B, const int32_t* active) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P.nb * 6) return;
  const int64_t b = t / 6;
  const int i = (int)(t % 6);
  const uint32_t m = P.blk_model[b];
  if (!active[m]) return;
  const uint32_t id = P.blk_id[b];
  double gv;
  if (!P.blk_is_lens[b]) {
    gv = B.camgj[6 * (size_t)id + i];
    if (i >= 3 && P.prior_mask && P.prior_mask[id]) {
      const double sd = P.prior[6 * (size_t)id + i];
      gv += (1.0 / (sd * sd)) * (P.prior[6 * (size_t)id + i - 3] - st.center[3 * (size_t)id + i - 3]);
    }
    gv -= B.camgs[6 * (size_t)id + i];
  } else {
    gv = i < 3 ? B.grpg[3 * (size_t)id + i] : 0.0;
  }
  B.g[6 * b + i] = (R)gv;
}

template <typename R>
__global__ void precond_kernel(Prob P, StructView S, IterBufs<R> B, const int32_t* active) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= P.nb) return;
  if (!active[P.blk_model[b]]) return;
  double A[36], Ai[36];
  const R* d = B.S + (size_t)S.diag_pos[b] * 36;
#pragma unroll
  for (int i = 0; i < 36; ++i) A[i] = (double)d[i];
  if (!inv6(A, Ai)) {  // ba.rs:159-160
#pragma unroll
    for (int i = 0; i < 36; ++i) Ai[i] = (i % 7 == 0) ? 1.0 : 0.0;
  }
  R* o = B.pre + 36 * (size_t)b;
#pragma unroll
  for (int i = 0; i < 36; ++i) o[i] = (R)Ai[i];
}

// ---- update (ba.rs:338-366) ---------------------------------------------------

template <typename R>
__global__ void update_cameras_kernel(Prob P, StateView cur, StateView trial, IterBufs<R> B,
                                      const int32_t* active) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < P.nc && active[P.cam_model[i]]) {
    const R* d = B.x + 6 * (size_t)P.cam_blk[i];
    const double w[3] = {(double)d[0], (double)d[1], (double)d[2]};
    double E[9];
    bacam::exp_so3(w, E);
    bacam::matmul3(E, cur.rot + 9 * i, trial.rot + 9 * i);
    for (int a = 0; a < 3; ++a) trial.center[3 * i + a] = cur.center[3 * i + a] + (double)d[3 + a];
  }
  if (i < P.ng) {
    const uint32_t b = P.grp_blk[i];
    const uint32_t m = P.blk_model[b];
    if (active[m]) {
      for (int a = 0; a < 5; ++a) trial.intr[5 * i + a] = cur.intr[5 * i + a];
      if (P.model_refine[m]) {
        const R* d = B.x + 6 * (size_t)b;
        trial.intr[5 * i + 0] += (double)d[0];
        trial.intr[5 * i + 3] += (double)d[1];
        trial.intr[5 * i + 4] += (double)d[2];
      }
    }
  }
}

// Mixed form, J^T J recomputed where it is used (the matrix-free PCG with
// nothing of size (observations x factor) stored, the Schur factors' other
// readers): observation k's factor Z_k = Y_k L_p, Y_k = w Jc^T Jp, from its
// stored FP32 record and its point's FP32 L (kept points), or from an FP64
// re-linearisation at the current state and the point's FP64 L (points with
// kept == 2).  The arithmetic of obs_factor_kernel and point_system_mixed_ill,
// so the values are those the factor passes store.
static __device__ __noinline__ void z_of_obs_ill(const Prob& P, const StateView& st,
                                                 const double* ptL, const double* sigma,
                                                 int64_t k, uint32_t p, float* z) {
  const uint32_t m = P.pt_model[p];
  double o[kLinW];
  if (!linearise<double>(P, st, k, sigma[m], P.model_refine[m] != 0, o)) {
#pragma unroll
    for (int i = 0; i < 18; ++i) z[i] = 0.0f;
    return;
  }
  const double* L = ptL + 6 * (size_t)p;
  const double w = o[26];
  const double j0 = o[12], j1 = o[13], j2 = o[14], j3 = o[15], j4 = o[16], j5 = o[17];
#pragma unroll
  for (int r = 0; r < 6; ++r) {
    const double ca = o[r], cb = o[6 + r];
    const double y0 = (ca * j0 + cb * j3) * w;
    const double y1 = (ca * j1 + cb * j4) * w;
    const double y2 = (ca * j2 + cb * j5) * w;
    z[3 * r + 0] = (float)(y0 * L[0] + y1 * L[1] + y2 * L[3]);
    z[3 * r + 1] = (float)(y1 * L[2] + y2 * L[4]);
    z[3 * r + 2] = (float)(y2 * L[5]);
  }
}

struct ZSource {
  Prob P;
  StateView st;         // the current state (ill-conditioned points)
  const float* lin;     // [no][kLinW] records
  const float* ptf;     // [np][9] FP32 L | t
  const double* ptL;    // [np][6] FP64 L
  const uint8_t* kept;  // [np]
  const double* sigma;  // [nm]
};

__device__ __forceinline__ void z_of_obs(const ZSource& Q, int64_t k, uint32_t p, float* z) {
  const uint32_t kp = Q.kept[p];
  if (kp == 2) {
    z_of_obs_ill(Q.P, Q.st, Q.ptL, Q.sigma, k, p, z);
    return;
  }
  const float* o = Q.lin + (size_t)k * kLinW;
  const float2 wv = *reinterpret_cast<const float2*>(o + 26);  // w, valid
  if (kp == 0 || wv.y == 0.0f) {
#pragma unroll
    for (int i = 0; i < 18; ++i) z[i] = 0.0f;
    return;
  }
  float j[20];
  const float4* o4 = reinterpret_cast<const float4*>(o);
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    const float4 q = o4[i];
    j[4 * i] = q.x, j[4 * i + 1] = q.y, j[4 * i + 2] = q.z, j[4 * i + 3] = q.w;
  }
  const float* pf = Q.ptf + 9 * (size_t)p;
  const float l00 = pf[0], l10 = pf[1], l11 = pf[2], l20 = pf[3], l21 = pf[4], l22 = pf[5];
  const float w = wv.x;
  const float j0 = j[12], j1 = j[13], j2 = j[14], j3 = j[15], j4 = j[16], j5 = j[17];
#pragma unroll
  for (int r = 0; r < 6; ++r) {
    const float ca = j[r], cb = j[6 + r];
    const float y0 = (ca * j0 + cb * j3) * w;
    const float y1 = (ca * j1 + cb * j4) * w;
    const float y2 = (ca * j2 + cb * j5) * w;
    z[3 * r + 0] = y0 * l00 + y1 * l10 + y2 * l20;
    z[3 * r + 1] = y1 * l11 + y2 * l21;
    z[3 * r + 2] = y2 * l22;
  }
}

// Mixed form, first pass of the back-substitution: a thread per observation
// of a kept, well-conditioned point forms u_k = Z_k^T dx of its camera (FP32,
// coalesced; the per-point pass then sums the point's u_k in order).
// kRecompute: the factors are not stored (B.Z null) but recomputed from zsrc.
template <bool kRecompute>
static __global__ void __launch_bounds__(256)
    obs_backsub_kernel(Prob P, IterBufs<float> B, float* obs_u, const int32_t* active,
                       ZSource zsrc) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P.no) return;
  const uint32_t p = P.obs_pt[k];
  if (!active[P.pt_model[p]] || B.kept[p] != 1) return;
  float z[18];
  if (kRecompute)
    z_of_obs(zsrc, k, p, z);
  else if (B.zpitch == 24)
    load_Z24(B.Z + z_index(B.zpos, k) * 24, z);
  else
    load_Z18(B.Z + z_index(B.zpos, k) * B.zpitch, z);
  const float* d = B.x + 6 * (size_t)P.cam_blk[P.obs_cam[k]];
  float u0 = 0.0f, u1 = 0.0f, u2 = 0.0f;
#pragma unroll
  for (int r = 0; r < 6; ++r) {
    const float dr = d[r];
    u0 += z[3 * r] * dr;
    u1 += z[3 * r + 1] * dr;
    u2 += z[3 * r + 2] * dr;
  }
  float* u = obs_u + 3 * (size_t)k;
  u[0] = u0, u[1] = u1, u[2] = u2;
}

template <typename R>
__global__ void backsub_kernel(Prob P, StructView S, StateView cur, StateView trial,
                               IterBufs<R> B, const double* sigma, const int32_t* active,
                               const float* obs_u) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= P.np) return;
  const int64_t p = S.pt_order ? S.pt_order[tid] : tid;
  const uint32_t m = P.pt_model[p];
  if (!active[m]) return;
  const double* X = cur.points + 3 * p;
  double* Xt = trial.points + 3 * p;
  const uint8_t kept = B.kept[p];
  if (!kept) {
    Xt[0] = X[0], Xt[1] = X[1], Xt[2] = X[2];
    return;
  }
  const uint32_t s = S.pt_ptr[p], e = S.pt_ptr[p + 1];
  const double* L = B.ptL + 6 * p;
  double a0, a1, a2;
  if (sizeof(R) == 4 && kept == 2) {
    // Mixed form, ill-conditioned point: u = sum_k Y_k^T dx from an FP64
    // re-linearisation, then a = zv - L^T u.
    const bool refine = P.model_refine[m] != 0;
    double u0 = 0.0, u1 = 0.0, u2 = 0.0;
    for (uint32_t k = s; k < e; ++k) {
      double o[kLinW];
      if (!linearise<double>(P, cur, k, sigma[m], refine, o)) continue;
      const R* d = B.x + 6 * (size_t)P.cam_blk[P.obs_cam[k]];
      double jd0 = 0.0, jd1 = 0.0;
#pragma unroll
      for (int r = 0; r < 6; ++r) jd0 += o[r] * (double)d[r], jd1 += o[6 + r] * (double)d[r];
      if (refine) {
        const R* dg = B.x + 6 * (size_t)P.grp_blk[P.cam_group[P.obs_cam[k]]];
#pragma unroll
        for (int r = 0; r < 3; ++r) jd0 += o[18 + r] * (double)dg[r], jd1 += o[21 + r] * (double)dg[r];
      }
      const double w = o[26];
      u0 += (o[12] * jd0 + o[15] * jd1) * w;
      u1 += (o[13] * jd0 + o[16] * jd1) * w;
      u2 += (o[14] * jd0 + o[17] * jd1) * w;
    }
    a0 = B.ptzv[3 * p] - (L[0] * u0 + L[1] * u1 + L[3] * u2);
    a1 = B.ptzv[3 * p + 1] - (L[2] * u1 + L[4] * u2);
    a2 = B.ptzv[3 * p + 2] - L[5] * u2;
  } else {
    R b0 = (R)B.ptzv[3 * p], b1 = (R)B.ptzv[3 * p + 1], b2 = (R)B.ptzv[3 * p + 2];
    if constexpr (sizeof(R) == 4) {  // u_k from obs_backsub_kernel
      for (uint32_t k = s; k < e; ++k) {
        const float* u = obs_u + 3 * (size_t)k;
        b0 -= u[0];
        b1 -= u[1];
        b2 -= u[2];
      }
    } else {
      for (uint32_t k = s; k < e; ++k) {
        const R* Z = B.Z + (size_t)k * 18;
        const R* d = B.x + 6 * (size_t)P.cam_blk[P.obs_cam[k]];
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          const R dr = d[r];
          b0 -= Z[3 * r] * dr;
          b1 -= Z[3 * r + 1] * dr;
          b2 -= Z[3 * r + 2] * dr;
        }
      }
    }
    for (uint32_t j = S.lens_ptr[p]; j < S.lens_ptr[p + 1]; ++j) {
      const R* Z = B.Zl + (size_t)j * 9;
      const R* d = B.x + 6 * (size_t)P.grp_blk[S.lens_grp[j]];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const R dr = d[r];
        b0 -= Z[3 * r] * dr;
        b1 -= Z[3 * r + 1] * dr;
        b2 -= Z[3 * r + 2] * dr;
      }
    }
    a0 = (double)b0, a1 = (double)b1, a2 = (double)b2;
  }
  Xt[0] = X[0] + L[0] * a0;
  Xt[1] = X[1] + (L[1] * a0 + L[2] * a1);
  Xt[2] = X[2] + (L[3] * a0 + L[4] * a1 + L[5] * a2);
}

}  // namespace ba
