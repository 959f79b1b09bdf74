// Adjoint (vector-Jacobian products) of the reprojection + distortion
// residuals and the GPS-prior residuals, plus the per-observation Jacobians
// and the robust cost at a context's current state.
//
// Residuals (ba.rs:56-128):
//   e_k = u_k − π(K_g, R_c (X_p − C_c))           per observation in front
//   r_c = (C_c − prior_c) / σ_c  (per axis)       per camera with a prior
// Jacobians J = ∂π/∂θ are the reference's (ba.rs:79-98): left rotation
// perturbation R ← exp(ω) R, then the centre, the point and the intrinsics
// (f, cx, cy, k1, k2; the reference refines f, k1, k2).  The VJP returns
//   g_θ = Σ_k (∂e_k/∂θ)ᵀ λ_k + Σ_c (∂r_c/∂θ)ᵀ μ_c,   ∂e/∂θ = −J.
// The gradient of the robust cost is the VJP with λ_k = ρ'(|e_k|²)·2e_k and
// μ_c = 2 r_c.
#include <cstring>
#include <vector>

#include "context.cuh"
#include "lm_kernels.cuh"

namespace ba {
namespace {

constexpr unsigned T = 256;

// Per observation: pred Jacobians in FP64 (rows u, v): jc 2x6, jp 2x3,
// ji 2x5 (f, cx, cy, k1, k2), residual e, weight w; false if behind.
__device__ bool full_jacobian(const Prob& P, const StateView& st, int64_t k, double sigma,
                              double* jc, double* jp, double* ji, double* e, double* w) {
  double o[kLinW];
  if (!linearise<double>(P, st, k, sigma, true, o)) return false;
  for (int i = 0; i < 12; ++i) jc[i] = o[i];
  for (int i = 0; i < 6; ++i) jp[i] = o[12 + i];
  // intrinsics: (f, cx, cy, k1, k2); linearise gives d/d(f, k1, k2)
  ji[0] = o[18], ji[1] = 1.0, ji[2] = 0.0, ji[3] = o[19], ji[4] = o[20];
  ji[5] = o[21], ji[6] = 0.0, ji[7] = 1.0, ji[8] = o[22], ji[9] = o[23];
  e[0] = o[24], e[1] = o[25];
  *w = o[26];
  return true;
}

__global__ void linearise_all_kernel(Prob P, StateView st, double sigma, double* out,
                                     const uint8_t* refine_model) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P.no) return;
  double* o = out + (size_t)k * kLinW;
  const bool refine = refine_model[P.pt_model[P.obs_pt[k]]] != 0;
  if (!linearise<double>(P, st, k, sigma, refine, o))
    for (int i = 0; i < kLinW; ++i) o[i] = 0.0;
}

// Per observation VJP contributions: camera (6), point (3), intrinsics (5).
// cot: caller's residual cotangents [2n], or null for the cost gradient.
__global__ void vjp_obs_kernel(Prob P, StateView st, double sigma, const double* cot,
                               double* gcam, double* gpt, double* gint) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P.no) return;
  double jc[12], jp[6], ji[10], e[2], w;
  double* c6 = gcam + 6 * (size_t)k;
  double* p3 = gpt + 3 * (size_t)k;
  double* i5 = gint + 5 * (size_t)k;
  if (!full_jacobian(P, st, k, sigma, jc, jp, ji, e, &w)) {
    for (int i = 0; i < 6; ++i) c6[i] = 0.0;
    for (int i = 0; i < 3; ++i) p3[i] = 0.0;
    for (int i = 0; i < 5; ++i) i5[i] = 0.0;
    return;
  }
  double l0, l1;
  if (cot) {
    l0 = cot[2 * k], l1 = cot[2 * k + 1];
  } else {  // d rho / d e = rho'(|e|^2) * 2 e, rho' = the IRLS weight
    l0 = 2.0 * w * e[0], l1 = 2.0 * w * e[1];
  }
  for (int i = 0; i < 6; ++i) c6[i] = -(jc[i] * l0 + jc[6 + i] * l1);
  for (int i = 0; i < 3; ++i) p3[i] = -(jp[i] * l0 + jp[3 + i] * l1);
  for (int i = 0; i < 5; ++i) i5[i] = -(ji[i] * l0 + ji[5 + i] * l1);
}

// Thread per point: its observations' contributions in order.
__global__ void vjp_point_kernel(Prob P, const uint32_t* pt_ptr, const double* gpt, double* out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.np) return;
  double a[3] = {0, 0, 0};
  for (uint32_t k = pt_ptr[p]; k < pt_ptr[p + 1]; ++k)
    for (int i = 0; i < 3; ++i) a[i] += gpt[3 * (size_t)k + i];
  for (int i = 0; i < 3; ++i) out[3 * p + i] = a[i];
}

// CTA per camera: observations in camera order, plus the prior term.
__global__ void __launch_bounds__(128)
    vjp_camera_kernel(Prob P, StateView st, const uint32_t* cam_ptr, const uint32_t* cam_obs,
                      const double* gcam, const double* gint, const double* cot_prior,
                      double* out_cam, double* out_cam_int) {
  __shared__ double scratch[11 * 32];
  const int64_t c = blockIdx.x;
  double a[11];
  for (int i = 0; i < 11; ++i) a[i] = 0.0;
  for (uint32_t i = cam_ptr[c] + threadIdx.x; i < cam_ptr[c + 1]; i += blockDim.x) {
    const uint32_t k = cam_obs[i];
    for (int t = 0; t < 6; ++t) a[t] += gcam[6 * (size_t)k + t];
    for (int t = 0; t < 5; ++t) a[6 + t] += gint[5 * (size_t)k + t];
  }
  block_sum<11>(a, scratch);
  if (threadIdx.x == 0) {
    if (P.prior_mask && P.prior_mask[c]) {
      const double* q = P.prior + 6 * (size_t)c;
      for (int t = 0; t < 3; ++t) {
        const double r = (st.center[3 * c + t] - q[t]) / q[3 + t];
        const double mu = cot_prior ? cot_prior[3 * c + t] : 2.0 * r;
        a[3 + t] += mu / q[3 + t];
      }
    }
    for (int t = 0; t < 6; ++t) out_cam[6 * c + t] = a[t];
    for (int t = 0; t < 5; ++t) out_cam_int[5 * c + t] = a[6 + t];
  }
}

__global__ void vjp_group_kernel(Prob P, const uint32_t* grp_ptr, const uint32_t* grp_cams,
                                 const double* cam_int, double* out) {
  const int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (g >= P.ng) return;
  double a[5] = {0, 0, 0, 0, 0};
  for (uint32_t i = grp_ptr[g] + lane; i < grp_ptr[g + 1]; i += 32)
    for (int t = 0; t < 5; ++t) a[t] += cam_int[5 * (size_t)grp_cams[i] + t];
  for (int t = 0; t < 5; ++t) a[t] = warp_sum(a[t]);
  if (lane == 0)
    for (int t = 0; t < 5; ++t) out[5 * g + t] = a[t];
}

void require(const Context& c) {
  if (!c.uploaded) throw BadInput("no problem uploaded");
  check(cudaSetDevice(c.device), "cudaSetDevice");
}

// Cost chunks aligned to model boundaries (the solver's cost plan).
struct CostPlan {
  DevBuf<uint32_t> model, begin, end, m0;
  int64_t n = 0;
  StructView view() const {
    StructView v{};
    v.cost_chunk_model = model;
    v.cost_chunk_begin = begin;
    v.cost_chunk_end = end;
    v.model_chunk0 = m0;
    v.ncost = n;
    return v;
  }
};

void make_cost_plan(const Context& c, CostPlan& pl) {
  constexpr uint32_t CH = 4096;
  std::vector<uint32_t> cm, cb, ce, m0(c.nm + 1);
  for (int64_t m = 0; m < c.nm; ++m) {
    m0[m] = (uint32_t)cm.size();
    uint32_t x = c.h_obs0[m];
    const uint32_t e = c.h_obs0[m + 1];
    do {
      cm.push_back((uint32_t)m), cb.push_back(x), ce.push_back(std::min(e, x + CH));
      x += CH;
    } while (x < e);
  }
  m0[c.nm] = (uint32_t)cm.size();
  pl.n = (int64_t)cm.size();
  cudaStream_t s = c.stream;
  pl.model.alloc(pl.n, s), pl.begin.alloc(pl.n, s), pl.end.alloc(pl.n, s), pl.m0.alloc(c.nm + 1, s);
  check(cudaMemcpyAsync(pl.model, cm.data(), 4 * cm.size(), cudaMemcpyHostToDevice, s), "h2d");
  check(cudaMemcpyAsync(pl.begin, cb.data(), 4 * cb.size(), cudaMemcpyHostToDevice, s), "h2d");
  check(cudaMemcpyAsync(pl.end, ce.data(), 4 * ce.size(), cudaMemcpyHostToDevice, s), "h2d");
  check(cudaMemcpyAsync(pl.m0, m0.data(), 4 * m0.size(), cudaMemcpyHostToDevice, s), "h2d");
  check(cudaStreamSynchronize(s), "cost plan");
}

void context_cost(Context& c, const ba_options* opt, double* cost, double* rms, int64_t* nf) {
  require(c);
  const Opts o = resolve_options(opt);
  cudaStream_t s = c.stream;
  const Prob P = c.prob(o.loss);
  CostPlan pl;
  make_cost_plan(c, pl);
  const StructView SV = pl.view();
  DevBuf<double> part(std::max<int64_t>(pl.n, 1) * 3, s), sg(c.nm, s), dc(c.nm, s), dsq(c.nm, s);
  DevBuf<int64_t> dn(c.nm, s);
  std::vector<double> h_sg(c.nm, o.sigma);
  check(cudaMemcpyAsync(sg.p, h_sg.data(), 8 * c.nm, cudaMemcpyHostToDevice, s), "h2d");
  BA_LAUNCH(cost_chunk_kernel<<<(unsigned)std::max<int64_t>(pl.n, 1), kCostThreads, 0, s>>>(
      P, c.cur(), SV, part, nullptr, sg));
  BA_LAUNCH(cost_final_kernel<<<(unsigned)c.nm, kCostFinalThreads, 0, s>>>(P, c.cur(), SV, part,
                                                                      nullptr, dc, dsq, dn));
  std::vector<double> hc(c.nm), hsq(c.nm);
  std::vector<int64_t> hn(c.nm);
  check(cudaMemcpyAsync(hc.data(), dc.p, 8 * c.nm, cudaMemcpyDeviceToHost, s), "d2h");
  check(cudaMemcpyAsync(hsq.data(), dsq.p, 8 * c.nm, cudaMemcpyDeviceToHost, s), "d2h");
  check(cudaMemcpyAsync(hn.data(), dn.p, 8 * c.nm, cudaMemcpyDeviceToHost, s), "d2h");
  check(cudaStreamSynchronize(s), "cost");
  for (int64_t m = 0; m < c.nm; ++m) {
    if (cost) cost[m] = hc[m];
    if (rms) rms[m] = std::sqrt(hsq[m] / (double)std::max<int64_t>(hn[m], 1));
    if (nf) nf[m] = hn[m];
  }
}

void context_linearise(Context& c, const ba_options* opt, double* e, double* jc, double* jg,
                       double* jp, double* w, uint8_t* valid) {
  require(c);
  const Opts o = resolve_options(opt);
  cudaStream_t s = c.stream;
  const int64_t no = c.no;
  if (no == 0) return;
  DevBuf<double> out(no * kLinW, s);
  BA_LAUNCH(linearise_all_kernel<<<grid_for(no, T), T, 0, s>>>(c.prob(o.loss), c.cur(), o.sigma,
                                                              out, c.model_refine));
  std::vector<double> h(no * kLinW);
  check(cudaMemcpyAsync(h.data(), out.p, 8 * h.size(), cudaMemcpyDeviceToHost, s), "d2h");
  check(cudaStreamSynchronize(s), "linearise");
  for (int64_t k = 0; k < no; ++k) {
    const double* r = h.data() + k * kLinW;
    if (e) std::memcpy(e + 2 * k, r + 24, 16);
    if (jc) std::memcpy(jc + 12 * k, r, 96);
    if (jp) std::memcpy(jp + 6 * k, r + 12, 48);
    if (jg) std::memcpy(jg + 6 * k, r + 18, 48);
    if (w) w[k] = r[26];
    if (valid) valid[k] = r[27] != 0.0 ? 1 : 0;
  }
}

void context_vjp(Context& c, const ba_options* opt, const double* cot_obs,
                 const double* cot_prior, double* g_cam, double* g_pt, double* g_intr) {
  require(c);
  const Opts o = resolve_options(opt);
  cudaStream_t s = c.stream;
  const Prob P = c.prob(o.loss);
  const int64_t no = c.no, nc = c.nc, np = c.np, ng = c.ng;
  StructBufs SB;
  SB.pt_ptr.alloc(np + 1, s);
  lower_bounds_u32(P.obs_pt, no, SB.pt_ptr, np, s);
  build_cam_index(P, SB, s);
  DevBuf<double> d_cot(cot_obs ? 2 * no : 0, s), d_cotp(cot_prior ? 3 * nc : 0, s);
  if (cot_obs && no)
    check(cudaMemcpyAsync(d_cot.p, cot_obs, 16 * no, cudaMemcpyHostToDevice, s), "h2d");
  if (cot_prior && nc)
    check(cudaMemcpyAsync(d_cotp.p, cot_prior, 24 * nc, cudaMemcpyHostToDevice, s), "h2d");
  DevBuf<double> gc(std::max<int64_t>(no, 1) * 6, s), gp(std::max<int64_t>(no, 1) * 3, s),
      gi(std::max<int64_t>(no, 1) * 5, s);
  DevBuf<double> oc(std::max<int64_t>(nc, 1) * 6, s), oci(std::max<int64_t>(nc, 1) * 5, s),
      op(std::max<int64_t>(np, 1) * 3, s), og(std::max<int64_t>(ng, 1) * 5, s);
  if (no)
    BA_LAUNCH(vjp_obs_kernel<<<grid_for(no, T), T, 0, s>>>(P, c.cur(), o.sigma,
                                                          cot_obs ? d_cot.p : nullptr, gc, gp, gi));
  if (np) BA_LAUNCH(vjp_point_kernel<<<grid_for(np, T), T, 0, s>>>(P, SB.pt_ptr, gp, op));
  if (nc)
    BA_LAUNCH(vjp_camera_kernel<<<(unsigned)nc, 128, 0, s>>>(
        P, c.cur(), SB.cam_ptr, SB.cam_obs, gc, gi, cot_prior ? d_cotp.p : nullptr, oc, oci));
  if (ng)
    BA_LAUNCH(vjp_group_kernel<<<grid_for(ng * 32, 128), 128, 0, s>>>(P, SB.grp_ptr, SB.grp_cams,
                                                                     oci, og));
  if (g_cam && nc) check(cudaMemcpyAsync(g_cam, oc.p, 48 * nc, cudaMemcpyDeviceToHost, s), "d2h");
  if (g_pt && np) check(cudaMemcpyAsync(g_pt, op.p, 24 * np, cudaMemcpyDeviceToHost, s), "d2h");
  if (g_intr && ng) check(cudaMemcpyAsync(g_intr, og.p, 40 * ng, cudaMemcpyDeviceToHost, s), "d2h");
  check(cudaStreamSynchronize(s), "vjp");
}

}  // namespace
}  // namespace ba

using namespace ba;

extern "C" {

ba_status ba_context_cost(ba_context* c, const ba_options* opt, double* cost, double* rms,
                          int64_t* n_in_front) {
  if (!c) return set_error(BA_BAD_INPUT, "null context");
  return guarded([&] { context_cost(*c, opt, cost, rms, n_in_front); });
}

ba_status ba_context_linearise(ba_context* c, const ba_options* opt, double* e, double* jc,
                               double* jg, double* jp, double* w, uint8_t* valid) {
  if (!c) return set_error(BA_BAD_INPUT, "null context");
  return guarded([&] { context_linearise(*c, opt, e, jc, jg, jp, w, valid); });
}

ba_status ba_context_vjp(ba_context* c, const ba_options* opt, const double* cot_obs,
                         const double* cot_prior, double* g_cam, double* g_points,
                         double* g_intr) {
  if (!c) return set_error(BA_BAD_INPUT, "null context");
  return guarded([&] { context_vjp(*c, opt, cot_obs, cot_prior, g_cam, g_points, g_intr); });
}

ba_status ba_context_intrinsics_grad(ba_context* c, const ba_options* opt, double* grad) {
  if (!c) return set_error(BA_BAD_INPUT, "null context");
  if (!grad) return set_error(BA_BAD_INPUT, "null gradient array");
  return guarded([&] { context_vjp(*c, opt, nullptr, nullptr, nullptr, nullptr, grad); });
}

}  // extern "C"
