// C ABI of the solver (include/ba_gb300.h): contexts, upload / download,
// option handling, error reporting.
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "ba_gb300.h"
#include "context.cuh"
#include "structure.cuh"

namespace ba {

thread_local std::string g_last_error;

namespace {

double now_ms() {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

__device__ __forceinline__ uint32_t model_of(const uint32_t* r0, int64_t nm, uint64_t i) {
  int64_t lo = 0, hi = nm;  // last m with r0[m] <= i
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (r0[mid] <= i)
      lo = mid;
    else
      hi = mid;
  }
  return (uint32_t)lo;
}

// Offsets of concatenated models and the derived per-element tables.
__global__ void fixup_kernel(int64_t nm, const uint32_t* obs0, const uint32_t* cam0,
                             const uint32_t* pt0, const uint32_t* grp0, const uint32_t* blk0,
                             int64_t no, int64_t nc, int64_t np, int64_t ng, uint32_t* obs_cam,
                             uint32_t* obs_pt, uint32_t* cam_group, uint32_t* cam_model,
                             uint32_t* pt_model, uint32_t* grp_model, uint32_t* cam_blk,
                             uint32_t* grp_blk, uint32_t* blk_model, uint32_t* blk_id,
                             uint8_t* blk_is_lens) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < no) {
    const uint32_t m = model_of(obs0, nm, i);
    obs_cam[i] += cam0[m];
    obs_pt[i] += pt0[m];
  }
  if (i < nc) {
    const uint32_t m = model_of(cam0, nm, i);
    cam_group[i] += grp0[m];
    cam_model[i] = m;
    const uint32_t b = blk0[m] + (uint32_t)(i - cam0[m]);
    cam_blk[i] = b;
    blk_model[b] = m;
    blk_id[b] = (uint32_t)i;
    blk_is_lens[b] = 0;
  }
  if (i < np) pt_model[i] = model_of(pt0, nm, i);
  if (i < ng) {
    const uint32_t m = model_of(grp0, nm, i);
    grp_model[i] = m;
    const uint32_t b = blk0[m] + (cam0[m + 1] - cam0[m]) + (uint32_t)(i - grp0[m]);
    grp_blk[i] = b;
    blk_model[b] = m;
    blk_id[b] = (uint32_t)i;
    blk_is_lens[b] = 1;
  }
}

template <typename T>
void up(DevBuf<T>& d, const T* h, size_t off, size_t n, cudaStream_t s) {
  if (n) check(cudaMemcpyAsync(d.p + off, h, n * sizeof(T), cudaMemcpyDefault, s), "h2d");
}

}  // namespace

// Copies into the context: host or device source arrays (unified addressing).
void upload(Context& c, const ba_problem* P, const ba_state* S, int32_t n) {
  if (n < 1) throw BadInput("n_models must be >= 1");
  if (!P || !S) throw BadInput("null problem or state");
  std::vector<uint32_t> obs0{0}, cam0{0}, pt0{0}, grp0{0}, blk0{0};
  std::vector<uint8_t> refine;
  bool prior = false;
  for (int m = 0; m < n; ++m) {
    const ba_problem& p = P[m];
    if (p.n_cams < 0 || p.n_points < 0 || p.n_obs < 0 || p.n_groups < 0)
      throw BadInput("negative size in model " + std::to_string(m));
    if (p.n_cams > 0 && p.n_groups < 1)
      throw BadInput("model " + std::to_string(m) + " has cameras but no lens group");
    if (p.n_obs > 0 && (!p.obs_cam || !p.obs_pt || !p.obs_uv))
      throw BadInput("null observation array in model " + std::to_string(m));
    if (p.n_cams > 0 && !p.cam_group)
      throw BadInput("null cam_group in model " + std::to_string(m));
    if (p.prior_mask && !p.prior) throw BadInput("prior_mask without prior");
    const ba_state& st = S[m];
    if ((p.n_cams > 0 && (!st.rot || !st.center)) || (p.n_groups > 0 && !st.intr) ||
        (p.n_points > 0 && !st.points))
      throw BadInput("null state array in model " + std::to_string(m));
    prior = prior || (p.prior_mask != nullptr);
    const uint64_t lim = 0xfffffff0ULL;
    if ((uint64_t)obs0.back() + p.n_obs > lim || (uint64_t)pt0.back() + p.n_points > lim ||
        (uint64_t)cam0.back() + p.n_cams > (1ULL << 26) ||
        (uint64_t)grp0.back() + p.n_groups > (1ULL << 26))
      throw BadInput("batch too large for 32-bit indexing");
    obs0.push_back(obs0.back() + (uint32_t)p.n_obs);
    cam0.push_back(cam0.back() + (uint32_t)p.n_cams);
    pt0.push_back(pt0.back() + (uint32_t)p.n_points);
    grp0.push_back(grp0.back() + (uint32_t)p.n_groups);
    blk0.push_back(blk0.back() + (uint32_t)(p.n_cams + p.n_groups));
    refine.push_back(p.refine_intrinsics ? 1 : 0);
  }
  cudaStream_t s = c.stream;
  c.nm = n;
  c.no = obs0.back(), c.nc = cam0.back(), c.np = pt0.back(), c.ng = grp0.back();
  c.nb = blk0.back();
  c.has_prior = prior;
  c.h_obs0 = obs0, c.h_cam0 = cam0, c.h_pt0 = pt0, c.h_grp0 = grp0, c.h_blk0 = blk0;
  c.h_refine = refine;
  const size_t no = c.no, nc = c.nc, np = c.np, ng = c.ng, nb = c.nb;
  auto A = [&](auto& d, size_t cnt) { d.alloc(std::max<size_t>(cnt, 1), s); };
  A(c.obs_cam, no), A(c.obs_pt, no), A(c.obs_uv, 2 * no), A(c.cam_group, nc);
  A(c.prior, 6 * nc), A(c.prior_mask, nc);
  A(c.cam_model, nc), A(c.pt_model, np), A(c.grp_model, ng), A(c.cam_blk, nc), A(c.grp_blk, ng);
  A(c.blk_model, nb), A(c.blk_id, nb), A(c.blk_is_lens, nb);
  A(c.init_rot, 9 * nc), A(c.init_center, 3 * nc), A(c.init_intr, 5 * ng), A(c.init_points, 3 * np);
  A(c.rot, 9 * nc), A(c.center, 3 * nc), A(c.intr, 5 * ng), A(c.points, 3 * np);
  A(c.trot, 9 * nc), A(c.tcenter, 3 * nc), A(c.tintr, 5 * ng), A(c.tpoints, 3 * np);
  if (prior) c.prior_mask.zero();
  const double t0 = now_ms();
  int64_t bytes = 0;
  for (int m = 0; m < n; ++m) {
    const ba_problem& p = P[m];
    const ba_state& st = S[m];
    up(c.obs_cam, p.obs_cam, obs0[m], p.n_obs, s);
    up(c.obs_pt, p.obs_pt, obs0[m], p.n_obs, s);
    up(c.obs_uv, p.obs_uv, 2 * (size_t)obs0[m], 2 * p.n_obs, s);
    up(c.cam_group, p.cam_group, cam0[m], p.n_cams, s);
    if (p.prior_mask) {
      up(c.prior_mask, p.prior_mask, cam0[m], p.n_cams, s);
      up(c.prior, p.prior, 6 * (size_t)cam0[m], 6 * p.n_cams, s);
    }
    up(c.init_rot, st.rot, 9 * (size_t)cam0[m], 9 * p.n_cams, s);
    up(c.init_center, st.center, 3 * (size_t)cam0[m], 3 * p.n_cams, s);
    up(c.init_intr, st.intr, 5 * (size_t)grp0[m], 5 * p.n_groups, s);
    up(c.init_points, st.points, 3 * (size_t)pt0[m], 3 * p.n_points, s);
    bytes += p.n_obs * (4 + 4 + 16) + p.n_cams * (4 + 72 + 24) + p.n_groups * 40 +
             p.n_points * 24 + (p.prior_mask ? p.n_cams * 49 : 0);
  }
  DevBuf<uint32_t> d_obs0, d_cam0, d_pt0, d_grp0, d_blk0;
  A(d_obs0, n + 1), A(d_cam0, n + 1), A(d_pt0, n + 1), A(d_grp0, n + 1);
  A(c.model_obs0, n + 1), A(c.model_cam0, n + 1), A(c.model_blk0, n + 1), A(c.model_refine, n);
  up(c.model_obs0, obs0.data(), 0, n + 1, s);
  up(c.model_cam0, cam0.data(), 0, n + 1, s);
  up(c.model_blk0, blk0.data(), 0, n + 1, s);
  up(d_pt0, pt0.data(), 0, n + 1, s);
  up(d_grp0, grp0.data(), 0, n + 1, s);
  up(c.model_refine, refine.data(), 0, n, s);
  const size_t mx = std::max(std::max(no, nc), std::max(np, ng));
  if (mx > 0)
    BA_LAUNCH(fixup_kernel<<<grid_for(mx, 256), 256, 0, s>>>(
        n, c.model_obs0, c.model_cam0, d_pt0, d_grp0, c.model_blk0, no, nc, np, ng, c.obs_cam,
        c.obs_pt, c.cam_group, c.cam_model, c.pt_model, c.grp_model, c.cam_blk, c.grp_blk,
        c.blk_model, c.blk_id, c.blk_is_lens));
  check(cudaStreamSynchronize(s), "upload");
  c.last_h2d_ms = now_ms() - t0;
  c.last_h2d_bytes = bytes;
  // Validate indices, ordering and finiteness once (device).
  c.err.zero();
  validate_problem(c.prob(0), StateView{c.init_rot, c.init_center, c.init_intr, c.init_points},
                   c.grp_model, c.err, s);
  uint32_t e = 0;
  check(cudaMemcpyAsync(&e, c.err.p, 4, cudaMemcpyDeviceToHost, s), "d2h");
  check(cudaStreamSynchronize(s), "validate");
  c.uploaded = true;
  reset_states(c);
  check(cudaStreamSynchronize(s), "upload");
  if (e) {
    c.uploaded = false;
    std::string msg = "invalid problem:";
    if (e & ERR_BAD_INDEX) msg += " camera/point/group index out of range;";
    if (e & ERR_UNSORTED) msg += " observations are not sorted by point;";
    if (e & ERR_MODEL_MIX) msg += " an observation links different models;";
    if (e & ERR_NONFINITE)
      msg += " a measurement, prior or initial state value is not finite (or a prior sigma <= 0);";
    throw BadInput(msg);
  }
}

namespace {

void download(Context& c, ba_state* S, int32_t n) {
  if (!c.uploaded) throw BadInput("no problem uploaded");
  if (n != c.nm) throw BadInput("n_models does not match the uploaded batch");
  cudaStream_t s = c.stream;
  const double t0 = now_ms();
  int64_t bytes = 0;
  for (int m = 0; m < n; ++m) {
    const size_t c0 = c.h_cam0[m], nc = c.h_cam0[m + 1] - c0;
    const size_t g0 = c.h_grp0[m], ng = c.h_grp0[m + 1] - g0;
    const size_t p0 = c.h_pt0[m], np = c.h_pt0[m + 1] - p0;
    if (nc) {
      check(cudaMemcpyAsync(S[m].rot, c.rot.p + 9 * c0, 72 * nc, cudaMemcpyDeviceToHost, s), "d2h");
      check(cudaMemcpyAsync(S[m].center, c.center.p + 3 * c0, 24 * nc, cudaMemcpyDeviceToHost, s), "d2h");
    }
    if (ng) check(cudaMemcpyAsync(S[m].intr, c.intr.p + 5 * g0, 40 * ng, cudaMemcpyDeviceToHost, s), "d2h");
    if (np) check(cudaMemcpyAsync(S[m].points, c.points.p + 3 * p0, 24 * np, cudaMemcpyDeviceToHost, s), "d2h");
    bytes += 96 * nc + 40 * ng + 24 * np;
  }
  check(cudaStreamSynchronize(s), "download");
  c.last_d2h_ms = now_ms() - t0;
  c.last_d2h_bytes = bytes;
}

}  // namespace

Opts resolve_options(const ba_options* o) {
  Opts r;
  if (o) {
    r.max_iter = o->max_iter;
    r.sigma = o->sigma_px;
    r.loss = o->loss;
    r.precision = o->precision;
    r.pcg_max_iter = o->pcg_max_iter > 0 ? o->pcg_max_iter : 400;
    r.pcg_tol = o->pcg_tol > 0 ? o->pcg_tol : 1e-20;
    r.matrix_free = o->matrix_free;
    r.memory_cap = o->memory_cap_bytes;
    r.log = o->log;
    r.profile = o->profile;
    r.pcg_kernel = o->pcg_kernel;
    r.graph = o->no_graph ? 0 : 1;
    r.autotune = o->autotune;
    r.stop_patience = o->stop_patience;
    r.coarse = o->coarse;
    r.hold_cta = o->fault_hold_pcg_cta;
    if (o->wait_limit_cycles > 0) r.wait_limit = o->wait_limit_cycles;
    r.workspace_limit = o->workspace_limit_bytes > 0 ? o->workspace_limit_bytes : 0;
    r.pcg_end_max_iter = o->pcg_end_max_iter;
    if (o->pcg_end_rel > 0.0) r.pcg_end_rel = o->pcg_end_rel;
    r.point_kernel = o->point_kernel;
  }
  if (r.max_iter < 0) throw BadInput("max_iter must be >= 0");
  if (!(r.sigma > 0.0) || !std::isfinite(r.sigma)) throw BadInput("sigma_px must be finite and > 0");
  if (r.loss != 0 && r.loss != 1) throw BadInput("unknown loss");
  if (r.precision != 0 && r.precision != 1) throw BadInput("unknown precision");
  if (r.matrix_free < 0 || r.matrix_free > 3) throw BadInput("unknown matrix_free mode");
  if (r.pcg_kernel < 0 || r.pcg_kernel > 3) throw BadInput("unknown pcg_kernel");
  if (r.stop_patience < 0) throw BadInput("stop_patience must be >= 0");
  if (r.coarse != 0 && r.coarse != 1) throw BadInput("coarse must be 0 or 1");
  if (r.hold_cta < 0) throw BadInput("fault_hold_pcg_cta must be >= 0");
  if (r.pcg_end_max_iter < 0) throw BadInput("pcg_end_max_iter must be >= 0");
  if (r.point_kernel < 0 || r.point_kernel > 3) throw BadInput("unknown point_kernel");
  if (!std::isfinite(r.pcg_end_rel)) throw BadInput("pcg_end_rel must be finite");
  return r;
}

ba_status set_error(ba_status st, const std::string& msg) {
  g_last_error = msg;
  return st;
}

ba_status run_guarded(void (*fn)(void*), void* arg) {
  try {
    fn(arg);
    return BA_OK;
  } catch (const BadInput& e) {
    return set_error(BA_BAD_INPUT, e.what());
  } catch (const CudaError& e) {
    if (e.code == cudaErrorMemoryAllocation) return set_error(BA_OOM, e.what());
    if (e.code == cudaErrorNotSupported) return set_error(BA_NOT_SUPPORTED, e.what());
    if (e.code == cudaErrorLaunchTimeout) return set_error(BA_TIMEOUT, e.what());
    return set_error(BA_CUDA_ERROR, e.what());
  } catch (const std::bad_alloc&) {
    return set_error(BA_OOM, "host allocation failed");
  } catch (const std::exception& e) {
    return set_error(BA_CUDA_ERROR, e.what());
  }
}

namespace {

void init_context(Context& c, int device, void* stream) {
  int n = 0;
  check(cudaGetDeviceCount(&n), "no CUDA device");
  if (n < 1) throw CudaError(cudaErrorNoDevice, "no CUDA device");
  if (device < 0) check(cudaGetDevice(&device), "cudaGetDevice");
  check(cudaSetDevice(device), "cudaSetDevice");
  c.device = device;
  int major = 0;
  check(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device), "attr");
  check(cudaDeviceGetAttribute(&c.n_sm, cudaDevAttrMultiProcessorCount, device), "attr");
  int coop = 0;
  check(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device), "attr");
  if (!coop) throw CudaError(cudaErrorNotSupported, "device lacks cooperative launch");
  if (stream) {
    c.stream = (cudaStream_t)stream;
    c.own_stream = false;
  } else {
    check(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking), "stream");
    c.own_stream = true;
  }
  // Keep freed blocks in the stream-ordered pool for the next solve.
  cudaMemPool_t pool;
  check(cudaDeviceGetDefaultMemPool(&pool, device), "mempool");
  uint64_t thr = UINT64_MAX;
  check(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr), "mempool");
  c.err.alloc(1, c.stream);
  c.err.zero();
}

void destroy_context(Context& c) {
  cudaSetDevice(c.device);
  cudaStream_t s = c.stream;
  bool own = c.own_stream;
  c = Context();  // frees every buffer on the context's stream
  if (s) cudaStreamSynchronize(s);
  if (own && s) cudaStreamDestroy(s);
}

void solve(Context& c, const ba_options* opt, ba_stats* stats) {
  if (!c.uploaded) throw BadInput("no problem uploaded");
  const Opts o = resolve_options(opt);
  check(cudaSetDevice(c.device), "cudaSetDevice");
  DevBudgetScope budget(o.workspace_limit);
  const int64_t l0 = g_launches;
  dev_bytes_peak() = dev_bytes_live();
  const double t0 = now_ms();
  c.err.zero();
  if (o.precision == 0)
    run_lm<double>(c, o);
  else
    run_lm<float>(c, o);
  uint32_t e = 0;
  check(cudaMemcpyAsync(&e, c.err.p, 4, cudaMemcpyDeviceToHost, c.stream), "d2h");
  check(cudaStreamSynchronize(c.stream), "solve");
  if (e & ERR_BARRIER_TIMEOUT)
    throw CudaError(cudaErrorLaunchTimeout, "a device-side barrier gave up waiting");
  if (e)
    throw CudaError(cudaErrorAssert, "device check failed (error bits " + std::to_string(e) + ")");
  const double t1 = now_ms();
  if (stats) {
    for (int64_t m = 0; m < c.nm; ++m) {
      const ModelResult& r = c.results[m];
      ba_stats& st = stats[m];
      std::memset(&st, 0, sizeof st);
      st.iterations = r.iterations;
      st.initial_rms = r.initial_rms;
      st.final_rms = r.final_rms;
      st.initial_cost = r.initial_cost;
      st.final_cost = r.final_cost;
      st.pcg_iterations = r.pcg;
      st.kernel_launches = g_launches - l0;
      st.ms_total = t1 - t0;
      st.device_bytes = (int64_t)dev_bytes_peak();
      for (int k = 0; k < kPhases; ++k) st.ms_phase[k] = c.phase_ms[k], st.n_phase[k] = c.phase_n[k];
      st.n_blocks = c.nb, st.n_nonzero_blocks = c.last_nz, st.n_schur_pairs = c.last_pairs;
      st.n_lens_entries = c.last_nl;
      st.pcg_kernel = c.last_pcg_kernel;
      st.pcg_cluster = c.last_pcg_cluster;
      st.graph = c.last_graph ? 1 : 0;
      st.pcg_ctas = c.last_pcg_ctas;
      st.pcg_threads = c.last_pcg_threads;
      st.point_kernel = c.last_point_kernel;
      st.point_tuned_us = c.tuning[o.precision == BA_PRECISION_MIXED ? 1 : 0].valid
                              ? c.tuning[o.precision == BA_PRECISION_MIXED ? 1 : 0].point_us
                              : 0.0;
      st.pcg_coarse_dim = c.last_coarse_dim;
      st.schur_sub_len = c.last_sub_len;
      st.schur_tuned_us = c.tuning[o.precision == BA_PRECISION_MIXED ? 1 : 0].valid
                              ? c.tuning[o.precision == BA_PRECISION_MIXED ? 1 : 0].schur_us
                              : 0.0;
      st.pcg_tuned_us = c.tuning[o.precision == BA_PRECISION_MIXED ? 1 : 0].valid
                            ? c.tuning[o.precision == BA_PRECISION_MIXED ? 1 : 0].us_per_iter
                            : 0.0;
    }
  }
}

}  // namespace

void reset_states(Context& c) {
  cudaStream_t s = c.stream;
  auto cp = [&](DevBuf<double>& d, const DevBuf<double>& src) {
    if (src.n) check(cudaMemcpyAsync(d.p, src.p, src.bytes(), cudaMemcpyDeviceToDevice, s), "d2d");
  };
  cp(c.rot, c.init_rot), cp(c.center, c.init_center), cp(c.intr, c.init_intr),
      cp(c.points, c.init_points);
  cp(c.trot, c.init_rot), cp(c.tcenter, c.init_center), cp(c.tintr, c.init_intr),
      cp(c.tpoints, c.init_points);
}

}  // namespace ba

using namespace ba;

extern "C" {

void ba_default_options(ba_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  o->max_iter = 60;
  o->sigma_px = 1.0;
  o->loss = BA_LOSS_CAUCHY;
  o->precision = BA_PRECISION_FP64;
  o->pcg_max_iter = 400;
  o->pcg_tol = 1e-20;
}

ba_status ba_context_create(int32_t device, void* stream, ba_context** out) {
  if (!out) return set_error(BA_BAD_INPUT, "null output pointer");
  *out = nullptr;
  std::unique_ptr<ba_context> c(new ba_context());
  ba_status st = guarded([&] { init_context(*c, device, stream); });
  if (st == BA_OK) *out = c.release();
  return st;
}

void ba_context_destroy(ba_context* c) {
  if (!c) return;
  destroy_context(*c);
  delete c;
}

ba_status ba_context_upload(ba_context* c, const ba_problem* p, const ba_state* s, int32_t n) {
  if (!c) return set_error(BA_BAD_INPUT, "null context");
  return guarded([&] {
    check(cudaSetDevice(c->device), "cudaSetDevice");
    upload(*c, p, s, n);
  });
}

ba_status ba_context_solve(ba_context* c, const ba_options* opt, ba_stats* stats) {
  if (!c) return set_error(BA_BAD_INPUT, "null context");
  return guarded([&] { solve(*c, opt, stats); });
}

ba_status ba_context_download(ba_context* c, ba_state* s, int32_t n) {
  if (!c) return set_error(BA_BAD_INPUT, "null context");
  return guarded([&] {
    check(cudaSetDevice(c->device), "cudaSetDevice");
    download(*c, s, n);
  });
}

namespace {
std::mutex g_default_mu;
}

ba_status ba_solve_batch(const ba_problem* problems, ba_state* states, int32_t n,
                         const ba_options* opt, ba_stats* stats) {
  // One context per call: the reference's entry point has no handle, and a
  // call must not race another thread's call.
  ba_context* c = nullptr;
  const double t0 = now_ms();
  // The workspace limit covers the whole call: problem copies and solve.
  DevBudgetScope budget(opt ? opt->workspace_limit_bytes : 0);
  ba_status st = ba_context_create(-1, opt ? opt->stream : nullptr, &c);
  if (st != BA_OK) return st;
  st = ba_context_upload(c, problems, states, n);
  if (st == BA_OK) st = ba_context_solve(c, opt, stats);
  if (st == BA_OK) st = ba_context_download(c, states, n);
  if (st == BA_OK && stats) {
    const double t1 = now_ms();
    for (int m = 0; m < n; ++m) {
      stats[m].ms_total = t1 - t0;
      stats[m].ms_h2d = c->last_h2d_ms;
      stats[m].ms_d2h = c->last_d2h_ms;
      stats[m].h2d_bytes = c->last_h2d_bytes;
      stats[m].d2h_bytes = c->last_d2h_bytes;
    }
  }
  ba_context_destroy(c);
  return st;
}

ba_status ba_solve(const ba_problem* problem, ba_state* state, const ba_options* opt,
                   ba_stats* stats) {
  return ba_solve_batch(problem, state, 1, opt, stats);
}

ba_status ba_context_debug_step(ba_context* c, const ba_options* opt, double lambda,
                                double* S_dense, double* g, double* dx, int32_t* pcg_iters,
                                double* trial_cost) {
  if (!c) return set_error(BA_BAD_INPUT, "null context");
  return guarded([&] {
    if (!c->uploaded) throw BadInput("no problem uploaded");
    if (c->nm != 1) throw BadInput("debug step takes a single model");
    const Opts o = resolve_options(opt);
    check(cudaSetDevice(c->device), "cudaSetDevice");
    if (o.precision == 0)
      debug_lm_step<double>(*c, o, lambda, S_dense, g, dx, pcg_iters, trial_cost);
    else
      debug_lm_step<float>(*c, o, lambda, S_dense, g, dx, pcg_iters, trial_cost);
  });
}

const char* ba_last_error(void) { return g_last_error.c_str(); }
int32_t ba_abi_version(void) { return BA_GB300_ABI_VERSION; }
const char* ba_version(void) { return "ba_gb300 1.0 (sm_103a)"; }

}  // extern "C"
