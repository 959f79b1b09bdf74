// Device-resident problem batch held by a ba_context.
#pragma once

#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "ba_gb300.h"
#include "solver.cuh"

namespace ba {

struct ModelResult {
  int64_t iterations = 0;
  double initial_rms = 0, final_rms = 0, initial_cost = 0, final_cost = 0;
  int64_t pcg = 0;
};

constexpr int kPhases = 9;

// PCG configuration chosen by the autotuner for one form (FP64 / mixed).
struct PcgTuning {
  bool valid = false;
  int kernel = 1;       // 1 grid, 2 cluster
  int rows_target = 4;  // grid kernel: block rows per CTA
  int cluster = 0;      // cluster kernel: CTAs per cluster
  int cg_threads = 512; // cluster kernel: threads per CTA (512 or 1024)
  double us_per_iter = 0.0;
  int sub_len = 0;      // Schur pairs per warp sub-segment (0: the default)
  double schur_us = 0.0;
  int point_kernel = 0;  // mixed form's per-observation passes (0: the default)
  double point_us = 0.0;
};

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int n_sm = 0;

  // Sizes of the uploaded batch.
  int64_t nc = 0, np = 0, no = 0, ng = 0, nb = 0, nm = 0;
  bool has_prior = false;
  bool uploaded = false;
  std::vector<uint32_t> h_obs0, h_cam0, h_pt0, h_grp0, h_blk0;  // [nm+1]
  std::vector<uint8_t> h_refine;

  // Problem (device).
  DevBuf<uint32_t> obs_cam, obs_pt, cam_group;
  DevBuf<double> obs_uv, prior;
  DevBuf<uint8_t> prior_mask;
  DevBuf<uint32_t> cam_model, pt_model, grp_model, cam_blk, grp_blk, blk_model, blk_id;
  DevBuf<uint8_t> blk_is_lens, model_refine;
  DevBuf<uint32_t> model_obs0, model_cam0, model_blk0;
  // States: uploaded initial, current, trial.
  DevBuf<double> init_rot, init_center, init_intr, init_points;
  DevBuf<double> rot, center, intr, points;
  DevBuf<double> trot, tcenter, tintr, tpoints;
  DevBuf<uint32_t> err;  // device error bits

  std::vector<ModelResult> results;
  double phase_ms[kPhases] = {0};
  int64_t phase_n[kPhases] = {0};
  int64_t last_nz = 0, last_pairs = 0, last_nl = 0;
  int32_t last_pcg_kernel = 0, last_pcg_cluster = 0, last_pcg_ctas = 0, last_coarse_dim = 0;
  int32_t last_pcg_threads = 0, last_point_kernel = 0;
  int32_t last_sub_len = 0;
  PcgTuning tuning[2];  // [0] FP64 form, [1] mixed form
  bool last_graph = false;
  bool last_matrix_free = false;
  double last_h2d_ms = 0, last_d2h_ms = 0;
  int64_t last_h2d_bytes = 0, last_d2h_bytes = 0;

  Prob prob(int32_t loss) const {
    Prob P{};
    P.obs_cam = obs_cam;
    P.obs_pt = obs_pt;
    P.obs_uv = obs_uv;
    P.cam_group = cam_group;
    P.prior_mask = has_prior ? (const uint8_t*)prior_mask : nullptr;
    P.prior = prior;
    P.cam_model = cam_model;
    P.pt_model = pt_model;
    P.cam_blk = cam_blk;
    P.grp_blk = grp_blk;
    P.blk_model = blk_model;
    P.blk_id = blk_id;
    P.blk_is_lens = blk_is_lens;
    P.model_refine = model_refine;
    P.model_obs0 = model_obs0;
    P.model_cam0 = model_cam0;
    P.model_blk0 = model_blk0;
    P.nc = nc, P.np = np, P.no = no, P.ng = ng, P.nb = nb, P.nm = nm;
    P.loss = loss;
    return P;
  }
  StateView cur() const { return StateView{rot, center, intr, points}; }
  StateView trial() const { return StateView{trot, tcenter, tintr, tpoints}; }
};

// Resolved options.
struct Opts {
  int32_t max_iter = 60;
  double sigma = 1.0;
  int32_t loss = 0;
  int32_t precision = 0;
  int32_t pcg_max_iter = 400;
  double pcg_tol = 1e-20;
  int32_t matrix_free = 0;
  int64_t memory_cap = 0;
  ba_log* log = nullptr;
  int32_t profile = 0;
  int32_t pcg_kernel = 0;  // 0 auto, 1 grid, 2 cluster
  int32_t graph = 1;       // capture each LM iteration as a CUDA graph
  int32_t autotune = 0;    // tune the PCG configuration before solving
  int32_t stop_patience = 0;  // 0 or 1: the reference's stop rule
  int32_t pcg_end_max_iter = 0;  // PCG cap once a step's relative decrease < pcg_end_rel (0: off)
  double pcg_end_rel = 1e-5;
  int32_t coarse = 0;         // mixed cluster PCG: two-level preconditioner
  int32_t hold_cta = 0;       // fault injection: grid PCG CTA hold_cta-1 skips its exchanges
  long long wait_limit = kSpinCycles;  // spin limit of device-side waits (cycles)
  int64_t workspace_limit = 0;         // device bytes the call may hold (0: no limit)
  int32_t point_kernel = 0;  // mixed form's per-observation passes (ba_options numbering)
};

// One solve of the uploaded batch from its initial states, in precision R.
template <typename R>
void run_lm(Context& ctx, const Opts& o);

template <typename R>
void debug_lm_step(Context& ctx, const Opts& o, double lam, double* S_dense, double* g,
                   double* dx, int32_t* pcg_iters, double* trial_cost);

void reset_states(Context& ctx);

// Copy problems and initial states (host or device arrays) into the context.
void upload(Context& c, const ba_problem* P, const ba_state* S, int32_t n);

struct BadInput : std::runtime_error {
  using std::runtime_error::runtime_error;
};

Opts resolve_options(const ba_options* o);

// Status plumbing of the C ABI: run f, map exceptions to a status and keep
// the message for ba_last_error().
ba_status set_error(ba_status st, const std::string& msg);
ba_status run_guarded(void (*fn)(void*), void* arg);

template <typename F>
ba_status guarded(F&& f) {
  using Fn = std::remove_reference_t<F>;
  return run_guarded([](void* a) { (*static_cast<Fn*>(a))(); }, &f);
}

}  // namespace ba

struct ba_context : ba::Context {};
