// Device data model of the bundle-adjustment solver.
//
// A call solves a batch of independent models (one model is the batch of
// one, the drop-in for ba.rs:198).  The models are concatenated: cameras,
// lens groups, points and observations of model m occupy contiguous ranges,
// and the reduced-system block rows of model m are its cameras followed by its
// lens groups (for one model: cameras 0..nc-1, then lens blocks nc..nc+ng-1,
// as in ba.rs:199-201).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "ba_common.cuh"
#include "primitives.cuh"

namespace ba {

constexpr uint64_t kSentinel = 0xffffffffffffffffULL;  // diagonal marker in the pair list
constexpr uint32_t kNone = 0xffffffffu;
constexpr int kSubLen = 512;  // Schur pair contributions per warp sub-segment

// Read-only problem (device pointers).
struct Prob {
  const uint32_t* obs_cam;
  const uint32_t* obs_pt;
  const double* obs_uv;
  const uint32_t* cam_group;   // global group id
  const uint8_t* prior_mask;   // may be null
  const double* prior;         // 6 per camera
  const uint32_t* cam_model;
  const uint32_t* pt_model;
  const uint32_t* cam_blk;     // block row of each camera
  const uint32_t* grp_blk;     // block row of each group
  const uint32_t* blk_model;
  const uint32_t* blk_id;      // camera or group id of each block
  const uint8_t* blk_is_lens;
  const uint8_t* model_refine;
  const uint32_t* model_obs0;  // [nm+1]
  const uint32_t* model_cam0;  // [nm+1]
  const uint32_t* model_blk0;  // [nm+1]
  int64_t nc, np, no, ng, nb, nm;
  int32_t loss;
};

struct StateView {
  double* rot;
  double* center;
  double* intr;
  double* points;
};

// Per-call structure (fixed while a call iterates).
struct StructView {
  const uint32_t* pt_ptr;    // [np+1] observation range of each point
  const uint32_t* pt_order;  // [np] points by observation count (thread order of per-point kernels)
  const uint32_t* cam_ptr;   // [nc+1]
  const uint32_t* cam_obs;   // [no] observations ordered by camera (stable)
  const uint32_t* grp_ptr;   // [ng+1]
  const uint32_t* grp_cams;  // [nc] cameras ordered by group (stable)
  const uint32_t* lens_ptr;  // [np+1] lens entries of each point
  const uint32_t* lens_grp;  // [nl]
  const uint32_t* obs_lens;  // [no] lens entry fed by each observation
  const uint64_t* pairs;     // [npairs] (entry a) | (entry b) << 32
  const uint32_t* slot_ptr;  // [ns+1]
  const uint32_t* slot_row;  // [ns] block row (a <= b)
  const uint32_t* slot_col;  // [ns]
  const uint32_t* slot_pos_ab;  // [ns] position of (a,b) in the full BSR
  const uint32_t* slot_pos_ba;  // [ns] position of (b,a)
  const uint32_t* sub_slot;  // [nsub]
  const uint32_t* sub_begin; // [nsub]
  const uint32_t* sub_end;   // [nsub]
  const uint32_t* slot_sub_ptr;  // [ns+1]
  const uint32_t* row_ptr;   // [nb+1] full symmetric BSR
  const uint32_t* col_idx;   // [nz]
  const uint32_t* diag_pos;  // [nb]
  const uint32_t* cost_chunk_model;  // [ncost]
  const uint32_t* cost_chunk_begin;  // [ncost]
  const uint32_t* cost_chunk_end;    // [ncost]
  const uint32_t* model_chunk0;      // [nm+1]
  int64_t nl, npairs, ns, nsub, nz, ncost;
};

// Per-model LM control (device).
struct Control {
  double* lambda;
  double* cost;       // accepted cost
  double* new_cost;   // cost of the trial state
  double* rms;
  double* sq;
  int64_t* n_front;
  int32_t* active;    // model still iterating
  int32_t* accepted;  // trial accepted this iteration
  int32_t* iters;     // LM iterations done
  int32_t* pcg_iters; // PCG products this iteration
  int64_t* pcg_total;
  int32_t* any_active;
  double* sigma;      // per model
  int32_t* small;     // consecutive accepted steps below the 1e-6 decrease
  int32_t patience;   // stop after this many (1: the reference's rule)
  int32_t max_iter;
  // End-game PCG cap: once an accepted step decreases a model's cost by less
  // than end_rel (relative), pcg_cap[m] becomes end_cap (end_cap 0: off).
  int32_t* pcg_cap;
  int32_t end_cap;
  double end_rel;
  // per-iteration log of model 0 (device arrays, log_cap entries)
  int32_t log_cap;
  double* log_new_cost;
  double* log_lambda;
  int32_t* log_pcg;
  int32_t* log_accept;
  // mixed form: per model, 1 if the stored records are not at the current
  // state (set after every trial cost; null in the FP64 form)
  int32_t* rec_stale = nullptr;
};

}  // namespace ba
