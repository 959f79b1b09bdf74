// Per-call structure builder (see structure.cu).
#pragma once

#include <vector>

#include "solver.cuh"

namespace ba {

struct StructBufs {
  DevBuf<uint32_t> pt_ptr, pt_order, cam_ptr, cam_obs, grp_ptr, grp_cams, lens_ptr, lens_grp, obs_lens;
  // Camera-major Schur factors: the position of each observation in the
  // camera ordering (cam_pos[cam_obs[i]] = i), which the pair list then
  // holds in place of observation indices.
  DevBuf<uint32_t> cam_pos;
  bool z_by_camera = false;
  DevBuf<uint64_t> pairs;
  DevBuf<uint32_t> slot_ptr, slot_row, slot_col, slot_pos_ab, slot_pos_ba;
  DevBuf<uint32_t> sub_slot, sub_begin, sub_end, slot_sub_ptr;
  DevBuf<uint32_t> row_ptr, col_idx, diag_pos;
  DevBuf<uint32_t> cost_chunk_model, cost_chunk_begin, cost_chunk_end, model_chunk0;
  int64_t nl = 0, npairs = 0, ns = 0, nsub = 0, nz = 0, ncost = 0;
  bool implicit = false;  // no pair list / reduced matrix (matrix-free PCG)
  std::vector<uint32_t> h_row_ptr;
  StructView view() const;
};

// Index, ordering and model checks of the problem, and finiteness of the
// measurements, priors (sigmas > 0) and initial state `st`: error bits into
// d_err.
void validate_problem(const Prob& P, const StateView& st, const uint32_t* grp_model,
                      uint32_t* d_err, cudaStream_t s);
// Observations by camera (cam_ptr, cam_obs) and cameras by group (grp_ptr,
// grp_cams), both stable.
void build_cam_index(const Prob& P, StructBufs& S, cudaStream_t s);
// pair_bytes_cap: < 0 always build the Schur pair list and the reduced
// matrix layout; 0 never (matrix-free); > 0 only if they fit in that many
// bytes.  z_by_camera: the pair list addresses Schur factors stored in the
// camera ordering of the observations (cam_pos) instead of observation order.
// Warp sub-segments of the Schur sums: each destination block's pair range
// cut into runs of at most sub_len pairs (a warp each); replaces any earlier
// sub-segments of S.
void build_subsegments(StructBufs& S, uint32_t sub_len, cudaStream_t s);
void build_structure(const Prob& P, const std::vector<uint32_t>& h_model_obs0, StructBufs& S,
                     uint32_t* err, cudaStream_t s, int64_t pair_bytes_cap = -1,
                     bool z_by_camera = false);

}  // namespace ba
