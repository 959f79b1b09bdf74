// Per-call structure of the reduced camera system, built on the device.
//
// The reference rebuilds the point ranges every call (ba.rs:203-214) and
// discovers the sparsity of the reduced matrix while adding blocks into hash
// maps (ba.rs:130-153, 270-331).  Here the sparsity is fixed once per call,
// because it does not change while the call iterates:
//   * observation ranges of points (obs are sorted by point) and a stable
//     camera ordering of the observations;
//   * the lens entries of each point: one per distinct lens group among its
//     observations, in first-occurrence order (ba.rs:251-259);
//   * every ordered pair (a, b) of a point's entries with block(a) <=
//     block(b): the Schur contributions Y_a V^-1 Y_b^T (ba.rs:320-331),
//     radix-sorted by destination block so each upper block of the reduced
//     matrix is a contiguous segment, summed in point order (deterministic);
//   * the full symmetric block-sparse-row layout used by PCG.
#include <algorithm>
#include <vector>

#include "structure.cuh"

namespace ba {
namespace {

__device__ __forceinline__ bool all_finite(const double* v, int n) {
  bool ok = true;
  for (int i = 0; i < n; ++i) ok = ok && isfinite(v[i]);
  return ok;
}

__global__ void validate_kernel(Prob P, StateView st, const uint32_t* grp_model, uint32_t* err) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t e = 0;
  if (k < P.no) {
    const uint32_t c = P.obs_cam[k], p = P.obs_pt[k];
    if (c >= P.nc || p >= P.np) {
      e |= ERR_BAD_INDEX;
    } else {
      if (P.cam_model[c] != P.pt_model[p]) e |= ERR_MODEL_MIX;
      if (k > 0 && P.obs_pt[k - 1] > p) e |= ERR_UNSORTED;
    }
    if (!all_finite(P.obs_uv + 2 * k, 2)) e |= ERR_NONFINITE;
  }
  if (k < P.nc) {
    const uint32_t g = P.cam_group[k];
    if (g >= P.ng)
      e |= ERR_BAD_INDEX;
    else if (grp_model[g] != P.cam_model[k])
      e |= ERR_MODEL_MIX;
    if (!all_finite(st.rot + 9 * k, 9) || !all_finite(st.center + 3 * k, 3)) e |= ERR_NONFINITE;
    // A prior's sigmas divide its residual (ba.rs:120-126).
    if (P.prior_mask && P.prior_mask[k]) {
      const double* q = P.prior + 6 * k;
      if (!all_finite(q, 6) || !(q[3] > 0.0 && q[4] > 0.0 && q[5] > 0.0)) e |= ERR_NONFINITE;
    }
  }
  if (k < P.np && !all_finite(st.points + 3 * k, 3)) e |= ERR_NONFINITE;
  if (k < P.ng && !all_finite(st.intr + 5 * k, 5)) e |= ERR_NONFINITE;
  if (e) atomicOr(err, e);
}

__global__ void iota_keys_kernel(const uint32_t* src, uint64_t* keys, uint32_t* vals,
                                 int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    keys[i] = src[i];
    vals[i] = (uint32_t)i;
  }
}

__device__ __forceinline__ bool point_has_lens(const Prob& P, uint32_t p) {
  return P.model_refine[P.pt_model[p]] != 0;
}

__global__ void order_keys_kernel(int64_t np, const uint32_t* pt_ptr, uint64_t* key,
                                  uint32_t* idx) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  key[p] = min(pt_ptr[p + 1] - pt_ptr[p], 0xffffu);
  idx[p] = (uint32_t)p;
}

__global__ void lens_count_kernel(Prob P, const uint32_t* pt_ptr, uint32_t* cnt) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.np) return;
  const uint32_t s = pt_ptr[p], e = pt_ptr[p + 1];
  uint32_t n = 0;
  if (e - s >= 2 && point_has_lens(P, (uint32_t)p)) {
    for (uint32_t k = s; k < e; ++k) {
      const uint32_t g = P.cam_group[P.obs_cam[k]];
      bool seen = false;
      for (uint32_t j = s; j < k; ++j)
        if (P.cam_group[P.obs_cam[j]] == g) {
          seen = true;
          break;
        }
      if (!seen) ++n;
    }
  }
  cnt[p] = n;
}

__global__ void lens_fill_kernel(Prob P, const uint32_t* pt_ptr, const uint32_t* lens_ptr,
                                 uint32_t* lens_grp, uint32_t* obs_lens) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.np) return;
  const uint32_t s = pt_ptr[p], e = pt_ptr[p + 1];
  const uint32_t l0 = lens_ptr[p], l1 = lens_ptr[p + 1];
  if (l1 == l0) {
    for (uint32_t k = s; k < e; ++k) obs_lens[k] = kNone;
    return;
  }
  uint32_t n = 0;
  for (uint32_t k = s; k < e; ++k) {
    const uint32_t g = P.cam_group[P.obs_cam[k]];
    uint32_t ent = kNone;
    for (uint32_t j = l0; j < l0 + n; ++j)
      if (lens_grp[j] == g) {
        ent = j;
        break;
      }
    if (ent == kNone) {
      ent = l0 + n++;
      lens_grp[ent] = g;
    }
    obs_lens[k] = ent;
  }
}

// Entries of point p: its observations (camera blocks), then its lens entries.
struct Entries {
  uint32_t s, m, l0, nl;
  __device__ __forceinline__ uint32_t count() const { return m + nl; }
  __device__ __forceinline__ void get(const Prob& P, const uint32_t* lens_grp, uint32_t t,
                                      uint32_t& eid, uint32_t& blk) const {
    if (t < m) {
      eid = s + t;
      blk = P.cam_blk[P.obs_cam[s + t]];
    } else {
      const uint32_t j = l0 + (t - m);
      eid = (uint32_t)P.no + j;
      blk = P.grp_blk[lens_grp[j]];
    }
  }
};

__device__ __forceinline__ Entries entries_of(const uint32_t* pt_ptr, const uint32_t* lens_ptr,
                                              int64_t p) {
  Entries E;
  E.s = pt_ptr[p];
  E.m = pt_ptr[p + 1] - E.s;
  E.l0 = lens_ptr[p];
  E.nl = lens_ptr[p + 1] - E.l0;
  return E;
}

// Pair enumeration, a warp per point: lane t holds entry t's id and block
// (entries 32.. are loaded as needed), and entry i is broadcast from its lane
// while the lanes test and emit the pairs (i, j), j = lane, lane + 32, ...;
// a ballot ranks the emitted pairs, so they keep the order of a sequential
// loop over i, then j.
struct WarpEntries {
  Entries E;
  uint32_t ne, my_e, my_b;
  __device__ __forceinline__ void load(const Prob& P, const uint32_t* lens_grp, int lane) {
    ne = E.count();
    my_e = 0, my_b = 0;
    if ((uint32_t)lane < ne) E.get(P, lens_grp, (uint32_t)lane, my_e, my_b);
  }
  __device__ __forceinline__ void at(const Prob& P, const uint32_t* lens_grp, uint32_t t,
                                     uint32_t& e, uint32_t& b) const {
    if (t < 32) {  // uniform over the warp
      e = __shfl_sync(kFull, my_e, (int)t);
      b = __shfl_sync(kFull, my_b, (int)t);
    } else {
      E.get(P, lens_grp, t, e, b);
    }
  }
};

__global__ void pair_count_kernel(Prob P, const uint32_t* pt_ptr, const uint32_t* lens_ptr,
                                  const uint32_t* lens_grp, uint32_t* cnt) {
  const int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (p >= P.np) return;
  WarpEntries W;
  W.E = entries_of(pt_ptr, lens_ptr, p);
  uint32_t n = 0;
  if (W.E.m >= 2) {
    W.load(P, lens_grp, lane);
    for (uint32_t i = 0; i < W.ne; ++i) {
      uint32_t ei, bi;
      W.at(P, lens_grp, i, ei, bi);
      for (uint32_t j0 = 0; j0 < W.ne; j0 += 32) {
        const uint32_t j = j0 + lane;
        uint32_t ej = 0, bj = 0;
        if (j0 == 0) {
          ej = W.my_e, bj = W.my_b;
        } else if (j < W.ne) {
          W.E.get(P, lens_grp, j, ej, bj);
        }
        n += __popc(__ballot_sync(kFull, j < W.ne && bi <= bj));
      }
    }
  }
  if (lane == 0) cnt[p] = n;
}

// zpos: null, or the storage position of each observation's Schur factor
// (entries of observations are stored as that position; lens entries,
// numbered from no, are kept).
__global__ void pair_fill_kernel(Prob P, const uint32_t* pt_ptr, const uint32_t* lens_ptr,
                                 const uint32_t* lens_grp, const uint32_t* off,
                                 const uint32_t* zpos, uint64_t* keys, uint64_t* vals) {
  const int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (p >= P.np) return;
  WarpEntries W;
  W.E = entries_of(pt_ptr, lens_ptr, p);
  if (W.E.m < 2) return;  // uniform over the warp
  W.load(P, lens_grp, lane);
  // the first 32 entries' storage positions, looked up once per point
  if (zpos && (uint32_t)lane < W.ne && (int64_t)W.my_e < P.no) W.my_e = zpos[W.my_e];
  uint64_t o = off[p];
  const uint64_t nb = (uint64_t)P.nb;
  const uint32_t lt = (1u << lane) - 1u;
  for (uint32_t i = 0; i < W.ne; ++i) {
    uint32_t ei, bi;
    W.at(P, lens_grp, i, ei, bi);
    if (i >= 32 && zpos && (int64_t)ei < P.no) ei = zpos[ei];
    for (uint32_t j0 = 0; j0 < W.ne; j0 += 32) {
      const uint32_t j = j0 + lane;
      uint32_t ej = 0, bj = 0;
      if (j0 == 0) {
        ej = W.my_e, bj = W.my_b;
      } else if (j < W.ne) {
        W.E.get(P, lens_grp, j, ej, bj);
        if (zpos && (int64_t)ej < P.no) ej = zpos[ej];
      }
      const bool take = j < W.ne && bi <= bj;
      const uint32_t mask = __ballot_sync(kFull, take);
      if (take) {
        const uint64_t q = o + __popc(mask & lt);
        keys[q] = (uint64_t)bi * nb + bj;
        vals[q] = (uint64_t)ei | ((uint64_t)ej << 32);
      }
      o += __popc(mask);
    }
  }
}

__global__ void inverse_perm_kernel(const uint32_t* perm, int64_t n, uint32_t* inv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) inv[perm[i]] = (uint32_t)i;
}

__global__ void diag_marker_kernel(uint64_t* keys, uint64_t* vals, int64_t base, int64_t nb) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  keys[base + b] = (uint64_t)b * (uint64_t)nb + (uint64_t)b;
  vals[base + b] = kSentinel;
}

__global__ void head_flags_kernel(const uint64_t* keys, int64_t n, uint32_t* head) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) head[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

__global__ void slot_fill_kernel(const uint64_t* keys, int64_t n, const uint32_t* head,
                                 const uint32_t* sid, int64_t nb, uint32_t* slot_ptr,
                                 uint64_t* slot_key) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && head[i]) {
    slot_ptr[sid[i]] = (uint32_t)i;
    slot_key[sid[i]] = keys[i];
  }
}

__global__ void slot_rowcol_kernel(const uint64_t* slot_key, int64_t ns, int64_t nb,
                                   uint32_t* row, uint32_t* col, uint32_t* offdiag) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  const uint64_t k = slot_key[s];
  row[s] = (uint32_t)(k / (uint64_t)nb);
  col[s] = (uint32_t)(k % (uint64_t)nb);
  offdiag[s] = (row[s] != col[s]) ? 1u : 0u;
}

__global__ void transpose_keys_kernel(const uint32_t* row, const uint32_t* col,
                                      const uint32_t* offdiag, const uint32_t* toff, int64_t ns,
                                      int64_t nb, uint64_t* tkeys, uint32_t* tvals) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns || !offdiag[s]) return;
  const uint32_t o = toff[s];
  tkeys[o] = (uint64_t)col[s] * (uint64_t)nb + row[s];
  tvals[o] = (uint32_t)s;
}

__global__ void row_count_kernel(const uint32_t* up_first, const uint32_t* lo_first, int64_t nb,
                                 uint32_t* cnt) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nb) cnt[r] = (up_first[r + 1] - up_first[r]) + (lo_first[r + 1] - lo_first[r]);
}

__global__ void place_upper_kernel(const uint32_t* row, const uint32_t* col, int64_t ns,
                                   const uint32_t* row_ptr, const uint32_t* up_first,
                                   const uint32_t* lo_first, uint32_t* col_idx,
                                   uint32_t* pos_ab, uint32_t* pos_ba, uint32_t* diag_pos,
                                   int64_t nb, int64_t nz, uint32_t* err) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  const uint32_t a = row[s], b = col[s];
  if (a >= nb || b >= nb || (uint32_t)s < up_first[a] || (uint32_t)s >= up_first[a + 1]) {
    atomicOr(err, ERR_STRUCTURE);
    return;
  }
  const uint32_t pos = row_ptr[a] + (lo_first[a + 1] - lo_first[a]) + ((uint32_t)s - up_first[a]);
  if (pos >= row_ptr[a + 1] || pos >= nz) {
    atomicOr(err, ERR_STRUCTURE);
    return;
  }
  col_idx[pos] = b;
  pos_ab[s] = pos;
  if (a == b) {
    pos_ba[s] = pos;
    diag_pos[a] = pos;
  }
}

__global__ void place_lower_kernel(const uint64_t* tkeys, const uint32_t* tvals, int64_t nt,
                                   int64_t nb, const uint32_t* row_ptr, const uint32_t* lo_first,
                                   uint32_t* col_idx, uint32_t* pos_ba, int64_t ns, int64_t nz,
                                   uint32_t* err) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  const uint64_t k = tkeys[i];
  const uint32_t r = (uint32_t)(k / (uint64_t)nb), c = (uint32_t)(k % (uint64_t)nb);
  if (r >= nb || (uint32_t)i < lo_first[r] || (uint32_t)i >= lo_first[r + 1] || tvals[i] >= ns) {
    atomicOr(err, ERR_STRUCTURE);
    return;
  }
  const uint32_t pos = row_ptr[r] + ((uint32_t)i - lo_first[r]);
  if (pos >= nz) {
    atomicOr(err, ERR_STRUCTURE);
    return;
  }
  col_idx[pos] = c;
  pos_ba[tvals[i]] = pos;
}

__global__ void sub_count_kernel(const uint32_t* slot_ptr, int64_t ns, uint32_t sub_len,
                                 uint32_t* cnt) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  const uint32_t len = slot_ptr[s + 1] - slot_ptr[s];
  cnt[s] = len == 0 ? 1u : (len + sub_len - 1) / sub_len;
}

__global__ void sub_fill_kernel(const uint32_t* slot_ptr, const uint32_t* sub_ptr, int64_t ns,
                                uint32_t sub_len, uint32_t* sub_slot, uint32_t* sub_begin,
                                uint32_t* sub_end) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  const uint32_t b = slot_ptr[s], e = slot_ptr[s + 1];
  const uint32_t n = sub_ptr[s + 1] - sub_ptr[s];
  for (uint32_t t = 0; t < n; ++t) {
    const uint32_t o = sub_ptr[s] + t;
    sub_slot[o] = (uint32_t)s;
    sub_begin[o] = b + t * sub_len;
    sub_end[o] = min(e, b + (t + 1) * sub_len);
  }
}

int bits_for(uint64_t maxval) {
  int b = 0;
  while (b < 64 && (maxval >> b) != 0) ++b;
  return b;
}

constexpr unsigned T = 256;

}  // namespace

StructView StructBufs::view() const {
  StructView v{};
  v.pt_ptr = pt_ptr;
  v.pt_order = pt_order;
  v.cam_ptr = cam_ptr;
  v.cam_obs = cam_obs;
  v.grp_ptr = grp_ptr;
  v.grp_cams = grp_cams;
  v.lens_ptr = lens_ptr;
  v.lens_grp = lens_grp;
  v.obs_lens = obs_lens;
  v.pairs = pairs;
  v.slot_ptr = slot_ptr;
  v.slot_row = slot_row;
  v.slot_col = slot_col;
  v.slot_pos_ab = slot_pos_ab;
  v.slot_pos_ba = slot_pos_ba;
  v.sub_slot = sub_slot;
  v.sub_begin = sub_begin;
  v.sub_end = sub_end;
  v.slot_sub_ptr = slot_sub_ptr;
  v.row_ptr = row_ptr;
  v.col_idx = col_idx;
  v.diag_pos = diag_pos;
  v.cost_chunk_model = cost_chunk_model;
  v.cost_chunk_begin = cost_chunk_begin;
  v.cost_chunk_end = cost_chunk_end;
  v.model_chunk0 = model_chunk0;
  v.nl = nl;
  v.npairs = npairs;
  v.ns = ns;
  v.nsub = nsub;
  v.nz = nz;
  v.ncost = ncost;
  return v;
}

void validate_problem(const Prob& P, const StateView& st, const uint32_t* grp_model,
                      uint32_t* d_err, cudaStream_t s) {
  const int64_t n = std::max(std::max(P.no, P.nc), std::max(P.np, P.ng));
  if (n > 0) BA_LAUNCH(validate_kernel<<<grid_for(n, T), T, 0, s>>>(P, st, grp_model, d_err));
}

void build_cam_index(const Prob& P, StructBufs& S, cudaStream_t s) {
  const int64_t nc = P.nc, no = P.no, ng = P.ng;
  // Observations ordered by camera, stable in observation order.
  {
    DevBuf<uint64_t> k(std::max<int64_t>(no, 1), s), kt(std::max<int64_t>(no, 1), s);
    DevBuf<uint32_t> vt(std::max<int64_t>(no, 1), s);
    S.cam_obs.alloc(std::max<int64_t>(no, 1), s);
    if (no > 0) {
      BA_LAUNCH(iota_keys_kernel<<<grid_for(no, T), T, 0, s>>>(P.obs_cam, k, S.cam_obs, no));
      radix_sort_u64_u32(k, S.cam_obs, kt, vt, no, bits_for((uint64_t)nc), s);
    }
    S.cam_ptr.alloc(nc + 1, s);
    lower_bounds_u64(k, no, S.cam_ptr, nc, 1, s);
  }
  // Cameras ordered by lens group.
  {
    DevBuf<uint64_t> k(nc, s), kt(nc, s);
    DevBuf<uint32_t> vt(nc, s);
    S.grp_cams.alloc(nc, s);
    BA_LAUNCH(iota_keys_kernel<<<grid_for(nc, T), T, 0, s>>>(P.cam_group, k, S.grp_cams, nc));
    radix_sort_u64_u32(k, S.grp_cams, kt, vt, nc, bits_for((uint64_t)ng), s);
    S.grp_ptr.alloc(ng + 1, s);
    lower_bounds_u64(k, nc, S.grp_ptr, ng, 1, s);
  }
}

void build_subsegments(StructBufs& S, uint32_t sub_len, cudaStream_t s) {
  const int64_t ns = S.ns;
  if (ns <= 0) return;
  DevBuf<uint32_t> cnt(ns + 1, s);
  BA_LAUNCH(sub_count_kernel<<<grid_for(ns, T), T, 0, s>>>(S.slot_ptr, ns, sub_len, cnt));
  check(cudaMemsetAsync(cnt.p + ns, 0, 4, s), "memset");
  S.slot_sub_ptr.alloc(ns + 1, s);
  S.nsub = (int64_t)exclusive_scan_u32(cnt, S.slot_sub_ptr, ns + 1, s);
  S.sub_slot.alloc(S.nsub, s);
  S.sub_begin.alloc(S.nsub, s);
  S.sub_end.alloc(S.nsub, s);
  BA_LAUNCH(sub_fill_kernel<<<grid_for(ns, T), T, 0, s>>>(S.slot_ptr, S.slot_sub_ptr, ns, sub_len,
                                                        S.sub_slot, S.sub_begin, S.sub_end));
}

void build_structure(const Prob& P, const std::vector<uint32_t>& h_model_obs0, StructBufs& S,
                     uint32_t* err, cudaStream_t s, int64_t pair_bytes_cap, bool z_by_camera) {
  const int64_t nc = P.nc, np = P.np, no = P.no, ng = P.ng, nb = P.nb, nm = P.nm;

  // Point ranges (obs are sorted by point).
  S.pt_ptr.alloc(np + 1, s);
  lower_bounds_u32(P.obs_pt, no, S.pt_ptr, np, s);
  // Thread order of the per-point kernels: points by observation count
  // (stable), so that the threads of a warp loop over the same number of
  // observations.  Results do not depend on it: points are independent.
  S.pt_order.alloc(std::max<int64_t>(np, 1), s);
  if (np > 0) {
    DevBuf<uint64_t> key(np, s), ktmp(np, s);
    DevBuf<uint32_t> vtmp(np, s);
    BA_LAUNCH(order_keys_kernel<<<grid_for(np, T), T, 0, s>>>(np, S.pt_ptr, key, S.pt_order));
    radix_sort_u64_u32(key, S.pt_order, ktmp, vtmp, np, 16, s);
  }

  build_cam_index(P, S, s);
  // Lens entries.
  S.lens_ptr.alloc(np + 1, s);
  S.obs_lens.alloc(std::max<int64_t>(no, 1), s);
  {
    DevBuf<uint32_t> cnt(np + 1, s);
    cnt.zero();
    if (np > 0)
      BA_LAUNCH(lens_count_kernel<<<grid_for(np, T), T, 0, s>>>(P, S.pt_ptr, cnt));
    S.nl = (int64_t)exclusive_scan_u32(cnt, S.lens_ptr, np + 1, s);
    S.lens_grp.alloc(std::max<int64_t>(S.nl, 1), s);
    if (np > 0)
      BA_LAUNCH(lens_fill_kernel<<<grid_for(np, T), T, 0, s>>>(P, S.pt_ptr, S.lens_ptr,
                                                             S.lens_grp, S.obs_lens));
  }
  // Schur pair list, sorted by destination block.
  DevBuf<uint64_t> keys;
  int64_t npairs = 0;
  S.implicit = false;
  DevBuf<uint32_t> cnt(np + 1, s), off(np + 1, s);
  cnt.zero();
  if (np > 0)
    BA_LAUNCH(pair_count_kernel<<<grid_for(np * 32, T), T, 0, s>>>(P, S.pt_ptr, S.lens_ptr,
                                                                 S.lens_grp, cnt));
  const uint64_t npt = exclusive_scan_u32(cnt, off, np + 1, s);
  const uint64_t total = npt + (uint64_t)nb;
  // Matrix-free calls (cap 0), or a pair list (with its sort buffers and the
  // Schur partial sums) above the memory cap: no pair list, no S.
  if (pair_bytes_cap == 0 || (pair_bytes_cap > 0 && (int64_t)total * 40 > pair_bytes_cap))
    S.implicit = true;
  S.z_by_camera = !S.implicit && z_by_camera && no > 0;
  if (S.z_by_camera) {
    S.cam_pos.alloc(no, s);
    BA_LAUNCH(inverse_perm_kernel<<<grid_for(no, T), T, 0, s>>>(S.cam_obs, no, S.cam_pos));
  }
  if (!S.implicit) {
    if (total >= 0xffffffffULL)
      throw std::runtime_error("too many Schur pair contributions for one call");
    npairs = (int64_t)total;
    keys.alloc(npairs, s);
    S.pairs.alloc(npairs, s);
    if (np > 0)
      BA_LAUNCH(pair_fill_kernel<<<grid_for(np * 32, T), T, 0, s>>>(
          P, S.pt_ptr, S.lens_ptr, S.lens_grp, off, S.z_by_camera ? S.cam_pos.p : nullptr, keys,
          S.pairs));
    BA_LAUNCH(diag_marker_kernel<<<grid_for(nb, T), T, 0, s>>>(keys, S.pairs, (int64_t)npt, nb));
    DevBuf<uint64_t> kt(npairs, s), vt(npairs, s);
    radix_sort_u64_u64(keys, S.pairs, kt, vt, npairs, bits_for((uint64_t)nb * nb - 1), s);
  }
  cnt.release();
  off.release();
  S.npairs = npairs;
  if (!S.implicit) {
    // Slots = distinct destination blocks (upper triangle incl. diagonal).
    DevBuf<uint64_t> slot_key;
    {
      DevBuf<uint32_t> head(npairs, s), sid(npairs, s);
      BA_LAUNCH(head_flags_kernel<<<grid_for(npairs, T), T, 0, s>>>(keys, npairs, head));
      S.ns = (int64_t)exclusive_scan_u32(head, sid, npairs, s);
      S.slot_ptr.alloc(S.ns + 1, s);
      slot_key.alloc(S.ns, s);
      BA_LAUNCH(slot_fill_kernel<<<grid_for(npairs, T), T, 0, s>>>(keys, npairs, head, sid, nb,
                                                                 S.slot_ptr, slot_key));
      const uint32_t np32 = (uint32_t)npairs;
      check(cudaMemcpyAsync(S.slot_ptr.p + S.ns, &np32, 4, cudaMemcpyHostToDevice, s), "slot");
    }
    keys.release();
    const int64_t ns = S.ns;
    // Full symmetric BSR.
    S.slot_row.alloc(ns, s);
    S.slot_col.alloc(ns, s);
    S.slot_pos_ab.alloc(ns, s);
    S.slot_pos_ba.alloc(ns, s);
    S.diag_pos.alloc(nb, s);
    {
      DevBuf<uint32_t> offd(ns + 1, s), toff(ns + 1, s);
      BA_LAUNCH(slot_rowcol_kernel<<<grid_for(ns, T), T, 0, s>>>(slot_key, ns, nb, S.slot_row,
                                                               S.slot_col, offd));
      check(cudaMemsetAsync(offd.p + ns, 0, 4, s), "memset");
      const int64_t nt = (int64_t)exclusive_scan_u32(offd, toff, ns + 1, s);
      DevBuf<uint64_t> tk(std::max<int64_t>(nt, 1), s), tkt(std::max<int64_t>(nt, 1), s);
      DevBuf<uint32_t> tv(std::max<int64_t>(nt, 1), s), tvt(std::max<int64_t>(nt, 1), s);
      BA_LAUNCH(transpose_keys_kernel<<<grid_for(ns, T), T, 0, s>>>(S.slot_row, S.slot_col, offd,
                                                                  toff, ns, nb, tk, tv));
      if (nt > 1) radix_sort_u64_u32(tk, tv, tkt, tvt, nt, bits_for((uint64_t)nb * nb - 1), s);
      DevBuf<uint32_t> up_first(nb + 1, s), lo_first(nb + 1, s), cnt(nb + 1, s);
      lower_bounds_u64(slot_key, ns, up_first, nb, (uint64_t)nb, s);
      lower_bounds_u64(tk, nt, lo_first, nb, (uint64_t)nb, s);
      BA_LAUNCH(row_count_kernel<<<grid_for(nb, T), T, 0, s>>>(up_first, lo_first, nb, cnt));
      check(cudaMemsetAsync(cnt.p + nb, 0, 4, s), "memset");
      S.row_ptr.alloc(nb + 1, s);
      S.nz = (int64_t)exclusive_scan_u32(cnt, S.row_ptr, nb + 1, s);
      S.col_idx.alloc(S.nz, s);
      BA_LAUNCH(place_upper_kernel<<<grid_for(ns, T), T, 0, s>>>(
          S.slot_row, S.slot_col, ns, S.row_ptr, up_first, lo_first, S.col_idx, S.slot_pos_ab,
          S.slot_pos_ba, S.diag_pos, nb, S.nz, err));
      if (nt > 0)
        BA_LAUNCH(place_lower_kernel<<<grid_for(nt, T), T, 0, s>>>(tk, tv, nt, nb, S.row_ptr,
                                                                 lo_first, S.col_idx,
                                                                 S.slot_pos_ba, ns, S.nz, err));
    }
    slot_key.release();
    build_subsegments(S, kSubLen, s);

  } else {
    S.ns = S.nsub = S.nz = 0;
    S.diag_pos.alloc(1, s);
  }
  // Cost-reduction chunks, aligned to model boundaries (host-side plan).
  {
    constexpr uint32_t CH = 4096;
    std::vector<uint32_t> cm, cb, ce, m0(nm + 1);
    for (int64_t m = 0; m < nm; ++m) {
      m0[m] = (uint32_t)cm.size();
      const uint32_t b = h_model_obs0[m], e = h_model_obs0[m + 1];
      uint32_t x = b;
      do {
        cm.push_back((uint32_t)m);
        cb.push_back(x);
        ce.push_back(std::min(e, x + CH));
        x += CH;
      } while (x < e);
    }
    m0[nm] = (uint32_t)cm.size();
    S.ncost = (int64_t)cm.size();
    S.cost_chunk_model.alloc(S.ncost, s);
    S.cost_chunk_begin.alloc(S.ncost, s);
    S.cost_chunk_end.alloc(S.ncost, s);
    S.model_chunk0.alloc(nm + 1, s);
    check(cudaMemcpyAsync(S.cost_chunk_model, cm.data(), 4 * cm.size(), cudaMemcpyHostToDevice, s), "h2d");
    check(cudaMemcpyAsync(S.cost_chunk_begin, cb.data(), 4 * cb.size(), cudaMemcpyHostToDevice, s), "h2d");
    check(cudaMemcpyAsync(S.cost_chunk_end, ce.data(), 4 * ce.size(), cudaMemcpyHostToDevice, s), "h2d");
    check(cudaMemcpyAsync(S.model_chunk0, m0.data(), 4 * m0.size(), cudaMemcpyHostToDevice, s), "h2d");
    // The host vectors must outlive the copies.
    check(cudaStreamSynchronize(s), "sync");
  }
  S.h_row_ptr.assign(nb + 1, 0);
  if (!S.implicit)
    check(cudaMemcpyAsync(S.h_row_ptr.data(), S.row_ptr, 4 * (nb + 1), cudaMemcpyDeviceToHost, s),
          "d2h");
  uint32_t e = 0;
  check(cudaMemcpyAsync(&e, err, 4, cudaMemcpyDeviceToHost, s), "d2h");
  check(cudaStreamSynchronize(s), "sync");
  if (e & ERR_STRUCTURE) throw std::runtime_error("internal error: reduced-system structure check failed");
}

}  // namespace ba
