// Host driver of the LM loop (ba.rs:198-391) for storage precision R.
#pragma once

#include <map>
#include <mutex>

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <vector>

#include "context.cuh"
#include "pcg.cuh"
#include "pcg_cluster.cuh"
#include "pcg_implicit.cuh"
#include "structure.cuh"

namespace ba {

constexpr size_t kPcgSmemBudget = 96 * 1024;  // dynamic shared memory per PCG CTA

namespace detail {

struct PcgPlan {
  std::vector<PcgJob> jobs;
  std::vector<int32_t> cta_job0;
  int32_t ncta = 0;
};

// Split the block rows of each model over a group of CTAs, a CTA's rows
// over its warps.  Each CTA gets about `rows_target` rows (never more than
// `rows_cap`, its shared-memory row capacity), balanced by blocks (a
// transposed lens row counts one block: its camera blocks are multiplied by
// the camera rows).  Models with more rows get more CTAs.
inline PcgPlan plan_pcg(const Context& ctx, const std::vector<uint32_t>& row_ptr_in,
                        const std::vector<int32_t>& lens_row, int max_ctas, int rows_target,
                        int rows_cap) {
  PcgPlan pl;
  const int64_t nm = ctx.nm;
  std::vector<int64_t> rc(row_ptr_in.size() - 1);  // per-row cost
  {
    std::vector<uint8_t> is_lens(row_ptr_in.size(), 0);
    for (int32_t r : lens_row)
      if (r >= 0) is_lens[r] = 1;
    for (size_t r = 0; r < rc.size(); ++r)
      rc[r] = (is_lens[r] ? 1 : (int64_t)(row_ptr_in[r + 1] - row_ptr_in[r])) + 8;
  }
  std::vector<int64_t> G(nm), rows(nm);
  int64_t tot = 0, need = 0;
  bool all_small = true;
  for (int64_t m = 0; m < nm; ++m) {
    rows[m] = ctx.h_blk0[m + 1] - ctx.h_blk0[m];
    G[m] = std::max<int64_t>(1, (rows[m] + rows_target - 1) / rows_target);
    G[m] = std::max<int64_t>(G[m], (rows[m] + rows_cap - 1) / rows_cap);
    tot += G[m];
    need += std::max<int64_t>(1, (rows[m] + rows_cap - 1) / rows_cap);
    all_small = all_small && rows[m] <= rows_cap;
  }
  max_ctas = std::min(max_ctas, kMaxGroupCtas);
  if (need > max_ctas && !all_small)
    throw CudaError(cudaErrorNotSupported,
                    "PCG plan: the batch needs more resident CTAs than the device holds");
  if (need > max_ctas) {
    // More models than resident CTAs: one CTA per model, dealt greedily to
    // the least-loaded CTA (largest first); a CTA solves its models in turn.
    pl.ncta = max_ctas;
    std::vector<std::vector<int64_t>> lists(max_ctas);
    std::vector<int64_t> load(max_ctas, 0), order(nm);
    for (int64_t m = 0; m < nm; ++m) order[m] = m;
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return rows[a] > rows[b]; });
    for (int64_t m : order) {
      const int64_t c = std::min_element(load.begin(), load.end()) - load.begin();
      lists[c].push_back(m);
      load[c] += rows[m];
    }
    for (int c = 0; c < max_ctas; ++c) {
      pl.cta_job0.push_back((int32_t)pl.jobs.size());
      for (int64_t m : lists[c])
        pl.jobs.push_back(PcgJob{(int32_t)m, 0, 1, c, ctx.h_blk0[m], ctx.h_blk0[m + 1]});
    }
    pl.cta_job0.push_back((int32_t)pl.jobs.size());
    return pl;
  }
  while (tot > max_ctas) {  // shrink the largest groups, keep the row cap
    int64_t best = -1;
    for (int64_t m = 0; m < nm; ++m)
      if (G[m] > (rows[m] + rows_cap - 1) / rows_cap && (best < 0 || G[m] > G[best])) best = m;
    if (best < 0) break;
    --G[best];
    --tot;
  }
  int32_t cta = 0;
  for (int64_t m = 0; m < nm; ++m) {
    const uint32_t r0 = ctx.h_blk0[m], r1 = ctx.h_blk0[m + 1];
    const int64_t g = G[m];
    int64_t total = 0;
    for (uint32_t r = r0; r < r1; ++r) total += rc[r];
    uint32_t row = r0;
    int64_t acc = 0;
    for (int64_t k = 0; k < g; ++k) {
      const uint32_t start = row;
      const int64_t target = (total * (k + 1)) / g;
      const int64_t left_after = (int64_t)(g - k - 1) * rows_cap;
      while (row < r1) {
        const int64_t taken = row - start;
        const int64_t remaining = r1 - row;
        if (taken >= rows_cap) break;
        const bool must = remaining > left_after;  // the rest would not fit
        if (!must && k < g - 1 && acc + rc[row] > target && taken > 0) break;
        acc += rc[row];
        ++row;
      }
      pl.cta_job0.push_back((int32_t)pl.jobs.size());
      pl.jobs.push_back(PcgJob{(int32_t)m, (int32_t)k, (int32_t)g, cta, start, row});
    }
    if (row != r1) throw std::runtime_error("PCG plan left rows unassigned");
    cta += (int32_t)g;
  }
  pl.ncta = cta;
  pl.cta_job0.push_back((int32_t)pl.jobs.size());
  return pl;
}

// Cluster plan (mixed form): every model gets one cluster of `csize` CTAs,
// its block rows split over them balanced by blocks.  row_loc[row] = owning
// rank << 16 | local row.  Returns false if a CTA would exceed the row cap.
struct ClusterPlan {
  std::vector<CgJob> jobs;
  std::vector<uint32_t> row_loc;
  uint32_t max_rows = 0, max_blocks = 0;
};

inline bool plan_cluster(const Context& ctx, const std::vector<uint32_t>& row_ptr,
                         const std::vector<int32_t>& lens_row, int csize, uint32_t rows_cap,
                         ClusterPlan& pl) {
  pl.jobs.clear();
  pl.row_loc.assign(row_ptr.size() - 1, 0);
  pl.max_rows = pl.max_blocks = 0;
  for (int64_t m = 0; m < ctx.nm; ++m) {
    const uint32_t r0 = ctx.h_blk0[m], r1 = ctx.h_blk0[m + 1];
    std::vector<int64_t> rc(r1 - r0);
    int64_t total = 0;
    for (uint32_t r = r0; r < r1; ++r) {
      rc[r - r0] = ((int32_t)r == lens_row[m] ? 1 : (int64_t)(row_ptr[r + 1] - row_ptr[r])) + 8;
      total += rc[r - r0];
    }
    uint32_t row = r0;
    int64_t acc = 0;
    for (int k = 0; k < csize; ++k) {
      const uint32_t start = row;
      const int64_t target = (total * (k + 1)) / csize;
      while (row < r1 && (k == csize - 1 || acc + rc[row - r0] <= target || row == start)) {
        acc += rc[row - r0];
        ++row;
        if (k < csize - 1 && acc >= target) break;
      }
      if (row - start > rows_cap || row - start > 0xffffu) return false;
      for (uint32_t r = start; r < row; ++r) pl.row_loc[r] = ((uint32_t)k << 16) | (r - start);
      pl.jobs.push_back(CgJob{(int32_t)m, start, row});
      pl.max_rows = std::max(pl.max_rows, row - start);
      pl.max_blocks = std::max(pl.max_blocks, row_ptr[row] - row_ptr[start]);
    }
    if (row != r1) return false;
  }
  return true;
}

// Neighbour caches of the cluster PCG: for each CTA the distinct columns its
// rows' blocks multiply (the lens row: its diagonal block only), in order of
// first use; blk_slot[k] = the cache slot of block k's column in its row's
// CTA; per row the (CTA rank << 16 | slot) entries of the caches that hold
// it, which its owner pushes the row's z and p into.  With own_rows false the
// CTA's own columns are not cached (blk_slot = kCgOwnRow | local row: read
// from the row state), for models whose row state leaves little room.
struct CachePlan {
  std::vector<uint32_t> blk_slot, sub_ptr, sub_ent;
  uint32_t cap = 0;
};

inline bool plan_cache(const ClusterPlan& cp, int csize, const std::vector<uint32_t>& row_ptr,
                       const std::vector<uint32_t>& col_idx, const std::vector<uint32_t>& diag_pos,
                       const std::vector<int32_t>& lens_row, int64_t nb, bool own_rows,
                       CachePlan& pl) {
  const std::vector<uint32_t>& row_loc = cp.row_loc;
  pl = CachePlan{};
  pl.blk_slot.assign(std::max<size_t>(col_idx.size(), 1), 0);
  std::vector<std::vector<uint32_t>> subs((size_t)nb);
  std::vector<int64_t> stamp((size_t)nb, -1);
  std::vector<uint32_t> slot_of((size_t)nb, 0);
  for (size_t g = 0; g < cp.jobs.size(); ++g) {
    const CgJob& J = cp.jobs[g];
    const uint32_t rank = (uint32_t)(g % (size_t)csize);
    const int32_t lens = lens_row[J.model];
    uint32_t n = 0;
    for (uint32_t r = J.row0; r < J.row1; ++r) {
      uint32_t b0 = row_ptr[r], b1 = row_ptr[r + 1];
      if ((int32_t)r == lens) b0 = diag_pos[r], b1 = b0 + 1;
      for (uint32_t k = b0; k < b1; ++k) {
        const uint32_t c = col_idx[k];
        if (!own_rows && (row_loc[c] >> 16) == rank) {  // own row: from the row state
          pl.blk_slot[k] = kCgOwnRow | (row_loc[c] & 0xffffu);
          continue;
        }
        if (stamp[c] != (int64_t)g) {
          stamp[c] = (int64_t)g;
          slot_of[c] = n++;
          subs[c].push_back((rank << 16) | slot_of[c]);
        }
        pl.blk_slot[k] = slot_of[c];
      }
    }
    if (n > 0xffffu) return false;
    pl.cap = std::max(pl.cap, n);
  }
  pl.sub_ptr.assign((size_t)nb + 1, 0);
  for (int64_t r = 0; r < nb; ++r) pl.sub_ptr[r + 1] = pl.sub_ptr[r] + (uint32_t)subs[r].size();
  pl.sub_ent.reserve(std::max<size_t>(pl.sub_ptr[nb], 1));
  for (int64_t r = 0; r < nb; ++r) pl.sub_ent.insert(pl.sub_ent.end(), subs[r].begin(), subs[r].end());
  if (pl.sub_ent.empty()) pl.sub_ent.push_back(0);
  return true;
}

// Coarse groups of the two-level preconditioner: each cluster CTA's camera
// rows (the lens row excluded) split into runs of consecutive rows, about 8
// rows each and at most kCoarseMaxGroups per model, so a group lives in one
// CTA.
struct CoarsePlan {
  std::vector<int32_t> grp_row0, grp_row1, grp_model, model_g0, row_grp, job_g0, job_g1;
  std::vector<int32_t> pair_row, pair_grp;  // (camera row, group of its model), row-major
  std::vector<int64_t> model_eoff, row_pair0;
  std::vector<uint32_t> grp_loc;
  uint32_t cap_groups = 0, dmax = 0;
  int64_t e_total = 0;
};

inline void plan_coarse(const Context& ctx, const ClusterPlan& cp,
                        const std::vector<int32_t>& lens_row, int csize, CoarsePlan& pl) {
  pl = CoarsePlan{};
  pl.row_grp.assign((size_t)ctx.nb, -1);
  pl.row_pair0.assign((size_t)ctx.nb, 0);
  constexpr int kPerCtaMax = 4;  // group slots per CTA (shared memory)
  for (int64_t m = 0; m < ctx.nm; ++m) {
    pl.model_g0.push_back((int32_t)pl.grp_row0.size());
    // Camera rows per CTA, then groups: about 8 rows each, at most
    // kCoarseMaxGroups per model shared out in proportion to the rows
    // (at least one for a CTA with camera rows).
    std::vector<int64_t> nrow(csize), ng(csize, 0);
    int64_t total = 0;
    for (int k = 0; k < csize; ++k) {
      const CgJob& J = cp.jobs[(size_t)m * csize + k];
      uint32_t c1 = J.row1;
      if (lens_row[m] >= 0 && (uint32_t)lens_row[m] >= J.row0 && (uint32_t)lens_row[m] < J.row1)
        c1 = (uint32_t)lens_row[m];
      nrow[k] = std::max<int64_t>(0, (int64_t)c1 - (int64_t)J.row0);
      total += nrow[k];
    }
    int64_t want = 0;
    for (int k = 0; k < csize; ++k) {
      ng[k] = nrow[k] > 0 ? std::min<int64_t>(kPerCtaMax, (nrow[k] + 7) / 8) : 0;
      want += ng[k];
    }
    while (want > kCoarseMaxGroups) {  // trim the CTA with the smallest groups
      int best = -1;
      double best_size = 1e300;
      for (int k = 0; k < csize; ++k)
        if (ng[k] > 1 && (double)nrow[k] / ng[k] < best_size)
          best = k, best_size = (double)nrow[k] / ng[k];
      if (best < 0) break;
      --ng[best], --want;
    }
    for (int k = 0; k < csize; ++k) {
      const CgJob& J = cp.jobs[(size_t)m * csize + k];
      const int64_t n = nrow[k];
      const int gk = (int)ng[k];
      pl.job_g0.push_back((int32_t)pl.grp_row0.size());
      for (int q = 0; q < gk; ++q) {
        const int32_t a = (int32_t)(J.row0 + n * q / gk), b = (int32_t)(J.row0 + n * (q + 1) / gk);
        const int32_t g = (int32_t)pl.grp_row0.size();
        pl.grp_row0.push_back(a), pl.grp_row1.push_back(b), pl.grp_model.push_back((int32_t)m);
        pl.grp_loc.push_back(((uint32_t)k << 16) | (uint32_t)q);
        for (int32_t r = a; r < b; ++r) pl.row_grp[r] = g;
      }
      pl.job_g1.push_back((int32_t)pl.grp_row0.size());
      pl.cap_groups = std::max(pl.cap_groups, (uint32_t)gk);
    }
    (void)total;
    const int32_t mg0 = pl.model_g0.back(), mg1 = (int32_t)pl.grp_row0.size();
    for (int32_t g = mg0; g < mg1; ++g)
      for (int32_t r = pl.grp_row0[g]; r < pl.grp_row1[g]; ++r) {
        pl.row_pair0[r] = (int64_t)pl.pair_row.size();
        for (int32_t h = mg0; h < mg1; ++h) pl.pair_row.push_back(r), pl.pair_grp.push_back(h);
      }
    const int64_t D = kCoarseModes * ((int64_t)pl.grp_row0.size() - pl.model_g0.back());
    pl.model_eoff.push_back(pl.e_total);
    pl.e_total += D * D;
    pl.dmax = std::max(pl.dmax, (uint32_t)D);
  }
  pl.model_g0.push_back((int32_t)pl.grp_row0.size());
}

template <typename T>
void h2d(DevBuf<T>& d, const std::vector<T>& h, cudaStream_t s) {
  d.alloc(h.size(), s);
  if (!h.empty())
    check(cudaMemcpyAsync(d.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s), "h2d");
}

inline int64_t at_least_1(int64_t n) { return n > 0 ? n : 1; }

// The cluster PCG kernel for the coarse flag and the threads per CTA.
using CgKernel = void (*)(CgArgs);
inline CgKernel cg_kernel(bool coarse, int threads) {
  if (threads == kCgThreadsWide)
    return coarse ? pcg_cluster_kernel<true, kCgThreadsWide>
                  : pcg_cluster_kernel<false, kCgThreadsWide>;
  return coarse ? pcg_cluster_kernel<true, kCgThreads> : pcg_cluster_kernel<false, kCgThreads>;
}

}  // namespace detail

// CUDA-event timing of kernel phases (only when profiling is asked for).
struct PhaseTimer {
  bool on = false;
  cudaStream_t s = nullptr;
  std::vector<std::pair<int, cudaEvent_t>> marks;  // (phase that ends here, event)
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  cudaEvent_t get() {
    if (used == pool.size()) {
      cudaEvent_t e;
      check(cudaEventCreate(&e), "event");
      pool.push_back(e);
    }
    return pool[used++];
  }
  void mark(int phase) {  // phase < 0: start mark
    if (!on) return;
    cudaEvent_t e = get();
    check(cudaEventRecord(e, s), "event record");
    marks.push_back({phase, e});
  }
  // Accumulate the elapsed times of completed marks (the stream is synced).
  void flush(double* ms, int64_t* n) {
    for (size_t i = 1; i < marks.size(); ++i) {
      if (marks[i].first < 0) continue;
      float t = 0;
      check(cudaEventElapsedTime(&t, marks[i - 1].second, marks[i].second), "elapsed");
      ms[marks[i].first] += t;
      n[marks[i].first] += 1;
    }
    marks.clear();
    used = 0;
  }
  ~PhaseTimer() {
    for (auto e : pool) cudaEventDestroy(e);
  }
};

// CUDA graph of one LM iteration, captured from the engine's stream on first
// use.  If the stream cannot be captured (the legacy default stream, or a
// capture error), the engine launches the kernels directly.
struct IterationGraph {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t kernels = 0;  // kernel nodes, counted into the launch statistics
  bool tried = false;

  template <typename Engine>
  bool ok(Engine* e) {
    if (tried) return exec != nullptr;
    tried = true;
    cudaStream_t s = e->s;
    if (s == nullptr || s == cudaStreamLegacy || s == cudaStreamPerThread) return false;
    const int64_t l0 = g_launches;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    bool captured = true;
    try {
      e->iteration();
    } catch (...) {
      captured = false;
    }
    cudaGraph_t gr = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(s, &gr);
    g_launches = l0;
    if (!captured || ce != cudaSuccess || gr == nullptr) {
      cudaGetLastError();
      if (gr) cudaGraphDestroy(gr);
      return false;
    }
    if (cudaGraphInstantiate(&exec, gr, 0) != cudaSuccess) {
      cudaGetLastError();
      cudaGraphDestroy(gr);
      exec = nullptr;
      return false;
    }
    g = gr;
    size_t n = 0;
    check(cudaGraphGetNodes(g, nullptr, &n), "graph nodes");
    std::vector<cudaGraphNode_t> nodes(n);
    check(cudaGraphGetNodes(g, nodes.data(), &n), "graph nodes");
    for (cudaGraphNode_t nd : nodes) {
      cudaGraphNodeType t;
      check(cudaGraphNodeGetType(nd, &t), "graph node type");
      if (t == cudaGraphNodeTypeKernel) ++kernels;
    }
    return true;
  }
  void launch(cudaStream_t s) {
    check(cudaGraphLaunch(exec, s), "graph launch");
    g_launches += kernels;
  }
  ~IterationGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (g) cudaGraphDestroy(g);
  }
};

// Autotuner results shared by the contexts of the process (ba_solve makes a
// context per call): keyed by form, coarse correction and the shape of the
// reduced system, so repeated calls on problems of one shape tune once.
struct TuneKey {
  int form, coarse;
  int64_t nm, nb, nz;
  bool operator<(const TuneKey& o) const {
    if (form != o.form) return form < o.form;
    if (coarse != o.coarse) return coarse < o.coarse;
    if (nm != o.nm) return nm < o.nm;
    if (nb != o.nb) return nb < o.nb;
    return nz < o.nz;
  }
};
inline std::mutex& tune_mutex() {
  static std::mutex m;
  return m;
}
inline std::map<TuneKey, PcgTuning>& tune_cache() {
  static std::map<TuneKey, PcgTuning> c;
  return c;
}

// All device state of one solve: structure, per-iteration buffers, LM
// control scalars and the PCG plan.
template <typename R>
struct LmEngine {
  Context& ctx;
  const Opts& o;
  cudaStream_t s;
  Prob P;
  StructBufs SB;
  StructView SV;
  DevBuf<R> lin, gsub, Z, Zl, S, pre, g, x, z, p;
  DevBuf<double> ptL, ptzv, part;
  DevBuf<uint8_t> kept;
  DevBuf<float> ptf, camf, obs_u;  // mixed form only
  // Mixed form's per-observation passes (ba_options.point_kernel numbering:
  // 1 three kernels, 2 / 3 fused over 128- / 256-observation chunks) and the
  // first point of every chunk of the fused kernel.
  int point_variant = 0;
  DevBuf<uint32_t> fu_p0;
  int64_t fu_chunks = 0;
  // Per model: 1 if the stored records are not at the current state (the
  // trial cost forms the trial state's records; see cost_record_kernel).
  DevBuf<int32_t> rec_stale;
  // Mixed form, J^T J recomputed in the matrix-free PCG (no Schur factors
  // stored): where the factors are recomputed from.
  bool z_recompute = false;
  ZSource zsrc{};
  DevBuf<double> camU, camgj, camgs, camX, caml, grpU, grpg, cost_part;
  IterBufs<R> B{};
  DevBuf<double> lambda, cost, new_cost, rms, sq, sigma;
  DevBuf<int64_t> n_front, pcg_total;
  DevBuf<int32_t> active, accepted, iters, pcg_iters, any, small, pcg_cap;
  DevBuf<double> log_cost, log_lam;
  DevBuf<int32_t> log_pcg, log_acc;
  int32_t log_cap = 0;
  int32_t pcg_limit = 0;  // PCG launch limit: the larger of the two caps
  Control C{};
  detail::PcgPlan plan;
  DevBuf<PcgJob> jobs;
  DevBuf<int32_t> cta_job0;
  DevBuf<unsigned long long> bar, bar_base;
  DevBuf<double> pcg_part;
  DevBuf<int32_t> lens_row, lens_pos;
  uint32_t smem_rows = 0, smem_blocks = 0;
  uint32_t sub_len = kSubLen;  // Schur pairs per warp sub-segment
  DevBuf<uint32_t> fold_slots, sub_end;  // blocks folded before assembly
  uint32_t n_fold = 0;
  size_t smem_bytes = 0;
  int pcg_rows_target = 0, grid_rows_target = 0, max_ctas = 0;
  std::vector<int32_t> h_lens;
  PcgArgs<R> pa{};
  // Matrix-free PCG.
  bool implicit = false;
  DevBuf<R> own, tbuf, rbuf, qbuf;
  DevBuf<double> lens_part;
  ImpArgs<R> ia{};
  int32_t imp_ncta = 0;
  // Cluster-resident PCG (mixed form).
  bool use_cluster = false;
  int cl_size = 0;
  int cl_threads = kCgThreads;  // threads per CTA of the cluster kernel
  DevBuf<CgJob> cg_jobs;
  DevBuf<uint32_t> cg_loc, cg_slot, cg_subp, cg_sube;
  std::vector<uint32_t> h_col_idx, h_diag_pos;  // host copies for the cache plan
  CgArgs ca{};
  size_t cg_smem = 0;
  // Two-level preconditioner (mixed form, cluster kernel).
  bool use_coarse = false;
  DevBuf<float> cW, cE, cEinv;
  DevBuf<double> cW64;
  DevBuf<int32_t> c_grp_row0, c_grp_row1, c_grp_model, c_model_g0, c_row_grp, c_job_g0, c_job_g1;
  DevBuf<int64_t> c_model_eoff, c_row_pair0;
  DevBuf<uint32_t> c_grp_loc;
  DevBuf<int32_t> c_pair_row, c_pair_grp;
  DevBuf<double> c_P, c_S64;
  int64_t c_npairs = 0;
  CoarseArgs cargs{};
  int32_t c_ngroups = 0;
  // The coarse setup (basis, W^T S W, its inverse) runs on a second stream:
  // the basis, which reads only the state, beside the point passes (forked
  // at the start of the iteration), the rest beside the right-hand side and
  // block-Jacobi kernels (forked after the assembly), joined before the PCG;
  // coarse_pending: forked, not joined; basis_forked: this iteration's basis
  // is on the side stream.
  cudaStream_t s2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // The camera sums run on the second stream beside the Schur sums.
  cudaEvent_t ev_cam = nullptr, ev_cam_join = nullptr;
  bool coarse_pending = false, basis_forked = false;
  PhaseTimer T;

  LmEngine(Context& c, const Opts& opts) : ctx(c), o(opts), s(c.stream) {
    T.on = o.profile != 0;
    T.s = s;
    for (int k = 0; k < kPhases; ++k) ctx.phase_ms[k] = 0, ctx.phase_n[k] = 0;
  }
  ~LmEngine() {
    if (s2) cudaStreamSynchronize(s2);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (ev_cam) cudaEventDestroy(ev_cam);
    if (ev_cam_join) cudaEventDestroy(ev_cam_join);
    if (s2) cudaStreamDestroy(s2);
  }
  LmEngine(const LmEngine&) = delete;
  LmEngine& operator=(const LmEngine&) = delete;

  // The stream s waits for the forked coarse setup (before the PCG reads it,
  // and before anything it uses is planned or freed again).
  void join_coarse() {
    if (!coarse_pending) return;
    check(cudaStreamWaitEvent(s, ev_join, 0), "join");
    coarse_pending = false;
  }

  // Coarse setup of the two-level PCG on stream st (basis: W as well).
  void launch_coarse_chain(cudaStream_t st, bool basis = true) {
    if (basis)
      BA_LAUNCH(coarse_basis_kernel<<<grid_for((int64_t)c_ngroups * 32, 128), 128, 0, st>>>(
          P, ctx.cur(), cargs));
    if (c_npairs > 0)
      BA_LAUNCH(coarse_rowgroup_kernel<<<grid_for(c_npairs * 32, kCoarseMatThreads),
                                         kCoarseMatThreads, 0, st>>>(SV, c_S64.p, cargs, c_npairs,
                                                                     c_pair_row, c_pair_grp, c_P));
    BA_LAUNCH(coarse_sum_kernel<<<dim3((unsigned)c_ngroups, 6), 224, 0, st>>>(cargs, c_row_pair0,
                                                                         c_P));
    check(cudaFuncSetAttribute(coarse_invert_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)kInvSmemBytes),
          "coarse inverse shared memory");
    BA_LAUNCH(coarse_invert_kernel<<<(unsigned)ctx.nm, kInvThreads, kInvSmemBytes, st>>>(cargs));
  }

  bool coarse_on() const { return use_cluster && use_coarse && c_ngroups > 0; }
  void side_stream() {
    if (s2) return;
    check(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking), "side stream");
    check(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming), "event");
    check(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming), "event");
    check(cudaEventCreateWithFlags(&ev_cam, cudaEventDisableTiming), "event");
    check(cudaEventCreateWithFlags(&ev_cam_join, cudaEventDisableTiming), "event");
  }

  // At the start of an iteration: fork the coarse basis onto the second
  // stream (it runs beside the point passes).
  void fork_coarse_basis() {
    if (!coarse_on()) return;
    join_coarse();
    side_stream();
    check(cudaEventRecord(ev_fork, s), "fork");
    check(cudaStreamWaitEvent(s2, ev_fork, 0), "fork");
    BA_LAUNCH(coarse_basis_kernel<<<grid_for((int64_t)c_ngroups * 32, 128), 128, 0, s2>>>(
        P, ctx.cur(), cargs));
    check(cudaEventRecord(ev_join, s2), "join");
    coarse_pending = true;
    basis_forked = true;
  }

  // After the assembly: fork the rest of the coarse setup onto the second
  // stream (the basis too unless it was forked at the start).
  void fork_coarse() {
    if (!coarse_on()) return;
    join_coarse();  // the basis, finished long before
    side_stream();
    check(cudaEventRecord(ev_fork, s), "fork");
    check(cudaStreamWaitEvent(s2, ev_fork, 0), "fork");
    launch_coarse_chain(s2, !basis_forked);
    basis_forked = false;
    check(cudaEventRecord(ev_join, s2), "join");
    coarse_pending = true;
  }

  void setup() {
    using detail::at_least_1;
    const int64_t nc = ctx.nc, np = ctx.np, no = ctx.no, ng = ctx.ng, nb = ctx.nb, nm = ctx.nm;
    reset_states(ctx);
    P = ctx.prob(o.loss);
    // Matrix-free PCG (no pair list, no reduced matrix): when asked for, or in
    // auto mode when the explicit layout would exceed the memory cap.  One
    // model with at most one lens group.
    const bool mf_ok = nm == 1 && ng <= 1;
    const bool mf_forced = o.matrix_free == 2 || o.matrix_free == 3;
    if (mf_forced && !mf_ok)
      throw CudaError(cudaErrorNotSupported,
                      "matrix-free PCG: one model with at most one lens group per call");
    if (o.matrix_free == 3 && sizeof(R) == 8)
      throw CudaError(cudaErrorNotSupported,
                      "J^T J recompute in the PCG: the mixed form (FP32 Jacobians) only");
    const int64_t cap = mf_forced ? 0
                        : (o.matrix_free == 0 && mf_ok && o.memory_cap > 0) ? o.memory_cap
                                                                            : -1;
    // Mixed form: Schur factors stored camera-major (the Schur kernel's
    // gathers of a destination block then walk two camera segments).
    build_structure(P, ctx.h_obs0, SB, ctx.err, s, cap, sizeof(R) == 4);
    implicit = SB.implicit;
    ctx.last_matrix_free = implicit;
    sub_len = kSubLen;
    ctx.last_sub_len = implicit ? 0 : (int32_t)sub_len;
    plan_fold();
    SV = SB.view();
    ctx.last_nz = SB.nz, ctx.last_pairs = SB.npairs - nb, ctx.last_nl = SB.nl;
    lin.alloc(at_least_1(no) * kLinW, s), gsub.alloc(at_least_1(no) * 9, s);
    // Schur factors: 24 values per record when stored camera-major (the
    // mixed form with a pair list), else 18; 4 values of padding after the
    // last record for the 16-byte loads of 18-value FP32 records.  The mixed
    // form's J^T J-recompute mode stores none (they are recomputed where used).
    const bool z24 = sizeof(R) == 4 && SB.z_by_camera;
    z_recompute = sizeof(R) == 4 && implicit && o.matrix_free == 3;
    if (z_recompute)
      Z.release();
    else
      Z.alloc(at_least_1(no) * (z24 ? 24 : 18) + 4, s);
    Zl.alloc(at_least_1(SB.nl) * 9, s);
    ptL.alloc(at_least_1(np) * 6, s), ptzv.alloc(at_least_1(np) * 3, s);
    kept.alloc(at_least_1(np), s);
    camU.alloc(at_least_1(nc) * 21, s), camgj.alloc(at_least_1(nc) * 6, s);
    camgs.alloc(at_least_1(nc) * 6, s), camX.alloc(at_least_1(nc) * 18, s);
    caml.alloc(at_least_1(nc) * 12, s), grpU.alloc(at_least_1(ng) * 6, s);
    grpg.alloc(at_least_1(ng) * 3, s);
    part.alloc(at_least_1(SB.nsub) * 36, s), S.alloc(at_least_1(SB.nz) * 36, s);
    if (implicit) {
      own.alloc(at_least_1(nb) * 36, s), tbuf.alloc(at_least_1(np) * 3, s);
      lens_part.alloc(9 * kLensChunks, s);
      rbuf.alloc(at_least_1(nb) * 6, s), qbuf.alloc(at_least_1(nb) * 6, s);
    }
    pre.alloc(at_least_1(nb) * 36, s);
    g.alloc(at_least_1(nb) * 6, s), x.alloc(at_least_1(nb) * 6, s);
    z.alloc(at_least_1(nb) * 6, s), p.alloc(at_least_1(nb) * 12, s);
    cost_part.alloc(at_least_1(SB.ncost) * 3, s);
    // Camera sums are read for every camera, including ones without observations.
    camU.zero(), camgj.zero(), camgs.zero(), camX.zero(), caml.zero(), grpU.zero(), grpg.zero();
    x.zero();
    if (sizeof(R) == 4) {
      ptf.alloc(at_least_1(np) * 9, s), camf.alloc(at_least_1(nc) * kCamF, s);
      obs_u.alloc(at_least_1(no) * 3, s);
    }
    // Two-level PCG (mixed form): the FP64 values of S for the coarse matrix,
    // written by every assembly (the autotuner assembles before it plans).
    if (sizeof(R) == 4 && o.coarse && !implicit) c_S64.alloc(at_least_1(SB.nz) * 36, s);
    B = IterBufs<R>{lin, gsub, Z, Zl, ptL, ptzv, kept, camU, camgj, camgs, camX, caml,
                    grpU, grpg, part, S, pre, g, x, cost_part, ptf.p};
    B.zpos = sizeof(R) == 4 && SB.z_by_camera ? SB.cam_pos.p : nullptr;
    B.zpitch = B.zpos ? 24 : 18;
    B.Z = z_recompute ? nullptr : Z.p;
    lambda.alloc(nm, s), cost.alloc(nm, s), new_cost.alloc(nm, s), rms.alloc(nm, s);
    sq.alloc(nm, s), sigma.alloc(nm, s), n_front.alloc(nm, s), pcg_total.alloc(nm, s);
    if constexpr (sizeof(R) == 4)
      zsrc = ZSource{P, ctx.cur(), lin.p, ptf.p, ptL.p, kept.p, sigma.p};
    active.alloc(nm, s), accepted.alloc(nm, s), iters.alloc(nm, s), pcg_iters.alloc(nm, s);
    any.alloc(1, s);
    log_cap = o.log ? std::max(0, o.log->cap) : 0;
    log_cost.alloc(std::max(log_cap, 1), s), log_lam.alloc(std::max(log_cap, 1), s);
    log_pcg.alloc(std::max(log_cap, 1), s), log_acc.alloc(std::max(log_cap, 1), s);
    set_lambda(1e-4);  // ba.rs:217
    {
      std::vector<double> sg(nm, o.sigma);
      std::vector<int32_t> act(nm, o.max_iter > 0 ? 1 : 0);
      check(cudaMemcpyAsync(sigma.p, sg.data(), 8 * nm, cudaMemcpyHostToDevice, s), "h2d");
      check(cudaMemcpyAsync(active.p, act.data(), 4 * nm, cudaMemcpyHostToDevice, s), "h2d");
      accepted.zero(), iters.zero(), pcg_iters.zero(), pcg_total.zero();
      check(cudaStreamSynchronize(s), "sync");
    }
    small.alloc(nm, s);
    small.zero();
    // PCG iteration cap per model: pcg_max_iter, raised to pcg_end_max_iter by
    // the control kernel in the end game; the kernels take the smaller of it
    // and their launch limit (which the autotuner lowers for its trials).
    pcg_limit = std::max(o.pcg_max_iter, o.pcg_end_max_iter);
    pcg_cap.alloc(nm, s);
    {
      std::vector<int32_t> cap(nm, o.pcg_max_iter);
      check(cudaMemcpyAsync(pcg_cap.p, cap.data(), 4 * nm, cudaMemcpyHostToDevice, s), "h2d");
      check(cudaStreamSynchronize(s), "sync");
    }
    const int32_t patience = o.stop_patience > 0 ? o.stop_patience : 1;
    C = Control{lambda, cost, new_cost, rms, sq, n_front, active, accepted, iters, pcg_iters,
                pcg_total, any, sigma, small, patience, o.max_iter, pcg_cap,
                o.pcg_end_max_iter, o.pcg_end_rel, log_cap, log_cost, log_lam, log_pcg, log_acc};
    if constexpr (sizeof(R) == 4) {
      rec_stale.alloc(nm, s);
      mark_records_stale();
      C.rec_stale = rec_stale.p;
    }
    // PCG: shared memory per grid-kernel CTA (a fixed budget) holds row state
    // for up to smem_rows rows, then as many S blocks as fit.  A large batch
    // needs more rows per CTA: all CTAs of the cooperative launch must be
    // resident at once.
    check(cudaFuncSetAttribute(pcg_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)kPcgSmemBudget),
          "pcg smem");
    int occ = 0;
    check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pcg_kernel<R>, kPcgThreads,
                                                        kPcgSmemBudget),
          "occupancy");
    max_ctas = std::min(std::max(1, occ) * ctx.n_sm, kMaxGroupCtas);
    const size_t row_bytes = kRowState * sizeof(R) + 12;
    const int64_t rows_fit = (int64_t)(kPcgSmemBudget / row_bytes);
    const int64_t rows_need = (nb * 5 / 4 + max_ctas - 1) / max_ctas + 8;
    smem_rows = (uint32_t)std::min<int64_t>(rows_fit, std::max<int64_t>(64, rows_need));
    smem_blocks = (uint32_t)((kPcgSmemBudget - (size_t)smem_rows * row_bytes) / (36 * sizeof(R) + 4));
    smem_bytes = pcg_smem_bytes<R>(smem_rows, smem_blocks);
    h_lens.assign(nm, -1);
    for (int64_t m = 0; m < nm; ++m)
      if (ctx.h_grp0[m + 1] - ctx.h_grp0[m] == 1)
        h_lens[m] = (int32_t)(ctx.h_blk0[m] + (ctx.h_cam0[m + 1] - ctx.h_cam0[m]));
    detail::h2d(lens_row, h_lens, s);
    lens_pos.alloc(detail::at_least_1(nb), s);
    bar.alloc(nm, s);
    bar_base.alloc(nm, s);
    if (implicit) {
      choose_point_variant();
      setup_implicit();
      return;
    }
    if (nb > 0)
      BA_LAUNCH(lens_pos_kernel<<<grid_for(nb, 256), 256, 0, s>>>(nb, SB.row_ptr, SB.col_idx,
                                                                 P.blk_model, lens_row, lens_pos));
    if (sizeof(R) == 8 && (o.pcg_kernel == 2 || o.pcg_kernel == 3))
      throw CudaError(cudaErrorNotSupported, "cluster PCG: the FP64 form uses the grid kernel");
    // Configuration: an earlier tuning of this context for this form, or the
    // defaults (FP64 instructions serialise per SM sub-partition: one row per
    // warp on four warps; FP32 rows are cheap: one per warp on all eight).
    PcgTuning& tu = ctx.tuning[sizeof(R) == 8 ? 0 : 1];
    if (!tu.valid && o.autotune && o.pcg_kernel == 0) {
      std::lock_guard<std::mutex> lk(tune_mutex());
      auto it = tune_cache().find(tune_key());
      if (it != tune_cache().end()) tu = it->second;
    }
    if (tu.valid && tu.sub_len > 0) set_sub_len((uint32_t)tu.sub_len);
    choose_point_variant();
    if (tu.valid && o.pcg_kernel == 0) {
      if (tu.kernel != 2 || !try_cluster(tu.cluster, false, true, tu.cg_threads))
        plan_grid(tu.rows_target);
    } else if (o.pcg_kernel == 2 || o.pcg_kernel == 3) {
      try_cluster(0, true, false, o.pcg_kernel == 3 ? kCgThreadsWide : kCgThreads);
    } else if (sizeof(R) == 4 && o.pcg_kernel == 0 && try_cluster(0, false)) {
      // mixed form: the cluster kernel when every model fits
    } else {
      plan_grid(pcg_rows_target > 0 ? pcg_rows_target : (sizeof(R) == 8 ? 4 : 8));
    }
  }

  // The mixed form's per-observation passes: the option, else this form's
  // tuning (of this context or of the problem shape in this process), else
  // the three kernels (measured fastest on the 500-camera survey: the fused
  // kernel's point pass runs a thread per point on the few points of a
  // chunk, and this GPU's FP64 warp instructions cost the same however few
  // lanes are active).
  void choose_point_variant() {
    if constexpr (sizeof(R) == 8) return;
    int v = o.point_kernel;
    if (v == 0) {
      PcgTuning tu = ctx.tuning[1];
      if (!tu.valid && o.autotune) {
        std::lock_guard<std::mutex> lk(tune_mutex());
        auto it = tune_cache().find(tune_key());
        if (it != tune_cache().end()) tu = it->second;
      }
      v = tu.valid && tu.point_kernel > 0 ? tu.point_kernel : 1;
    }
    set_point_variant(v);
  }

  void set_point_variant(int v) {
    if constexpr (sizeof(R) == 8) return;
    point_variant = v;
    ctx.last_point_kernel = v;
    if (v == 1) return;
    const int64_t chunk = v == 2 ? 128 : 256;
    fu_chunks = std::max<int64_t>(1, (ctx.no + chunk - 1) / chunk);
    fu_p0.alloc(fu_chunks + 1, s);
    BA_LAUNCH(chunk_points_kernel<<<grid_for(std::max<int64_t>(ctx.np, 1), 256), 256, 0, s>>>(
        ctx.np, SB.pt_ptr, (uint32_t)chunk, fu_chunks, fu_p0));
  }

  void mark_records_stale() {
    std::vector<int32_t> one(ctx.nm, 1);
    check(cudaMemcpyAsync(rec_stale.p, one.data(), 4 * ctx.nm, cudaMemcpyHostToDevice, s), "h2d");
    check(cudaStreamSynchronize(s), "sync");
  }

  // The mixed form's per-observation passes at the current state.
  void point_passes(const StateView& cur) {
    if (point_variant == 1) {
      if (ctx.no > 0)
        BA_LAUNCH(obs_record_kernel<<<grid_for(ctx.no, kObsThreads), kObsThreads, 0, s>>>(
            P, cur, B, camf, active, sigma, rec_stale.p));
      BA_LAUNCH(point_solve_mixed_kernel<<<grid_for(ctx.np, kPtSolveThreads), kPtSolveThreads, 0,
                                           s>>>(P, cur, SV, B, active, lambda, sigma));
      if (ctx.no > 0)
        BA_LAUNCH(obs_factor_kernel<<<grid_for(ctx.no, kObsThreads), kObsThreads, 0, s>>>(
            P, B, active));
    } else if (point_variant == 2) {
      launch_fused<128>(cur);
    } else {
      launch_fused<256>(cur);
    }
  }

  template <int kChunk>
  void launch_fused(const StateView& cur) {
    using F = FusedPoint<kChunk>;
    check(cudaFuncSetAttribute(point_fused_mixed_kernel<kChunk>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)F::kSmem),
          "fused point shared memory");
    BA_LAUNCH(point_fused_mixed_kernel<kChunk><<<(unsigned)fu_chunks, F::kThreads, F::kSmem, s>>>(
        P, cur, SV, B, camf, fu_p0, active, lambda, sigma, rec_stale.p));
  }

  // Schur sub-segments of at most L pairs (a warp each): rebuilt from the
  // pair list, with the partial-sum buffer they write.
  void set_sub_len(uint32_t L) {
    if (implicit || SB.ns == 0 || L == sub_len) return;
    build_subsegments(SB, L, s);
    part.alloc(detail::at_least_1(SB.nsub) * 36, s);
    SV = SB.view();
    B.part = part;
    sub_len = L;
    ctx.last_sub_len = (int32_t)L;
    plan_fold();
  }

  // Blocks with more than kFoldMin sub-segments, folded by schur_fold_kernel
  // before assembly, and every block's effective end of sub-segments.
  void plan_fold() {
    n_fold = 0;
    if (implicit || SB.ns == 0) return;
    std::vector<uint32_t> ptr((size_t)SB.ns + 1);
    check(cudaMemcpyAsync(ptr.data(), SB.slot_sub_ptr.p, 4 * ptr.size(), cudaMemcpyDeviceToHost, s),
          "d2h");
    check(cudaStreamSynchronize(s), "sync");
    std::vector<uint32_t> fs, end((size_t)SB.ns);
    for (int64_t k = 0; k < SB.ns; ++k) {
      const bool fold = ptr[k + 1] - ptr[k] > kFoldMin;
      if (fold) fs.push_back((uint32_t)k);
      end[k] = fold ? ptr[k] + 1 : ptr[k + 1];
    }
    n_fold = (uint32_t)fs.size();
    if (fs.empty()) fs.push_back(0);
    detail::h2d(fold_slots, fs, s);
    detail::h2d(sub_end, end, s);
    check(cudaStreamSynchronize(s), "sync");
  }

  // The matrix-free PCG kernel: Schur factors stored or recomputed.
  void (*implicit_kernel())(ImpArgs<R>) {
    return z_recompute ? pcg_implicit_kernel<R, true> : pcg_implicit_kernel<R, false>;
  }

  // Matrix-free PCG: one cooperative launch over every SM, one group.
  void setup_implicit() {
    join_coarse();
    use_cluster = false;
    use_coarse = false;
    ctx.last_coarse_dim = 0;
    int occ = 0;
    check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, implicit_kernel(), kPcgThreads, 0),
          "occupancy");
    imp_ncta = std::min(std::max(1, occ) * ctx.n_sm, kMaxGroupCtas);
    bar.zero();
    bar_base.zero();
    pcg_part.alloc(kParts * (size_t)imp_ncta, s);
    ia = ImpArgs<R>{bar, bar_base, pcg_part, imp_ncta, ctx.err, P, SV, B.Z, Zl, kept, own, camX,
                    pre, g, x, rbuf, z, p, qbuf, tbuf, h_lens[0], (int32_t)ctx.nb, pcg_iters,
                    pcg_limit, o.pcg_tol, o.wait_limit};
    ia.cap = pcg_cap;
    ia.zsrc = zsrc;
    ctx.last_pcg_kernel = 3, ctx.last_pcg_cluster = 0, ctx.last_pcg_ctas = imp_ncta;
    ctx.last_pcg_threads = kPcgThreads;
  }

  // Grid kernel plan: about rows_target block rows per CTA.
  void plan_grid(int rows_target) {
    join_coarse();
    use_cluster = false;
    use_coarse = false;
    ctx.last_coarse_dim = 0;
    plan = detail::plan_pcg(ctx, SB.h_row_ptr, h_lens, max_ctas, rows_target, (int)smem_rows);
    detail::h2d(jobs, plan.jobs, s);
    detail::h2d(cta_job0, plan.cta_job0, s);
    bar.zero();
    bar_base.zero();
    pcg_part.alloc(kParts * (size_t)plan.ncta, s);
    check(cudaStreamSynchronize(s), "sync");  // host plan vectors
    pa = PcgArgs<R>{jobs, cta_job0, bar, bar_base, pcg_part, plan.ncta, SB.row_ptr, SB.col_idx,
                    S, pre, g, x, z, p, ctx.nb, lens_row, lens_pos, SB.diag_pos, smem_rows,
                    smem_blocks, active, pcg_iters, pcg_limit, o.pcg_tol, ctx.err,
                    o.wait_limit, o.hold_cta};
    pa.cap = pcg_cap;
    grid_rows_target = rows_target;
    ctx.last_pcg_kernel = 1, ctx.last_pcg_cluster = 0, ctx.last_pcg_ctas = plan.ncta;
    ctx.last_pcg_threads = kPcgThreads;
  }

  // Mixed form: one cluster of `csize` CTAs (0: by size, up to 16) per model
  // with the whole PCG in distributed shared memory.  Returns false (or throws
  // BA_NOT_SUPPORTED when `required`) if a model does not fit.
  bool try_cluster(int csize_req, bool required, bool prefer_cluster = false,
                   int threads = kCgThreads) {
    join_coarse();
    if constexpr (sizeof(R) == 8) return false;
    auto unusable = [&](const std::string& why) {
      if (required) throw CudaError(cudaErrorNotSupported, "cluster PCG: " + why);
      return false;
    };
    int64_t max_rows = 0;
    for (int64_t m = 0; m < ctx.nm; ++m)
      max_rows = std::max<int64_t>(max_rows, ctx.h_blk0[m + 1] - ctx.h_blk0[m]);
    const int csize = csize_req > 0 ? std::min(csize_req, kCgMaxCluster)
                                    : (int)std::min<int64_t>(kCgMaxCluster,
                                                             std::max<int64_t>(1, (max_rows + 31) / 32));
    int smem_optin = 0;
    check(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx.device),
          "attr");
    const bool coarse = o.coarse != 0;
    if (threads != kCgThreadsWide) threads = kCgThreads;
    const detail::CgKernel kfn = detail::cg_kernel(coarse, threads);
    cudaFuncAttributes fa{};
    check(cudaFuncGetAttributes(&fa, kfn), "func attr");
    const size_t avail = (size_t)smem_optin - fa.sharedSizeBytes;
    // Row state takes at most half of the shared memory (the rest caches S
    // blocks); with the coarse correction, which needs far fewer PCG
    // iterations, rows may take all of it and S is read from L2.
    const size_t row_all = (size_t)kCgRow * 4 + (coarse ? (size_t)kCgCoarseRowF * 4 : 0);
    const size_t coarse_fixed = coarse ? cg_coarse_fixed_floats(4, kCoarseMaxDim) * 4 : 0;
    const uint32_t rows_cap =
        (uint32_t)std::min<size_t>(coarse ? (avail - coarse_fixed) / row_all : avail / 2 / (kCgRow * 4), 4096);
    detail::ClusterPlan cp;
    if (!detail::plan_cluster(ctx, SB.h_row_ptr, h_lens, csize, rows_cap, cp))
      return unusable("a model has too many block rows for one cluster");
    if (cp.max_blocks == 0 && cp.max_rows == 0) return unusable("empty plan");
    detail::CoarsePlan gp;
    size_t coarse_bytes = 0;
    if (coarse) {
      detail::plan_coarse(ctx, cp, h_lens, csize, gp);
      coarse_bytes = cg_coarse_smem_bytes(cp.max_rows, std::max(gp.cap_groups, 1u), std::max(gp.dmax, 1u));
    }
    if (h_col_idx.empty() && SB.nz > 0) {
      h_col_idx.resize((size_t)SB.nz);
      h_diag_pos.resize((size_t)ctx.nb);
      check(cudaMemcpyAsync(h_col_idx.data(), SB.col_idx.p, 4 * (size_t)SB.nz,
                            cudaMemcpyDeviceToHost, s), "d2h");
      check(cudaMemcpyAsync(h_diag_pos.data(), SB.diag_pos.p, 4 * (size_t)ctx.nb,
                            cudaMemcpyDeviceToHost, s), "d2h");
      check(cudaStreamSynchronize(s), "sync");
    }
    // Own rows in the cache too (vector loads, uniform reads) when it fits,
    // else from the row state.
    // Own rows in the cache too (vector loads) when that leaves room for a
    // quarter of the S blocks; else only other CTAs' rows (S blocks that do
    // not fit are read from L2).
    detail::CachePlan kp;
    const size_t row_bytes = (size_t)cp.max_rows * kCgRow * 4;
    if (!detail::plan_cache(cp, csize, SB.h_row_ptr, h_col_idx, h_diag_pos, h_lens, ctx.nb, true,
                            kp))
      return unusable("a CTA's neighbour cache exceeds 65,535 rows");
    if (row_bytes + coarse_bytes + (size_t)kp.cap * kCgCache * 4 +
            (size_t)(cp.max_blocks / 4 + 1) * (36 * 4 + 4) >= avail &&
        !detail::plan_cache(cp, csize, SB.h_row_ptr, h_col_idx, h_diag_pos, h_lens, ctx.nb, false,
                            kp))
      return unusable("a CTA's neighbour cache exceeds 65,535 rows");
    const size_t cache_bytes = (size_t)kp.cap * kCgCache * 4;
    if (row_bytes + coarse_bytes + cache_bytes >= avail)
      return unusable("row state and neighbour cache do not fit");
    const uint32_t cap_blocks = (uint32_t)std::min<size_t>(
        cp.max_blocks, (avail - row_bytes - coarse_bytes - cache_bytes) / (36 * 4 + 4));
    const size_t smem = cg_smem_bytes(cp.max_rows, cap_blocks, kp.cap) + coarse_bytes;
    check(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
          "cluster smem");
    if (csize > 8)
      check(cudaFuncSetAttribute(kfn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1),
            "cluster size");
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)csize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)cp.jobs.size());
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    const cudaError_t oe = cudaOccupancyMaxActiveClusters(&nclusters, kfn, &cfg);
    if (oe != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      return unusable(std::string("no cluster of ") + std::to_string(csize) + " CTAs with " +
                      std::to_string(smem) + " bytes of shared memory fits (" +
                      cudaGetErrorString(oe) + ")");
    }
    // Unless asked for, use clusters only when every model's cluster is
    // resident at once (one wave); otherwise models would queue behind each
    // other while the grid kernel runs them all together.
    if (!required && !prefer_cluster && (int64_t)nclusters < ctx.nm) return false;
    detail::h2d(cg_jobs, cp.jobs, s);
    detail::h2d(cg_loc, cp.row_loc, s);
    detail::h2d(cg_slot, kp.blk_slot, s);
    detail::h2d(cg_subp, kp.sub_ptr, s);
    detail::h2d(cg_sube, kp.sub_ent, s);
    ca = CgArgs{cg_jobs, cg_loc, SB.row_ptr, SB.col_idx, (const float*)S.p, (const float*)pre.p,
                (const float*)g.p, (float*)x.p, lens_row, lens_pos, SB.diag_pos, cp.max_rows,
                cap_blocks, active, pcg_iters, pcg_limit, o.pcg_tol};
    ca.cap = pcg_cap;
    ca.blk_slot = cg_slot, ca.sub_ptr = cg_subp, ca.sub_ent = cg_sube, ca.cap_cache = kp.cap;
    ca.err = ctx.err, ca.spin = o.wait_limit;
    use_coarse = coarse;
    ctx.last_coarse_dim = 0;
    if (coarse) {
      detail::h2d(c_grp_row0, gp.grp_row0, s), detail::h2d(c_grp_row1, gp.grp_row1, s);
      detail::h2d(c_grp_model, gp.grp_model, s), detail::h2d(c_model_g0, gp.model_g0, s);
      detail::h2d(c_row_grp, gp.row_grp, s), detail::h2d(c_job_g0, gp.job_g0, s);
      detail::h2d(c_job_g1, gp.job_g1, s), detail::h2d(c_model_eoff, gp.model_eoff, s);
      detail::h2d(c_grp_loc, gp.grp_loc, s);
      detail::h2d(c_pair_row, gp.pair_row, s), detail::h2d(c_pair_grp, gp.pair_grp, s);
      detail::h2d(c_row_pair0, gp.row_pair0, s);
      c_npairs = (int64_t)gp.pair_row.size();
      c_P.alloc(detail::at_least_1(c_npairs) * 49, s);
      cW.alloc(detail::at_least_1(ctx.nb) * kCoarseW, s);
      cW64.alloc(detail::at_least_1(ctx.nb) * kCoarseW, s);
      cE.alloc(detail::at_least_1(gp.e_total), s), cEinv.alloc(detail::at_least_1(gp.e_total), s);
      c_ngroups = (int32_t)gp.grp_row0.size();
      cargs = CoarseArgs{c_ngroups, c_grp_row0, c_grp_row1, c_grp_model, c_model_g0,
                         c_model_eoff, c_row_grp, active, cW, cW64, cE, cEinv};
      ca.W = cW, ca.Einv = cEinv, ca.model_eoff = c_model_eoff, ca.model_g0 = c_model_g0;
      ca.grp_row0 = c_grp_row0, ca.grp_row1 = c_grp_row1, ca.job_g0 = c_job_g0;
      ca.job_g1 = c_job_g1, ca.grp_loc = c_grp_loc;
      ca.cap_groups = std::max(gp.cap_groups, 1u), ca.cap_dim = std::max(gp.dmax, 1u);
      ctx.last_coarse_dim = (int32_t)gp.dmax;
    }
    check(cudaStreamSynchronize(s), "sync");
    cg_smem = smem;
    cl_size = csize;
    cl_threads = threads;
    use_cluster = true;
    ctx.last_pcg_kernel = 2, ctx.last_pcg_cluster = csize, ctx.last_pcg_threads = threads;
    ctx.last_pcg_ctas = (int32_t)cp.jobs.size();
    return true;
  }

  // Autotuner: time a short PCG run of every candidate configuration on the
  // system of the first iteration and keep the fastest per iteration.  The
  // choice is stored in the context and reused by later solves of this form.
  void autotune() {
    if (implicit) return;
    constexpr int kTuneIters = 40;
    const bool timing = T.on;
    T.on = false;  // tuning time is not a solve phase
    struct Restore {
      PhaseTimer& t;
      bool v;
      ~Restore() { t.on = v; }
    } restore{T, timing};
    build_system();
    // Per-observation passes of the mixed form: three kernels, or fused over
    // 128- or 256-observation chunks (all give the same values), timed as in
    // an LM iteration after an accepted step: the records are in place (the
    // build above formed them), so the record pass is skipped.
    double point_us = 0.0;
    if constexpr (sizeof(R) == 4) {
      if (o.point_kernel == 0 && ctx.no > 0) {
        check(cudaMemsetAsync(rec_stale.p, 0, 4 * ctx.nm, s), "memset");
        cudaEvent_t a, b;
        check(cudaEventCreate(&a), "event");
        check(cudaEventCreate(&b), "event");
        const StateView cur = ctx.cur();
        // an untimed run of each first, then the variants in turn (clock
        // ramps and cache state spread over all of them), best of four
        float best[4] = {1e30f, 1e30f, 1e30f, 1e30f};
        for (int rep = -1; rep < 4; ++rep)
          for (int v : {1, 2, 3}) {
            set_point_variant(v);
            check(cudaEventRecord(a, s), "event");
            point_passes(cur);
            check(cudaEventRecord(b, s), "event");
            check(cudaEventSynchronize(b), "tune");
            float ms = 0;
            check(cudaEventElapsedTime(&ms, a, b), "event");
            if (rep >= 0) best[v] = std::min(best[v], ms);
          }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        int best_v = 1;
        for (int v : {2, 3})
          if (best[v] < best[best_v]) best_v = v;
        set_point_variant(best_v);
        point_us = best[best_v] * 1000.0;
      }
    }
    // Schur sub-segment length: pairs per warp (more warps in flight to hide
    // the factor gathers, against more partial sums to add).
    double schur_us = 0.0;
    if (SB.ns > 0) {
      cudaEvent_t a, b;
      check(cudaEventCreate(&a), "event");
      check(cudaEventCreate(&b), "event");
      float best_ms = 1e30f;
      uint32_t best_L = sub_len;
      for (uint32_t L : {256u, 512u, 1024u, 2048u}) {
        set_sub_len(L);
        for (int rep = 0; rep < 3; ++rep) {
          check(cudaEventRecord(a, s), "event");
          BA_LAUNCH(schur_kernel<R><<<grid_for(SB.nsub * 32, 256), 256, 0, s>>>(P, SV, B, active));
          check(cudaEventRecord(b, s), "event");
          check(cudaEventSynchronize(b), "tune");
          float ms = 0;
          check(cudaEventElapsedTime(&ms, a, b), "event");
          if (ms < best_ms) best_ms = ms, best_L = L;
        }
      }
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      set_sub_len(best_L);
      schur_us = best_ms * 1000.0;
      build_system();  // the system with the kept sub-segments
    }
    struct Cand {
      int kernel, param, threads;  // grid: rows_target; cluster: CTAs per cluster
    };
    std::vector<Cand> cand;
    // With the two-level preconditioner (cluster kernel only) the PCG needs a
    // fraction of the iterations, so only cluster layouts compete; the grid
    // layouts remain the fallback when no cluster fits.
    const bool coarse_only = sizeof(R) == 4 && o.coarse != 0;
    if (!coarse_only)
      for (int rt : {2, 3, 4, 6, 8, 12, 16}) cand.push_back({1, rt, kPcgThreads});
    if constexpr (sizeof(R) == 4)
      for (int th : {kCgThreads, kCgThreadsWide})
        for (int cs : {4, 8, 12, 16}) cand.push_back({2, cs, th});
    cudaEvent_t e0, e1;
    check(cudaEventCreate(&e0), "event");
    check(cudaEventCreate(&e1), "event");
    struct Ev {
      cudaEvent_t a, b;
      ~Ev() { cudaEventDestroy(a), cudaEventDestroy(b); }
    } ev{e0, e1};
    double best = 1e300;
    Cand best_c{1, 4, kPcgThreads};
    bool any = false;
    std::vector<int32_t> hit(ctx.nm);
    for (const auto& c : cand) {
      if (c.kernel == 1) {
        plan_grid(c.param);
      } else if (!try_cluster(c.param, false, true, c.threads)) {
        continue;
      }
      const int32_t mi = pa.max_iter;
      pa.max_iter = ca.max_iter = kTuneIters;
      float tbest = 1e30f;
      for (int rep = 0; rep < 2; ++rep) {
        check(cudaEventRecord(e0, s), "event");
        solve_pcg();
        check(cudaEventRecord(e1, s), "event");
        check(cudaEventSynchronize(e1), "tune");
        float ms = 0;
        check(cudaEventElapsedTime(&ms, e0, e1), "event");
        tbest = std::min(tbest, ms);
      }
      pa.max_iter = ca.max_iter = mi;
      check(cudaMemcpy(hit.data(), pcg_iters.p, 4 * ctx.nm, cudaMemcpyDeviceToHost), "d2h");
      int32_t its = 1;
      for (int32_t v : hit) its = std::max(its, v);
      const double per = (double)tbest / its;
      if (per < best) best = per, best_c = c;
      any = true;
    }
    if (!any) {  // two-level form, but no cluster fits: grid layouts
      for (int rt : {2, 4, 8}) {
        plan_grid(rt);
        const int32_t mi = pa.max_iter;
        pa.max_iter = kTuneIters;
        check(cudaEventRecord(e0, s), "event");
        solve_pcg();
        check(cudaEventRecord(e1, s), "event");
        check(cudaEventSynchronize(e1), "tune");
        pa.max_iter = mi;
        float ms = 0;
        check(cudaEventElapsedTime(&ms, e0, e1), "event");
        const double per = (double)ms / kTuneIters;
        if (per < best) best = per, best_c = {1, rt, kPcgThreads};
      }
    }
    PcgTuning& tu = ctx.tuning[sizeof(R) == 8 ? 0 : 1];
    tu.valid = true;
    tu.kernel = best_c.kernel;
    tu.rows_target = best_c.kernel == 1 ? best_c.param : 4;
    tu.cluster = best_c.kernel == 2 ? best_c.param : 0;
    tu.cg_threads = best_c.kernel == 2 ? best_c.threads : kCgThreads;
    tu.us_per_iter = best * 1000.0;
    tu.sub_len = (int)sub_len;
    tu.schur_us = schur_us;
    tu.point_kernel = sizeof(R) == 4 && o.point_kernel == 0 ? point_variant : 0;
    tu.point_us = point_us;
    {
      std::lock_guard<std::mutex> lk(tune_mutex());
      tune_cache()[tune_key()] = tu;
    }
    if (best_c.kernel == 2 && try_cluster(best_c.param, false, true, best_c.threads)) return;
    plan_grid(tu.rows_target);
  }

  TuneKey tune_key() const {
    return TuneKey{sizeof(R) == 8 ? 0 : 1, o.coarse, ctx.nm, ctx.nb, SB.nz};
  }

  void set_lambda(double lam) {
    std::vector<double> v(ctx.nm, lam);
    check(cudaMemcpyAsync(lambda.p, v.data(), 8 * ctx.nm, cudaMemcpyHostToDevice, s), "h2d");
    check(cudaStreamSynchronize(s), "sync");
  }

  // records (mixed form): also form every active model's records at `st`.
  void eval_cost(const StateView& st, const int32_t* act, double* out_cost, double* out_sq,
                 int64_t* out_n, bool records = false) {
    bool done = false;
    if constexpr (sizeof(R) == 4) {
      if (records) {
        if (ctx.nc > 0)
          BA_LAUNCH(cam_f32_kernel<<<grid_for(ctx.nc, 128), 128, 0, s>>>(P, st, camf, act));
        BA_LAUNCH(cost_record_kernel<<<(unsigned)detail::at_least_1(SB.ncost), kCostThreads, 0,
                                       s>>>(P, st, SV, B, camf, cost_part, act, sigma));
        done = true;
      }
    }
    if (!done)
      BA_LAUNCH(cost_chunk_kernel<<<(unsigned)detail::at_least_1(SB.ncost), kCostThreads, 0, s>>>(
          P, st, SV, cost_part, act, sigma));
    BA_LAUNCH(cost_final_kernel<<<(unsigned)ctx.nm, kCostFinalThreads, 0, s>>>(
        P, st, SV, cost_part, act, out_cost, out_sq, out_n));
  }

  // Reduced system at the current state and damping (ba.rs:221-331).
  void build_system() {
    const StateView cur = ctx.cur();
    T.mark(-1);
    fork_coarse_basis();
    if constexpr (sizeof(R) == 4) {
      if (ctx.nc > 0)
        BA_LAUNCH(cam_f32_kernel<<<grid_for(ctx.nc, 128), 128, 0, s>>>(P, cur, camf, active));
      point_passes(cur);
    } else {
      BA_LAUNCH(point_kernel<R><<<grid_for(ctx.np, 128), 128, 0, s>>>(P, cur, SV, B, active,
                                                                     lambda, sigma));
    }
    T.mark(BA_PHASE_POINT);
    // The camera sums and the Schur sums read what the point passes wrote and
    // nothing of each other, and both wait mostly on gathers: the camera pass
    // runs on the second stream beside the Schur kernel (one after the other
    // when phases are timed, so that each phase has its own interval).
    const bool split = !implicit && !T.on;
    cudaStream_t cs = s;
    if (split) {
      side_stream();
      check(cudaEventRecord(ev_cam, s), "fork");
      check(cudaStreamWaitEvent(s2, ev_cam, 0), "fork");
      cs = s2;
    }
    if (ctx.nc > 0) {
      if constexpr (sizeof(R) == 4)
        BA_LAUNCH(camera_mixed_kernel<<<(unsigned)ctx.nc, kCamMixThreads, 0, cs>>>(P, SV, B,
                                                                                  active));
      else
        BA_LAUNCH(camera_kernel<R><<<(unsigned)ctx.nc, kCamThreads, 0, cs>>>(P, SV, B, active));
    }
    BA_LAUNCH(group_kernel<<<grid_for(ctx.ng * 32, 128), 128, 0, cs>>>(P, SV, caml, grpU, grpg,
                                                                      active));
    if (split) check(cudaEventRecord(ev_cam_join, s2), "join");
    T.mark(BA_PHASE_CAMERA);
    if (implicit) {
      T.mark(BA_PHASE_SCHUR);
      BA_LAUNCH(lens_diag_kernel<R><<<kLensChunks, 256, 0, s>>>(SV, B, lens_part));
      BA_LAUNCH(implicit_blocks_kernel<R><<<(unsigned)ctx.nb, 256, 0, s>>>(
          P, cur, SV, B, B.Z, own, active, lambda, lens_part, zsrc));
      BA_LAUNCH(rhs_kernel<R><<<grid_for(ctx.nb * 6, 256), 256, 0, s>>>(P, cur, B, active));
      T.mark(BA_PHASE_ASSEMBLE);
      return;
    }
    if (SB.nsub > 0)
      BA_LAUNCH(schur_kernel<R><<<grid_for(SB.nsub * 32, 256), 256, 0, s>>>(P, SV, B, active));
    if (n_fold > 0)
      BA_LAUNCH(schur_fold_kernel<<<n_fold, kFoldThreads, 0, s>>>(P, SV, part, fold_slots,
                                                                 active));
    if (split) check(cudaStreamWaitEvent(s, ev_cam_join, 0), "join");
    T.mark(BA_PHASE_SCHUR);
    if (SB.ns > 0)
      BA_LAUNCH(assemble_kernel<R><<<grid_for(SB.ns * 36, 256), 256, 0, s>>>(
          P, cur, SV, B, active, lambda, c_S64.p, sub_end.p));
    fork_coarse();
    BA_LAUNCH(rhs_kernel<R><<<grid_for(ctx.nb * 6, 256), 256, 0, s>>>(P, cur, B, active));
    BA_LAUNCH(precond_kernel<R><<<grid_for(ctx.nb, 128), 128, 0, s>>>(P, SV, B, active));
    T.mark(BA_PHASE_ASSEMBLE);
  }

  // Block-Jacobi PCG (ba.rs:155-196).
  void solve_pcg() {
    if (implicit) {
      void* args[] = {&ia};
      check(cudaLaunchCooperativeKernel((void*)implicit_kernel(), dim3(imp_ncta),
                                        dim3(kPcgThreads), args, 0, s),
            "pcg launch");
    } else if (use_cluster) {
      if (use_coarse && c_ngroups > 0) {
        // forked after the assembly of this system, or (a new PCG plan since)
        // run here
        if (coarse_pending && !basis_forked) {
          join_coarse();
        } else {
          join_coarse();
          basis_forked = false;
          launch_coarse_chain(s);
        }
      }
      cudaLaunchConfig_t cfg{};
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = (unsigned)cl_size;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3((unsigned)(ctx.nm * cl_size));
      cfg.blockDim = dim3((unsigned)cl_threads);
      cfg.dynamicSmemBytes = cg_smem;
      cfg.stream = s;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      check(cudaLaunchKernelEx(&cfg, detail::cg_kernel(use_coarse, cl_threads), ca),
            "pcg cluster launch");
    } else {
      void* args[] = {&pa};
      check(cudaLaunchCooperativeKernel((void*)pcg_kernel<R>, dim3(plan.ncta), dim3(kPcgThreads),
                                        args, smem_bytes, s),
            "pcg launch");
    }
    g_launches++;
    T.mark(BA_PHASE_PCG);
  }

  // Trial state = current state + step (ba.rs:338-366).
  void update() {
    const StateView cur = ctx.cur(), tri = ctx.trial();
    // The cameras' and lens groups' update and the points' back-substitution
    // write different parts of the trial state and read only the current one:
    // the former runs on the second stream (one after the other when phases
    // are timed).
    const bool split = !T.on;
    cudaStream_t us = s;
    if (split) {
      side_stream();
      check(cudaEventRecord(ev_cam, s), "fork");
      check(cudaStreamWaitEvent(s2, ev_cam, 0), "fork");
      us = s2;
    }
    BA_LAUNCH(update_cameras_kernel<R><<<grid_for(std::max(ctx.nc, ctx.ng), 256), 256, 0, us>>>(
        P, cur, tri, B, active));
    if (split) check(cudaEventRecord(ev_cam_join, s2), "join");
    if constexpr (sizeof(R) == 4) {
      if (ctx.no > 0)
      {
        if (z_recompute)
          BA_LAUNCH(obs_backsub_kernel<true><<<grid_for(ctx.no, 256), 256, 0, s>>>(
              P, B, obs_u.p, active, zsrc));
        else
          BA_LAUNCH(obs_backsub_kernel<false><<<grid_for(ctx.no, 256), 256, 0, s>>>(
              P, B, obs_u.p, active, zsrc));
      }
    }
    BA_LAUNCH(backsub_kernel<R><<<grid_for(ctx.np, 256), 256, 0, s>>>(P, SV, cur, tri, B, sigma,
                                                                     active, obs_u.p));
    if (split) check(cudaStreamWaitEvent(s, ev_cam_join, 0), "join");
    T.mark(BA_PHASE_UPDATE);
  }

  // Accept / reject (ba.rs:367-383).
  void control_and_commit() {
    check(cudaMemsetAsync(any.p, 0, 4, s), "memset");
    BA_LAUNCH(control_kernel<<<grid_for(ctx.nm, 128), 128, 0, s>>>(ctx.nm, C));
    BA_LAUNCH(commit_kernel<<<grid_for(std::max(std::max(ctx.np, ctx.nc), ctx.ng), 256), 256, 0, s>>>(
        P, ctx.grp_model, ctx.cur(), ctx.trial(), accepted));
    T.mark(BA_PHASE_CONTROL);
  }

  void iteration() {
    build_system();
    solve_pcg();
    update();
    eval_cost(ctx.trial(), active, new_cost, rms, n_front, true);
    T.mark(BA_PHASE_COST);
    control_and_commit();
  }

  void run() {
    const int64_t nm = ctx.nm;
    T.mark(-1);
    setup();
    T.mark(BA_PHASE_SETUP);
    if (o.autotune && !ctx.tuning[sizeof(R) == 8 ? 0 : 1].valid) autotune();
    eval_cost(ctx.cur(), nullptr, cost, sq, n_front, true);  // ba.rs:216
    if constexpr (sizeof(R) == 4)  // the records of the initial state are in place
      check(cudaMemsetAsync(rec_stale.p, 0, 4 * nm, s), "memset");
    std::vector<double> h_cost0(nm), h_sq0(nm);
    std::vector<int64_t> h_n0(nm);
    check(cudaMemcpyAsync(h_cost0.data(), cost.p, 8 * nm, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaMemcpyAsync(h_sq0.data(), sq.p, 8 * nm, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaMemcpyAsync(h_n0.data(), n_front.p, 8 * nm, cudaMemcpyDeviceToHost, s), "d2h");
    // Pinned words read after every LM iteration: [0] any model active,
    // [1] the device error bits (a wait that gave up ends the solve).
    int32_t* h_any = nullptr;
    check(cudaMallocHost((void**)&h_any, 2 * sizeof(int32_t)), "pinned");
    struct PinnedFree {
      int32_t* p;
      ~PinnedFree() { cudaFreeHost(p); }
    } pf{h_any};
    // One LM iteration is a fixed sequence of kernels over device-resident
    // data, so it is captured once as a CUDA graph and replayed; the host only
    // reads the "any model active" flag between iterations.  Phase timing
    // needs events between kernels and runs without the graph.
    IterationGraph graph;
    const bool use_graph = !T.on && o.graph != 0;
    for (int32_t it = 0; it < o.max_iter; ++it) {
      if (use_graph && graph.ok(this)) {
        graph.launch(s);
      } else {
        iteration();
      }
      check(cudaMemcpyAsync(h_any, any.p, 4, cudaMemcpyDeviceToHost, s), "d2h");
      check(cudaMemcpyAsync(h_any + 1, ctx.err.p, 4, cudaMemcpyDeviceToHost, s), "d2h");
      check(cudaStreamSynchronize(s), "lm iteration");
      T.flush(ctx.phase_ms, ctx.phase_n);
      if (!h_any[0] || h_any[1]) break;
    }
    ctx.last_graph = graph.exec != nullptr;
    eval_cost(ctx.cur(), nullptr, cost, sq, n_front);  // ba.rs:385
    std::vector<double> h_cost1(nm), h_sq1(nm);
    std::vector<int64_t> h_n1(nm), h_pcg(nm);
    std::vector<int32_t> h_it(nm);
    check(cudaMemcpyAsync(h_cost1.data(), cost.p, 8 * nm, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaMemcpyAsync(h_sq1.data(), sq.p, 8 * nm, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaMemcpyAsync(h_n1.data(), n_front.p, 8 * nm, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaMemcpyAsync(h_it.data(), iters.p, 4 * nm, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaMemcpyAsync(h_pcg.data(), pcg_total.p, 8 * nm, cudaMemcpyDeviceToHost, s), "d2h");
    if (log_cap > 0) {
      const ba_log* L = o.log;
      if (L->new_cost) check(cudaMemcpyAsync(L->new_cost, log_cost.p, 8 * log_cap, cudaMemcpyDeviceToHost, s), "d2h");
      if (L->lambda) check(cudaMemcpyAsync(L->lambda, log_lam.p, 8 * log_cap, cudaMemcpyDeviceToHost, s), "d2h");
      if (L->pcg_iters) check(cudaMemcpyAsync(L->pcg_iters, log_pcg.p, 4 * log_cap, cudaMemcpyDeviceToHost, s), "d2h");
      if (L->accepted) check(cudaMemcpyAsync(L->accepted, log_acc.p, 4 * log_cap, cudaMemcpyDeviceToHost, s), "d2h");
    }
    check(cudaStreamSynchronize(s), "final");
    ctx.results.assign(nm, ModelResult{});
    for (int64_t m = 0; m < nm; ++m) {
      ModelResult& res = ctx.results[m];
      res.iterations = h_it[m];
      res.initial_cost = h_cost0[m];
      res.final_cost = h_cost1[m];
      res.initial_rms = std::sqrt(h_sq0[m] / (double)std::max<int64_t>(h_n0[m], 1));
      res.final_rms = std::sqrt(h_sq1[m] / (double)std::max<int64_t>(h_n1[m], 1));
      res.pcg = h_pcg[m];
    }
  }

  // One system at damping `lam` from the uploaded state, without acceptance
  // (model 0; dense output for small problems).  Mirrors the oracle's step.
  void debug_step(double lam, double* S_dense, double* g_out, double* dx_out, int32_t* pcg_out,
                  double* trial_cost) {
    setup();
    set_lambda(lam);
    build_system();
    solve_pcg();
    update();
    eval_cost(ctx.trial(), active, new_cost, rms, n_front);
    const int64_t nb = ctx.h_blk0[1], nz = SB.h_row_ptr[nb];
    std::vector<R> hS(nz * 36), hg(nb * 6), hx(nb * 6);
    std::vector<uint32_t> hcol(std::max<int64_t>(nz, 1));
    if (nz) {
      check(cudaMemcpyAsync(hS.data(), S.p, sizeof(R) * hS.size(), cudaMemcpyDeviceToHost, s), "d2h");
      check(cudaMemcpyAsync(hcol.data(), SB.col_idx.p, 4 * nz, cudaMemcpyDeviceToHost, s), "d2h");
    }
    check(cudaMemcpyAsync(hg.data(), g.p, sizeof(R) * hg.size(), cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaMemcpyAsync(hx.data(), x.p, sizeof(R) * hx.size(), cudaMemcpyDeviceToHost, s), "d2h");
    int32_t it = 0;
    double tc = 0;
    check(cudaMemcpyAsync(&it, pcg_iters.p, 4, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaMemcpyAsync(&tc, new_cost.p, 8, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaStreamSynchronize(s), "debug");
    if (S_dense) {
      const int64_t n6 = 6 * nb;
      std::fill(S_dense, S_dense + n6 * n6, 0.0);
      for (int64_t row = 0; row < nb; ++row)
        for (uint32_t k = SB.h_row_ptr[row]; k < SB.h_row_ptr[row + 1]; ++k)
          for (int a = 0; a < 6; ++a)
            for (int b = 0; b < 6; ++b)
              S_dense[(6 * row + a) * n6 + 6 * (int64_t)hcol[k] + b] = (double)hS[36 * (size_t)k + 6 * a + b];
    }
    for (int64_t i = 0; i < 6 * nb; ++i) {
      if (g_out) g_out[i] = (double)hg[i];
      if (dx_out) dx_out[i] = (double)hx[i];
    }
    if (pcg_out) *pcg_out = it;
    if (trial_cost) *trial_cost = tc;
  }
};

template <typename R>
void run_lm(Context& ctx, const Opts& o) {
  LmEngine<R> e(ctx, o);
  e.run();
}

template <typename R>
void debug_lm_step(Context& ctx, const Opts& o, double lam, double* S_dense, double* g,
                   double* dx, int32_t* pcg_iters, double* trial_cost) {
  LmEngine<R> e(ctx, o);
  e.debug_step(lam, S_dense, g, dx, pcg_iters, trial_cost);
}

}  // namespace ba
