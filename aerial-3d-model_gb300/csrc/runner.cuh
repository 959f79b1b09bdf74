// Host driver of the LM loop (ba.rs:198-391) for storage precision R.
#pragma once

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <vector>

#include "context.cuh"
#include "pcg.cuh"
#include "pcg_cluster.cuh"
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
  for (int64_t m = 0; m < nm; ++m) {
    rows[m] = ctx.h_blk0[m + 1] - ctx.h_blk0[m];
    G[m] = std::max<int64_t>(1, (rows[m] + rows_target - 1) / rows_target);
    tot += G[m];
    need += std::max<int64_t>(1, (rows[m] + rows_cap - 1) / rows_cap);
  }
  max_ctas = std::min(max_ctas, kMaxGroupCtas);
  if (need > max_ctas) {
    // More models than resident CTAs: one CTA per model, dealt greedily to
    // the least-loaded CTA (largest first); a CTA solves its models in turn.
    for (int64_t m = 0; m < nm; ++m)
      if (rows[m] > rows_cap) throw std::runtime_error("batch too large for the PCG plan");
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

template <typename T>
void h2d(DevBuf<T>& d, const std::vector<T>& h, cudaStream_t s) {
  d.alloc(h.size(), s);
  if (!h.empty())
    check(cudaMemcpyAsync(d.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s), "h2d");
}

inline int64_t at_least_1(int64_t n) { return n > 0 ? n : 1; }

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
  DevBuf<double> camU, camgj, camgs, camX, caml, grpU, grpg, cost_part;
  IterBufs<R> B{};
  DevBuf<double> lambda, cost, new_cost, rms, sq, sigma;
  DevBuf<int64_t> n_front, pcg_total;
  DevBuf<int32_t> active, accepted, iters, pcg_iters, any;
  DevBuf<double> log_cost, log_lam;
  DevBuf<int32_t> log_pcg, log_acc;
  int32_t log_cap = 0;
  Control C{};
  detail::PcgPlan plan;
  DevBuf<PcgJob> jobs;
  DevBuf<int32_t> cta_job0;
  DevBuf<unsigned long long> bar, bar_base;
  DevBuf<double> pcg_part;
  DevBuf<int32_t> lens_row, lens_pos;
  uint32_t smem_rows = 0, smem_blocks = 0;
  size_t smem_bytes = 0;
  int pcg_rows_target = 0;
  PcgArgs<R> pa{};
  // Cluster-resident PCG (mixed form).
  bool use_cluster = false;
  int cl_size = 0;
  DevBuf<CgJob> cg_jobs;
  DevBuf<uint32_t> cg_loc;
  CgArgs ca{};
  size_t cg_smem = 0;
  PhaseTimer T;

  LmEngine(Context& c, const Opts& opts) : ctx(c), o(opts), s(c.stream) {
    T.on = o.profile != 0;
    T.s = s;
    for (int k = 0; k < kPhases; ++k) ctx.phase_ms[k] = 0, ctx.phase_n[k] = 0;
  }

  void setup() {
    using detail::at_least_1;
    const int64_t nc = ctx.nc, np = ctx.np, no = ctx.no, ng = ctx.ng, nb = ctx.nb, nm = ctx.nm;
    reset_states(ctx);
    P = ctx.prob(o.loss);
    build_structure(P, ctx.h_obs0, SB, ctx.err, s);
    SV = SB.view();
    ctx.last_nz = SB.nz, ctx.last_pairs = SB.npairs - nb, ctx.last_nl = SB.nl;
    lin.alloc(at_least_1(no) * kLinW, s), gsub.alloc(at_least_1(no) * 9, s);
    Z.alloc(at_least_1(no) * 18, s), Zl.alloc(at_least_1(SB.nl) * 9, s);
    ptL.alloc(at_least_1(np) * 6, s), ptzv.alloc(at_least_1(np) * 3, s);
    kept.alloc(at_least_1(np), s);
    camU.alloc(at_least_1(nc) * 21, s), camgj.alloc(at_least_1(nc) * 6, s);
    camgs.alloc(at_least_1(nc) * 6, s), camX.alloc(at_least_1(nc) * 18, s);
    caml.alloc(at_least_1(nc) * 12, s), grpU.alloc(at_least_1(ng) * 6, s);
    grpg.alloc(at_least_1(ng) * 3, s);
    part.alloc(at_least_1(SB.nsub) * 36, s), S.alloc(at_least_1(SB.nz) * 36, s);
    pre.alloc(at_least_1(nb) * 36, s);
    g.alloc(at_least_1(nb) * 6, s), x.alloc(at_least_1(nb) * 6, s);
    z.alloc(at_least_1(nb) * 6, s), p.alloc(at_least_1(nb) * 12, s);
    cost_part.alloc(at_least_1(SB.ncost) * 3, s);
    // Camera sums are read for every camera, including ones without observations.
    camU.zero(), camgj.zero(), camgs.zero(), camX.zero(), caml.zero(), grpU.zero(), grpg.zero();
    x.zero();
    B = IterBufs<R>{lin, gsub, Z, Zl, ptL, ptzv, kept, camU, camgj, camgs, camX, caml,
                    grpU, grpg, part, S, pre, g, x, cost_part};
    lambda.alloc(nm, s), cost.alloc(nm, s), new_cost.alloc(nm, s), rms.alloc(nm, s);
    sq.alloc(nm, s), sigma.alloc(nm, s), n_front.alloc(nm, s), pcg_total.alloc(nm, s);
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
    C = Control{lambda, cost, new_cost, rms, sq, n_front, active, accepted, iters, pcg_iters,
                pcg_total, any, sigma, o.max_iter, log_cap, log_cost, log_lam, log_pcg, log_acc};
    // PCG plan (cooperative launch: all CTAs co-resident).  Shared memory per
    // CTA: row state for up to kSmemRows rows, then as many S blocks as fit.
    smem_rows = 64;
    smem_blocks = (uint32_t)((kPcgSmemBudget - (size_t)smem_rows * kRowState * sizeof(R)) /
                             (36 * sizeof(R) + 4));
    smem_bytes = pcg_smem_bytes<R>(smem_rows, smem_blocks);
    check(cudaFuncSetAttribute(pcg_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem_bytes),
          "pcg smem");
    int occ = 0;
    check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pcg_kernel<R>, kPcgThreads,
                                                        smem_bytes),
          "occupancy");
    const int max_ctas = std::max(1, occ) * ctx.n_sm;
    std::vector<int32_t> h_lens(nm, -1);
    for (int64_t m = 0; m < nm; ++m)
      if (ctx.h_grp0[m + 1] - ctx.h_grp0[m] == 1)
        h_lens[m] = (int32_t)(ctx.h_blk0[m] + (ctx.h_cam0[m + 1] - ctx.h_cam0[m]));
    // FP64 instructions serialise per SM sub-partition: one row per warp on
    // four warps; FP32 rows are cheap: one per warp on all eight.
    const int rows_target = pcg_rows_target > 0 ? pcg_rows_target : (sizeof(R) == 8 ? 4 : 8);
    plan = detail::plan_pcg(ctx, SB.h_row_ptr, h_lens, max_ctas, rows_target, (int)smem_rows);
    detail::h2d(lens_row, h_lens, s);
    lens_pos.alloc(detail::at_least_1(nb), s);
    if (nb > 0)
      BA_LAUNCH(lens_pos_kernel<<<grid_for(nb, 256), 256, 0, s>>>(nb, SB.row_ptr, SB.col_idx,
                                                                 P.blk_model, lens_row, lens_pos));
    detail::h2d(jobs, plan.jobs, s);
    detail::h2d(cta_job0, plan.cta_job0, s);
    bar.alloc(nm, s);
    bar.zero();
    bar_base.alloc(nm, s);
    bar_base.zero();
    pcg_part.alloc(kParts * (size_t)plan.ncta, s);
    check(cudaStreamSynchronize(s), "sync");  // host plan vectors
    pa = PcgArgs<R>{jobs, cta_job0, bar, bar_base, pcg_part, plan.ncta, SB.row_ptr, SB.col_idx, S, pre, g,
                    x, z, p, nb, lens_row, lens_pos, smem_rows, smem_blocks, active, pcg_iters,
                    o.pcg_max_iter, o.pcg_tol, ctx.err};
    ctx.last_pcg_kernel = 1, ctx.last_pcg_cluster = 0;
    if constexpr (sizeof(R) == 4) setup_cluster(h_lens);
    else if (o.pcg_kernel == 2)
      throw CudaError(cudaErrorNotSupported, "cluster PCG: the FP64 form uses the grid kernel");
  }

  // Mixed form: one cluster of up to 16 CTAs per model with the whole PCG in
  // distributed shared memory, if every model fits; else the grid kernel.
  void setup_cluster(const std::vector<int32_t>& h_lens) {
    use_cluster = false;
    ctx.last_pcg_kernel = 1, ctx.last_pcg_cluster = 0;
    if (o.pcg_kernel == 1) return;  // grid kernel requested
    const bool required = o.pcg_kernel == 2;
    auto unusable = [&](const std::string& why) {
      if (required) throw CudaError(cudaErrorNotSupported, "cluster PCG: " + why);
    };
    int64_t max_rows = 0;
    for (int64_t m = 0; m < ctx.nm; ++m)
      max_rows = std::max<int64_t>(max_rows, ctx.h_blk0[m + 1] - ctx.h_blk0[m]);
    const int csize = (int)std::min<int64_t>(kCgMaxCluster, std::max<int64_t>(1, (max_rows + 31) / 32));
    int smem_optin = 0;
    check(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx.device),
          "attr");
    cudaFuncAttributes fa{};
    check(cudaFuncGetAttributes(&fa, pcg_cluster_kernel), "func attr");
    const size_t avail = (size_t)smem_optin - fa.sharedSizeBytes;
    const uint32_t rows_cap = (uint32_t)std::min<size_t>(avail / 2 / (kCgRow * 4), 4096);
    detail::ClusterPlan cp;
    if (!detail::plan_cluster(ctx, SB.h_row_ptr, h_lens, csize, rows_cap, cp))
      return unusable("a model has too many block rows for one cluster");
    const size_t row_bytes = (size_t)cp.max_rows * kCgRow * 4;
    const uint32_t cap_blocks = (uint32_t)std::min<size_t>(cp.max_blocks, (avail - row_bytes) / (36 * 4 + 4));
    const size_t smem = cg_smem_bytes(cp.max_rows, cap_blocks);
    check(cudaFuncSetAttribute(pcg_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem),
          "cluster smem");
    if (csize > 8)
      check(cudaFuncSetAttribute(pcg_cluster_kernel,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1),
            "cluster size");
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)csize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)cp.jobs.size());
    cfg.blockDim = dim3(kCgThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    const cudaError_t oe = cudaOccupancyMaxActiveClusters(&nclusters, pcg_cluster_kernel, &cfg);
    if (oe != cudaSuccess || nclusters < 1) {
      cudaGetLastError();
      return unusable(std::string("no cluster of ") + std::to_string(csize) + " CTAs with " +
                      std::to_string(smem) + " bytes of shared memory fits (" +
                      cudaGetErrorString(oe) + ")");
    }
    detail::h2d(cg_jobs, cp.jobs, s);
    detail::h2d(cg_loc, cp.row_loc, s);
    check(cudaStreamSynchronize(s), "sync");
    ca = CgArgs{cg_jobs, cg_loc, SB.row_ptr, SB.col_idx, (const float*)S.p, (const float*)pre.p,
                (const float*)g.p, (float*)x.p, lens_row, lens_pos, SB.diag_pos, cp.max_rows,
                cap_blocks, active, pcg_iters, o.pcg_max_iter, o.pcg_tol};
    cg_smem = smem;
    cl_size = csize;
    use_cluster = true;
    ctx.last_pcg_kernel = 2, ctx.last_pcg_cluster = csize;
  }

  void set_lambda(double lam) {
    std::vector<double> v(ctx.nm, lam);
    check(cudaMemcpyAsync(lambda.p, v.data(), 8 * ctx.nm, cudaMemcpyHostToDevice, s), "h2d");
    check(cudaStreamSynchronize(s), "sync");
  }

  void eval_cost(const StateView& st, const int32_t* act, double* out_cost, double* out_sq,
                 int64_t* out_n) {
    BA_LAUNCH(cost_chunk_kernel<<<(unsigned)detail::at_least_1(SB.ncost), kCostThreads, 0, s>>>(
        P, st, SV, cost_part, act, sigma));
    BA_LAUNCH(cost_final_kernel<<<grid_for(ctx.nm * 32, 128), 128, 0, s>>>(
        P, st, SV, cost_part, act, out_cost, out_sq, out_n));
  }

  // Reduced system at the current state and damping (ba.rs:221-331).
  void build_system() {
    const StateView cur = ctx.cur();
    T.mark(-1);
    BA_LAUNCH(point_kernel<R><<<grid_for(ctx.np, 128), 128, 0, s>>>(P, cur, SV, B, active, lambda,
                                                                   sigma));
    T.mark(BA_PHASE_POINT);
    if (ctx.nc > 0)
      BA_LAUNCH(camera_kernel<R><<<(unsigned)ctx.nc, kCamThreads, 0, s>>>(P, SV, B, active));
    BA_LAUNCH(group_kernel<<<grid_for(ctx.ng * 32, 128), 128, 0, s>>>(P, SV, caml, grpU, grpg,
                                                                     active));
    T.mark(BA_PHASE_CAMERA);
    if (SB.nsub > 0)
      BA_LAUNCH(schur_kernel<R><<<grid_for(SB.nsub * 32, 256), 256, 0, s>>>(P, SV, B, active));
    T.mark(BA_PHASE_SCHUR);
    if (SB.ns > 0)
      BA_LAUNCH(assemble_kernel<R><<<grid_for(SB.ns * 36, 256), 256, 0, s>>>(P, cur, SV, B, active,
                                                                            lambda));
    BA_LAUNCH(rhs_kernel<R><<<grid_for(ctx.nb * 6, 256), 256, 0, s>>>(P, cur, B, active));
    BA_LAUNCH(precond_kernel<R><<<grid_for(ctx.nb, 128), 128, 0, s>>>(P, SV, B, active));
    T.mark(BA_PHASE_ASSEMBLE);
  }

  // Block-Jacobi PCG (ba.rs:155-196).
  void solve_pcg() {
    if (use_cluster) {
      cudaLaunchConfig_t cfg{};
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = (unsigned)cl_size;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3((unsigned)(ctx.nm * cl_size));
      cfg.blockDim = dim3(kCgThreads);
      cfg.dynamicSmemBytes = cg_smem;
      cfg.stream = s;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      check(cudaLaunchKernelEx(&cfg, pcg_cluster_kernel, ca), "pcg cluster launch");
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
    BA_LAUNCH(update_cameras_kernel<R><<<grid_for(std::max(ctx.nc, ctx.ng), 256), 256, 0, s>>>(
        P, cur, tri, B, active));
    BA_LAUNCH(backsub_kernel<R><<<grid_for(ctx.np, 256), 256, 0, s>>>(P, SV, cur, tri, B, sigma,
                                                                     active));
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
    eval_cost(ctx.trial(), active, new_cost, rms, n_front);
    T.mark(BA_PHASE_COST);
    control_and_commit();
  }

  void run() {
    const int64_t nm = ctx.nm;
    T.mark(-1);
    setup();
    T.mark(BA_PHASE_SETUP);
    eval_cost(ctx.cur(), nullptr, cost, sq, n_front);  // ba.rs:216
    std::vector<double> h_cost0(nm), h_sq0(nm);
    std::vector<int64_t> h_n0(nm);
    check(cudaMemcpyAsync(h_cost0.data(), cost.p, 8 * nm, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaMemcpyAsync(h_sq0.data(), sq.p, 8 * nm, cudaMemcpyDeviceToHost, s), "d2h");
    check(cudaMemcpyAsync(h_n0.data(), n_front.p, 8 * nm, cudaMemcpyDeviceToHost, s), "d2h");
    int32_t* h_any = nullptr;
    check(cudaMallocHost((void**)&h_any, sizeof(int32_t)), "pinned");
    struct PinnedFree {
      int32_t* p;
      ~PinnedFree() { cudaFreeHost(p); }
    } pf{h_any};
    for (int32_t it = 0; it < o.max_iter; ++it) {
      iteration();
      check(cudaMemcpyAsync(h_any, any.p, 4, cudaMemcpyDeviceToHost, s), "d2h");
      check(cudaStreamSynchronize(s), "lm iteration");
      T.flush(ctx.phase_ms, ctx.phase_n);
      if (!*h_any) break;
    }
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
