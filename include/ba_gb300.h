/*
 * ba_gb300.h — C ABI of the GB300 (sm_103a) bundle-adjustment solver.
 *
 * Drop-in for stitch-core's
 *     pub fn bundle_adjust(p: &mut Problem, max_iter: usize, sigma_px: f64) -> BaStats
 * (crates/stitch-core/src/recon/ba.rs:198), with the reference's types
 * `Obs`, `Problem` and `BaStats` (ba.rs:21-46) flattened to
 * structure-of-arrays.  Plain pointers and sizes only; no torch or CUDA types
 * in the signatures (a CUDA stream is passed as `void*`).
 *
 * Semantics follow the reference: Levenberg–Marquardt over camera poses,
 * shared lens intrinsics (f, k1, k2) and points, a robust loss on
 * reprojection residuals and GPS priors on camera centres, points eliminated
 * by the Schur complement, the reduced camera(+lens) system solved by
 * block-Jacobi PCG (ba.rs:155-196), then point back-substitution.  The state
 * (`rot`, `center`, `points`, and `intr` when refining) is updated in place;
 * observations, groups and priors are read only.
 *
 * Unlike the reference, which cannot fail, every entry point returns a
 * status; the message of the last failure on the calling thread is available
 * from ba_last_error().  There is no CPU fallback: without a usable GPU the
 * calls fail with BA_CUDA_ERROR.
 *
 * Layouts (host or device memory as stated per call):
 *   obs_cam   u32[n_obs]          camera of each observation
 *   obs_pt    u32[n_obs]          point of each observation, non-decreasing
 *                                 (ba.rs:36: "Sorted by point")
 *   obs_uv    f64[2*n_obs]        measured pixel (u, v)
 *   cam_group u32[n_cams]         lens group of each camera (ba.rs:31-32)
 *   prior_mask u8[n_cams]         1 = camera has a GPS prior (may be NULL)
 *   prior     f64[6*n_cams]       prior centre xyz, then sigma xyz (ba.rs:33-34)
 *   rot       f64[9*n_cams]       world->camera rotation, ROW-major
 *                                 (nalgebra stores column-major: transpose)
 *   center    f64[3*n_cams]       camera centre in world coordinates
 *   intr      f64[5*n_groups]     f, cx, cy, k1, k2 (geometry.rs:15-23)
 *   points    f64[3*n_points]
 */
#ifndef BA_GB300_H
#define BA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BA_GB300_ABI_VERSION 1

typedef enum ba_status {
  BA_OK = 0,
  BA_BAD_INPUT = 1,     /* sizes, indices, ordering or options rejected   */
  BA_OOM = 2,           /* device memory could not be allocated           */
  BA_CUDA_ERROR = 3,    /* no device, launch failure, or device error     */
  BA_TIMEOUT = 4,       /* a device-side wait gave up (error flag)        */
  BA_NOT_SUPPORTED = 5  /* option combination not implemented             */
} ba_status;

typedef enum ba_loss {
  BA_LOSS_CAUCHY = 0, /* the reference's loss: s^2 ln(1 + e^2/s^2) (ba.rs:99,114) */
  BA_LOSS_HUBER = 1   /* Huber with delta = sigma_px (not in the reference)       */
} ba_loss;

typedef enum ba_precision {
  BA_PRECISION_FP64 = 0,  /* plain form: FP64 throughout                     */
  BA_PRECISION_MIXED = 1  /* FP32 Jacobians / Schur blocks / PCG vectors;
                             FP64 cost, PCG inner products, block inverses */
} ba_precision;

/* ba.rs:28-39 (`Problem`, read-only parts). */
typedef struct ba_problem {
  int64_t n_cams, n_points, n_obs, n_groups;
  const uint32_t* obs_cam;
  const uint32_t* obs_pt;
  const double* obs_uv;
  const uint32_t* cam_group;
  const uint8_t* prior_mask; /* NULL: no camera has a prior */
  const double* prior;
  int32_t refine_intrinsics; /* ba.rs:38 */
} ba_problem;

/* ba.rs:28-39 (`Problem`, the parts bundle_adjust mutates). */
typedef struct ba_state {
  double* rot;
  double* center;
  double* intr;
  double* points;
} ba_state;

/* Optional per-LM-iteration log, caller-owned arrays of `cap` entries. */
typedef struct ba_log {
  int32_t cap;
  double* new_cost;   /* robust cost of the trial state                 */
  double* lambda;     /* damping used to build the iteration's system   */
  int32_t* pcg_iters; /* PCG matrix-vector products                     */
  int32_t* accepted;  /* 1 if the trial state was accepted              */
} ba_log;

typedef struct ba_options {
  int32_t max_iter;     /* ba.rs:198 `max_iter`                            */
  double sigma_px;      /* ba.rs:198 `sigma_px` (loss scale, pixels)       */
  int32_t loss;         /* ba_loss, default BA_LOSS_CAUCHY                 */
  int32_t precision;    /* ba_precision, default BA_PRECISION_FP64         */
  int32_t pcg_max_iter; /* <=0: 400 (ba.rs:334)                            */
  double pcg_tol;       /* <=0: 1e-20, on |r|^2 / |b|^2 (ba.rs:182)        */
  int32_t matrix_free;  /* 0: auto (by memory cap), 1: stored S, 2: matrix-free
                           (S p applied from the per-observation Schur factors;
                           one model with at most one lens group), 3: the same
                           with J^T J recomputed in every product from the
                           stored FP32 Jacobians (mixed form; no Schur factors
                           stored; the results of mode 2)                  */
  int64_t memory_cap_bytes; /* auto mode: go matrix-free when the Schur pair list
                           and reduced matrix would exceed this (<=0: no cap) */
  void* stream;         /* cudaStream_t to run on, NULL: the library's own */
  ba_log* log;          /* NULL or per-iteration log (single-model calls)  */
  int32_t profile;      /* 1: time each kernel phase with CUDA events      */
  int32_t pcg_kernel;   /* 0: auto (mixed form: cluster kernel when every
                           model fits, else grid), 1: grid-wide kernel,
                           2: one thread-block cluster per model (mixed
                           form; BA_NOT_SUPPORTED when a model does not fit),
                           512 threads per CTA; 3: the same with 1024
                           threads per CTA (a warp per block row)        */
  int32_t no_graph;     /* 1: launch each kernel directly instead of replaying
                           a CUDA graph of the LM iteration                */
  int32_t autotune;     /* 1: before the first solve of a form on a context,
                           time the Schur sub-segment lengths (pairs per
                           warp) and the PCG configurations (grid rows per
                           CTA, cluster sizes) on its first system and keep
                           the fastest for this and later solves          */
  int32_t stop_patience; /* LM stops after this many consecutive accepted
                           steps with relative decrease < 1e-6; 0 or 1:
                           the reference's rule (ba.rs:372-374)          */
  int32_t coarse;       /* mixed form, cluster PCG: 1 adds a coarse correction
                           to the block-Jacobi preconditioner (the seven
                           similarity motions of each group of consecutive
                           cameras, up to 32 groups per model); 0: the
                           reference's block-Jacobi alone                 */
  int32_t fault_hold_pcg_cta; /* fault injection for tests of the timeout
                           path: k > 0 makes CTA k-1 of the grid-kernel PCG
                           launch leave before its first group exchange, so
                           the other CTAs of its group wait until
                           wait_limit_cycles runs out and the call returns
                           BA_TIMEOUT with the host state untouched; 0: off */
  int64_t wait_limit_cycles; /* spin limit of every device-side wait, in SM
                           clock cycles; <= 0: 4e9 (about 2 s)            */
  int64_t workspace_limit_bytes; /* device memory the call may hold at once
                           (problem copies and workspace); an allocation
                           beyond it fails with BA_OOM before it is made;
                           <= 0: no limit                                 */
  int32_t pcg_end_max_iter; /* end-game PCG cap: once an accepted LM step
                           decreases a model's cost by less than
                           pcg_end_rel (relative), that model's PCG runs up
                           to this many iterations per solve for the rest of
                           the call (tighter inner solves as the outer
                           iteration converges); 0: off                   */
  double pcg_end_rel;   /* <= 0: 1e-5                                      */
  int32_t point_kernel; /* mixed form, per-observation passes (ba.rs:222-268):
                           0: auto (the autotuner's choice, else the three
                           kernels), 1: three kernels (records,
                           point systems, Schur factors), 2: the three fused
                           in one kernel over 128-observation chunks, 3: the
                           same over 256-observation chunks (bit-identical
                           results; the fused kernels keep the records on chip) */
} ba_options;

/* Kernel phases timed when ba_options.profile is set (ba_stats.ms_phase). */
enum {
  BA_PHASE_POINT = 0,    /* linearise + per-point blocks (ba.rs:222-268)   */
  BA_PHASE_CAMERA = 1,   /* per-camera and per-lens sums (ba.rs:273-292)   */
  BA_PHASE_SCHUR = 2,    /* Schur products (ba.rs:320-331)                 */
  BA_PHASE_ASSEMBLE = 3, /* reduced matrix, rhs, damping, preconditioner   */
  BA_PHASE_PCG = 4,      /* block-Jacobi PCG (ba.rs:155-196)               */
  BA_PHASE_UPDATE = 5,   /* pose update + back-substitution (ba.rs:338-366)*/
  BA_PHASE_COST = 6,     /* robust cost of the trial state (ba.rs:367)     */
  BA_PHASE_CONTROL = 7,  /* accept / reject (ba.rs:368-383)                */
  BA_PHASE_SETUP = 8,    /* per-call structure build                       */
  BA_N_PHASES = 9
};

/* ba.rs:41-46 (`BaStats`) plus solver diagnostics. */
typedef struct ba_stats {
  int64_t iterations;  /* ba.rs:43 */
  double initial_rms;  /* ba.rs:44 */
  double final_rms;    /* ba.rs:45 */
  double initial_cost, final_cost;
  int64_t pcg_iterations; /* total PCG matrix-vector products              */
  int64_t kernel_launches;/* kernels launched by this call                 */
  double ms_total;        /* wall time of the call (host clock)            */
  double ms_h2d, ms_d2h;  /* host<->device copies inside the call          */
  int64_t h2d_bytes, d2h_bytes;
  int64_t device_bytes;   /* peak device workspace of the call             */
  double ms_phase[9];     /* per-phase device time (profile only)          */
  int64_t n_phase[9];     /* launches timed per phase (profile only)       */
  /* Size of the reduced system the call built (whole batch). */
  int64_t n_blocks;       /* block rows: cameras + lens groups             */
  int64_t n_nonzero_blocks;  /* 6x6 blocks of the symmetric matrix (full)  */
  int64_t n_schur_pairs;  /* point-entry pairs summed into upper blocks    */
  int64_t n_lens_entries; /* per-point lens entries                        */
  int32_t pcg_kernel;     /* PCG kernel that ran: 1 grid-wide, 2 cluster,
                             3 matrix-free (reduced matrix not formed)     */
  int32_t pcg_cluster;    /* CTAs per cluster (cluster kernel), else 0     */
  int32_t graph;          /* 1 if the LM iterations replayed a CUDA graph  */
  int32_t pcg_ctas;       /* CTAs of the PCG launch                        */
  double pcg_tuned_us;    /* autotuner's time per PCG iteration (0: none)  */
  int32_t pcg_coarse_dim; /* coarse unknowns of the two-level preconditioner
                             (largest model), 0: block-Jacobi alone       */
  int32_t schur_sub_len;  /* Schur pair contributions per warp sub-segment
                             (chosen by the autotuner, else 512)          */
  double schur_tuned_us;  /* autotuner's Schur kernel time (0: not tuned) */
  int32_t pcg_threads;    /* threads per CTA of the PCG launch (the cluster
                             kernel: 512 or 1024, chosen by the autotuner) */
  int32_t point_kernel;   /* mixed form's per-observation passes that ran
                             (ba_options.point_kernel numbering), else 0 */
  double point_tuned_us;  /* autotuner's time of those passes (0: not tuned) */
} ba_stats;

/* Defaults: max_iter 60, sigma_px 1, Cauchy, FP64, PCG 400 / 1e-20. */
void ba_default_options(ba_options* opt);

/* Solve one problem from HOST memory, updating `state` in place.
 * Replaces ba.rs:198 `bundle_adjust`. */
ba_status ba_solve(const ba_problem* problem, ba_state* state,
                   const ba_options* opt, ba_stats* stats);

/* Solve `n_models` independent problems (host memory) in one batched launch
 * sequence: every kernel covers all models, each model keeps its own damping,
 * PCG scalars and stopping state.  `stats` has n_models entries (may be NULL).
 * No counterpart in the reference, which solves one Problem per call
 * (sparse.rs:450); each model gives the same result as its own ba_solve. */
ba_status ba_solve_batch(const ba_problem* problems, ba_state* states,
                         int32_t n_models, const ba_options* opt,
                         ba_stats* stats);

/* ---- device-resident context (inputs stay in HBM between calls) ---------- */

typedef struct ba_context ba_context;

/* device < 0: the current device.  stream: NULL for a library-owned stream. */
ba_status ba_context_create(int32_t device, void* stream, ba_context** out);
void ba_context_destroy(ba_context* ctx);

/* Copy problems and initial states from host memory into the context. */
ba_status ba_context_upload(ba_context* ctx, const ba_problem* problems,
                            const ba_state* states, int32_t n_models);

/* Solve the uploaded problems starting from their uploaded initial states
 * (the initial states stay intact, so repeated calls solve the same problem).
 * Everything — structure, linearisation, Schur complement, PCG, updates —
 * runs on the device; only per-iteration control scalars are read back. */
ba_status ba_context_solve(ba_context* ctx, const ba_options* opt,
                           ba_stats* stats);

/* Copy the solved states back into host memory. */
ba_status ba_context_download(ba_context* ctx, ba_state* states,
                              int32_t n_models);

/* Gradient of the robust cost at the context's current (solved) state with
 * respect to each lens group's intrinsics (f, cx, cy, k1, k2): the adjoint
 * (vector-Jacobian product) of reprojection + distortion residuals; GPS
 * priors do not depend on intrinsics.  At a converged solve in which the
 * intrinsics were held fixed this is also the total derivative of the final
 * cost (the poses and points are stationary).  grad: f64[5 * total groups],
 * host memory.  No counterpart in the reference. */
ba_status ba_context_intrinsics_grad(ba_context* ctx, const ba_options* opt,
                                     double* grad);

/* Vector-Jacobian product of the residuals at the context's current state.
 * Residuals: e_k = u_k − pred_k per observation in front of its camera
 * (ba.rs:56-101) and r_c = (C_c − prior_c) / sigma_c per prior axis
 * (ba.rs:120-126).  With cotangents lambda (f64[2*n_obs]) and mu
 * (f64[3*n_cams]) it returns sum (de/dθ)^T lambda + sum (dr/dθ)^T mu for
 * θ = camera (rotation as the left perturbation R <- exp(w) R, then centre;
 * f64[6*n_cams]), points (f64[3*n_points]) and lens intrinsics
 * (f, cx, cy, k1, k2; f64[5*n_groups]).  lambda == NULL and mu == NULL give
 * the gradient of the robust cost.  Host arrays; outputs may be NULL.
 * No counterpart in the reference. */
ba_status ba_context_vjp(ba_context* ctx, const ba_options* opt,
                        const double* cot_obs, const double* cot_prior,
                        double* g_cam, double* g_points, double* g_intr);

/* Per-observation residual and Jacobians at the context's current state,
 * as the reference's linearise (ba.rs:56-101) defines them, written to host
 * arrays: e f64[2n], jc f64[12n] (2x6 row-major: rotation | centre),
 * jg f64[6n] (2x3: f, k1, k2), jp f64[6n], w f64[n], valid u8[n]. */
ba_status ba_context_linearise(ba_context* ctx, const ba_options* opt,
                               double* e, double* jc, double* jg, double* jp,
                               double* w, uint8_t* valid);

/* Robust cost (ba.rs:103-128) at the context's current state, per model:
 * cost (incl. priors), rms and in-front count; host arrays of n_models. */
ba_status ba_context_cost(ba_context* ctx, const ba_options* opt,
                          double* cost, double* rms, int64_t* n_in_front);

/* One LM system at damping `lambda` built at the context's uploaded state
 * (single model), solved by PCG and applied, without the accept step:
 * the dense reduced matrix S f64[(6 nb)^2] (row-major, may be NULL; for small
 * problems), the right-hand side g f64[6 nb], the step dx f64[6 nb], the PCG
 * iteration count and the robust cost of the trial state.  nb = n_cams +
 * n_groups, blocks ordered as in ba.rs:199-201.  A diagnostic for
 * element-wise checks of ba.rs:221-367; no counterpart in the reference. */
ba_status ba_context_debug_step(ba_context* ctx, const ba_options* opt,
                                double lambda, double* S_dense, double* g,
                                double* dx, int32_t* pcg_iters,
                                double* trial_cost);

/* Robust cost (ba.rs:103-128) of one problem whose arrays (every pointer in
 * `problem` and `state`) are already in DEVICE memory, computed without
 * allocating: for callers that cannot call cudaMalloc — a host whose device
 * memory is all held by another runtime's caching allocator, or a
 * latency-critical loop where cudaMalloc / cudaFree would synchronise the
 * whole device.  Runs on `stream` (NULL: the legacy default stream) on the
 * current device, then copies the result to host memory and synchronises
 * that stream: it must not be called while the stream is being captured
 * into a CUDA graph.
 * Scratch: a fixed 262,176-byte device array per device, part of this
 * library's device code.  With lazy module loading (the CUDA default) the
 * array is reserved when the first call on a device looks up its address,
 * so make one call on each device (n_obs = 0 is enough) before another
 * runtime takes the rest of its memory.  At most 33,554,432 observations
 * per call (BA_BAD_INPUT beyond).  Observation camera / point and camera
 * lens-group indices are checked on the device: an index out of range gives
 * BA_BAD_INPUT.  Calls share the scratch: calls that overlap on the GPU
 * race.  No counterpart in the reference. */
ba_status ba_robust_cost_noalloc(const ba_problem* problem, const ba_state* state,
                                 double sigma_px, int32_t loss, void* stream,
                                 double* cost, double* rms, int64_t* n_in_front);

/* ---- triangulation and gating of a sparse-stage round ---------------------- */

/* Feature tracks of the sparse stage (sparse.rs:389): track t's observations
 * are obs_cam / obs_uv[track_ptr[t] .. track_ptr[t+1]).  Pixels are full
 * resolution, distorted (as matched). */
typedef struct ba_tracks {
  int64_t n_tracks, n_obs, n_cams, n_groups;
  const uint32_t* track_ptr; /* n_tracks + 1 */
  const uint32_t* obs_cam;   /* n_obs */
  const double* obs_uv;      /* 2 * n_obs */
  const uint32_t* cam_group; /* n_cams */
} ba_tracks;

/* One round's triangulation and reprojection gating of every track
 * (sparse.rs:389-421): linear triangulation from the undistorted observations
 * (geometry.rs:115-144), observations kept if they reproject within thr_px,
 * track kept if two or more remain and their rays span more than 2 degrees
 * (three or more views) or 6 degrees (two views; geometry.rs:146-156).
 * Cameras: rot f64[9 n_cams] (row-major), center f64[3 n_cams], intr
 * f64[5 n_groups].  Host (or device) inputs; outputs (host, may be NULL):
 * kept u8[n_tracks], points f64[3 n_tracks], good u8[n_obs], n_kept.
 * Replaces the reference's per-round closure at sparse.rs:389-421. */
ba_status ba_triangulate(const ba_tracks* tracks, const double* rot, const double* center,
                         const double* intr, double thr_px, void* stream, uint8_t* kept,
                         double* points, uint8_t* good, int64_t* n_kept);

/* Triangulate and gate as ba_triangulate, then build the round's bundle
 * adjustment problem in the context's device memory (sparse.rs:429-449:
 * points of the kept tracks in track order, their kept observations sorted
 * by point; cameras and groups as given; priors optional) without a round
 * trip through the host.  `cams`: rot, center, intr (points ignored).  Then
 * ba_context_solve / ba_context_download as after ba_context_upload.
 * n_points / n_obs receive the problem's sizes.  No counterpart in the
 * reference, which builds the Problem on the host. */
ba_status ba_context_upload_tracks(ba_context* ctx, const ba_tracks* tracks,
                                   const ba_state* cams, const uint8_t* prior_mask,
                                   const double* prior, int32_t refine_intrinsics,
                                   double thr_px, int64_t* n_points, int64_t* n_obs);

/* ---- epipolar geometry of photo pairs ------------------------------------ */

/* Putative or verified matches of photo pairs: pair p joins cameras
 * pair_cam[2p] (i) and pair_cam[2p+1] (j) and owns the correspondences
 * match_ptr[p] .. match_ptr[p+1] of uv, each (u_i, v_i, u_j, v_j) in
 * full-resolution pixels (the keypoints the reference indexes with its
 * (u32, u32) match pairs, gathered).  seed: per-pair RANSAC seeds; NULL
 * means i * 7919 + j (sparse.rs:290).  Host or device pointers. */
typedef struct ba_pair_matches {
  int64_t n_pairs, n_matches;
  const uint32_t* pair_cam;  /* 2 n_pairs (may be NULL for RANSAC when seed is given) */
  const uint32_t* match_ptr; /* n_pairs + 1, from 0 to n_matches */
  const double* uv;          /* 4 n_matches */
  const uint64_t* seed;      /* n_pairs or NULL */
} ba_pair_matches;

/* Fundamental-matrix RANSAC of every pair (ransac_fundamental,
 * geometry.rs:248-300, as sparse.rs:290 calls it per pair: thresh_px 1.5,
 * iters 600): xorshift64 samples of eight distinct correspondences, the
 * normalised 8-point F with rank 2 enforced, inliers by squared Sampson
 * distance < thresh_px^2; the first hypothesis with the most inliers wins and
 * one refit on its inliers is kept when it has at least as many.  Pairs with
 * fewer than 12 correspondences get none.  Outputs (host or device, may be
 * NULL): inlier u8[n_matches], n_inliers i32[n_pairs], best_hypothesis
 * i32[n_pairs] (-1: none), refit u8[n_pairs].  The sparse stage keeps a
 * pair's inliers when there are at least 20 (sparse.rs:291-297).
 * Replaces the per-pair call at sparse.rs:290. */
ba_status ba_ransac_fundamental(const ba_pair_matches* m, double thresh_px, int32_t iters,
                                void* stream, uint8_t* inlier, int32_t* n_inliers,
                                int32_t* best_hypothesis, uint8_t* refit);

/* pair_fits (sparse.rs:620-645) of every pair under the current poses: the
 * median (element n/2 in total order) of sqrt(Sampson) * f_i of the pair's
 * matches for E = [t]x R, R = R_j R_i^T, t = R_j (C_i - C_j), on undistorted
 * normalised coordinates; DBL_MAX for a pair without matches.  Cameras: rot
 * f64[9 n_cams] (row-major), center f64[3 n_cams], intr f64[5 n_groups],
 * cam_group u32[n_cams].  Output median_px f64[n_pairs].  The sparse stage
 * drops pairs whose median is not below 6 px at its working scale
 * (sparse.rs:362-373).  Replaces the retain closure at sparse.rs:362-373. */
ba_status ba_pair_fits(const ba_pair_matches* m, const double* rot, const double* center,
                       const double* intr, const uint32_t* cam_group, int64_t n_cams,
                       int64_t n_groups, void* stream, double* median_px);

/* ---- sparse-stage outputs ------------------------------------------------- */

/* Per-camera summary of a finished sparse reconstruction, the fields of
 * cameras.json that come from the bundle-adjusted problem (sparse.rs:470-483
 * and 515-533), and the f32 points of sparse.ply (mod.rs:31-35).
 *   neighbours u32[n_cams * max_neighbours]: the cameras sharing the most
 *     points with each camera, best first (equal counts by ascending camera
 *     index, which the reference leaves to HashMap order), UINT32_MAX padded;
 *   shared u32[n_cams * max_neighbours]: those point counts, 0 padded;
 *   n_neighbours i32[n_cams];
 *   depth_range f64[2 n_cams]: (d[n/20] * 0.8, d[19n/20] * 1.25) of the
 *     sorted camera-frame depths of the camera's observed points when there
 *     are ten or more, else (0.3 agl, 3 agl);
 *   points_f32 f32[3 n_points]: the points rounded to f32.
 * Uses obs_cam, obs_pt (sorted by point) of `problem` and rot, center, points
 * of `state`; host or device pointers.  Outputs (may be NULL) are host or
 * device pointers.  max_neighbours in 1..64 (the reference keeps 8).
 * Replaces the host loops at sparse.rs:470-483 and 515-533 and the f32
 * conversion at mod.rs:31-35. */
ba_status ba_sparse_summary(const ba_problem* problem, const ba_state* state,
                            int32_t max_neighbours, double agl, void* stream,
                            uint32_t* neighbours, uint32_t* shared, int32_t* n_neighbours,
                            double* depth_range, float* points_f32);

/* ba_sparse_summary of the single model held by a context, with its current
 * (solved) state: a round's result summarised without leaving the device. */
ba_status ba_context_sparse_summary(ba_context* ctx, int32_t max_neighbours, double agl,
                                    uint32_t* neighbours, uint32_t* shared,
                                    int32_t* n_neighbours, double* depth_range,
                                    float* points_f32);

/* JSON text of an array as cameras.json holds it (mod.rs:30,
 * `serde_json::to_vec(&Sparse)`): "[a,b,c]" when group == 0, else rows of
 * `group` values "[[a,b,c],[d,e,f]]".  f64 values in the shortest text that
 * reads back exactly, in serde_json's layout (1.0, 0.001, 1e-7, 1.5e300;
 * non-finite as null); integers in decimal.  `cap` must be at least
 * n*(w+1) + 2*(n/group) + 3 bytes, w = 25 (f64), 3 (u8), 10 (u32); the text
 * is NUL-terminated and *len receives its length.  Host code only. */
ba_status ba_json_f64(const double* v, int64_t n, int32_t group, char* out, int64_t cap,
                      int64_t* len);
ba_status ba_json_u8(const uint8_t* v, int64_t n, int32_t group, char* out, int64_t cap,
                     int64_t* len);
ba_status ba_json_u32(const uint32_t* v, int64_t n, int32_t group, char* out, int64_t cap,
                      int64_t* len);

/* ---- misc ----------------------------------------------------------------- */

const char* ba_last_error(void);
int32_t ba_abi_version(void);
const char* ba_version(void);

#ifdef __cplusplus
}
#endif

#endif /* BA_GB300_H */
