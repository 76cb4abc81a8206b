/*
 * gba.h -- C ABI of the GB300 bundle-adjustment engine (libgba.so).
 *
 * The engine replaces the Levenberg-Marquardt bundle-adjustment path of
 * hs_sfm (include/hs_sfm/bundle_adjustment/camera_shared_*): the
 * camera-shared projection model, its analytical Jacobian, the block
 * normal equations, the Schur-complement reduced camera system and the
 * damped LM driver.  Everything here is plain C: pointers, sizes and status
 * codes, no C++ or torch types, no exceptions.
 *
 * Layout conventions follow the reference exactly so that a caller holding
 * the reference containers can pass them without copying:
 *   - feature_maps  = std::vector<std::pair<Index,Index>> (image_id, point_id)
 *     (camera_shared_vector_function.hpp:36-37), Index = ptrdiff_t (int64);
 *   - image_camera_map = std::vector<Index> (camera_shared_vector_function.hpp:39);
 *   - x = [points 3P][images 6I][cameras cC], each block dropped when fixed
 *     (camera_shared_vector_function.hpp:349-410);
 *   - image = (angle-axis r[3], translation t[3]), camera point = R(r) X + t
 *     (camera_shared_vector_function.hpp:688-710);
 *   - camera = [k1 k2 k3][d1 d2][f s cx cy a], each group present when its
 *     bit of the intrinsic mask is set (camera_shared_vector_function.hpp:247-263);
 *   - y = [keys 2K][point constraints][image constraints][camera constraints]
 *     (camera_shared_vector_function.hpp:412-632).
 */
#ifndef GBA_H_
#define GBA_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define GBA_API __attribute__((visibility("default")))
#else
#define GBA_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (0 / -1 are the reference's Err values) ------------- */
#define GBA_OK                 0
#define GBA_ERR               -1  /* generic failure (reference's -1)       */
#define GBA_ERR_INVALID       -2  /* size mismatch / bad argument           */
#define GBA_ERR_BAD_INDEX     -3  /* image/point/camera id out of range     */
#define GBA_ERR_DUPLICATE     -4  /* the same (image, point) key twice      */
#define GBA_ERR_UNSUPPORTED   -5  /* model variant not built on the GPU     */
#define GBA_ERR_NOT_SPD       -6  /* reduced system not positive definite   */
#define GBA_ERR_NAN           -7  /* non-finite residual or cost            */
#define GBA_ERR_OOM           -8  /* device allocation failed               */
#define GBA_ERR_CUDA          -9  /* CUDA runtime error                     */
#define GBA_ERR_TIMEOUT      -10  /* a bounded device wait ran out          */
#define GBA_ERR_NO_DEVICE    -11  /* no CUDA device visible                 */
#define GBA_ERR_BUSY         -12  /* admission refused (slots or memory)    */
#define GBA_ERR_CANCELLED    -13  /* request cancelled before it finished   */

/* ---- masks (camera_shared_common_types.hpp:14-104) --------------------- */
#define GBA_COMPUTE_RADIAL_DISTORTION       (1u << 0)
#define GBA_COMPUTE_DECENTERING_DISTORTION  (1u << 1)
#define GBA_COMPUTE_INTRINSIC_PARAMS        (1u << 2)

#define GBA_FIX_POINTS   (1u << 0)
#define GBA_FIX_IMAGES   (1u << 1)
#define GBA_FIX_CAMERAS  (1u << 2)

#define GBA_POINT_CONSTRAIN_X  (1u << 0)
#define GBA_POINT_CONSTRAIN_Y  (1u << 1)
#define GBA_POINT_CONSTRAIN_Z  (1u << 2)

#define GBA_IMAGE_CONSTRAIN_ROTATION    (1u << 0)
#define GBA_IMAGE_CONSTRAIN_POSITION_X  (1u << 1)
#define GBA_IMAGE_CONSTRAIN_POSITION_Y  (1u << 2)
#define GBA_IMAGE_CONSTRAIN_POSITION_Z  (1u << 3)

typedef struct gba_point_constraint {   /* PointConstraint, :30-34 */
  int64_t point_id;
  uint32_t mask;                        /* GBA_POINT_CONSTRAIN_* */
  uint32_t pad_;
} gba_point_constraint;

typedef struct gba_image_constraint {   /* ImageConstraint, :45-49 */
  int64_t image_id;
  uint32_t mask;                        /* GBA_IMAGE_CONSTRAIN_* */
  uint32_t pad_;
} gba_image_constraint;

typedef struct gba_camera_constraint {  /* CameraConstraint, :88-94 */
  int64_t camera_id;
  uint32_t radial_mask;                 /* bits k1 k2 k3 */
  uint32_t decentering_mask;            /* bits d1 d2 */
  uint32_t intrinsic_mask;              /* bits f s cx cy a */
  uint32_t pad_;
} gba_camera_constraint;

/*
 * One bundle-adjustment problem: the content of a
 * CameraSharedVectorFunction<double> (camera_shared_vector_function.hpp:746-763)
 * plus the inverse observation covariance of
 * CameraSharedYCovarianceInverse<double> (camera_shared_y_covariance_inverse.hpp:146-148).
 * All pointers are host pointers owned by the caller; the library copies
 * what it needs and never keeps them past the call that received them.
 */
typedef struct gba_problem {
  int64_t number_of_points;
  int64_t number_of_images;
  int64_t number_of_cameras;
  int64_t number_of_keys;
  const int64_t* feature_maps;      /* [2*K] (image_id, point_id) per key   */
  const int64_t* image_camera_map;  /* [I] camera id of each image          */
  uint32_t intrinsic_computations_mask;
  uint32_t fix_mask;
  const double* fix_points;         /* [3P]  used when GBA_FIX_POINTS       */
  const double* fix_images;         /* [6I]  used when GBA_FIX_IMAGES       */
  const double* fix_cameras;        /* [cC]  used when GBA_FIX_CAMERAS      */
  int64_t number_of_point_constraints;
  const gba_point_constraint* point_constraints;
  int64_t number_of_image_constraints;
  const gba_image_constraint* image_constraints;
  int64_t number_of_camera_constraints;
  const gba_camera_constraint* camera_constraints;
  /* Inverse covariance: per-key 2x2 row-major blocks [4K] (NULL = identity
   * for every key) and one weight per constraint row [y_size - 2K]
   * (NULL = 1 for every constraint row). */
  const double* key_covariance_inverse;
  const double* constraint_weights;
  /* Point priors: the ground control points of the GCP-constrained model
   * (ba_gcp_constrained_vector_function.hpp:60-110,
   * ba_gcp_constrained_normal_equation_builder.hpp:42-75).  y holds the
   * observed coordinates of each prior's point, 3 rows per prior after the
   * constraint rows, weighted by the prior's full 3x3 inverse covariance
   * (ba_gcp_constrained_y_covariance_inverse.hpp:18-25); points must be free. */
  int64_t number_of_point_priors;
  const int64_t* point_prior_ids;          /* [n] point ids */
  const double* point_prior_information;   /* [9n] row-major 3x3; NULL = identity */
} gba_problem;

/* Sizes derived from a problem (GetXSize / GetYSize,
 * camera_shared_vector_function.hpp:237-362). */
GBA_API int64_t gba_params_per_camera(uint32_t intrinsic_computations_mask);
GBA_API int64_t gba_x_size(const gba_problem* problem);
GBA_API int64_t gba_y_size(const gba_problem* problem);

/* ---- solver options ------------------------------------------------------ */
#define GBA_PRECISION_FP64   0   /* every stage in FP64 (the drop-in path)  */
#define GBA_PRECISION_MIXED  1   /* FP32 Jacobian/Schur, FP64 master x,
                                    cost sum and reduced-system factor     */

#define GBA_LOSS_TRIVIAL 0
#define GBA_LOSS_HUBER   1       /* rho(s)=s (s<=d^2), 2d*sqrt(s)-d^2 else */

#define GBA_LINEAR_DENSE_CHOLESKY 0
#define GBA_LINEAR_PCG            1  /* block-Jacobi PCG on the explicit
                                        block-sparse reduced system        */

#define GBA_Z_AUTO    0
#define GBA_Z_RECORDS 1  /* per-key records in key (point) order           */
#define GBA_Z_PLANES  2  /* nine planes of value pairs, keys image by image */

typedef struct gba_options {
  /* LevenbergMarquardt(max_itr_num, tau, eps1, eps2)
   * (camera_shared_levenberg_marquardt_optimizor.hpp:36-41). */
  int32_t max_iterations;
  double tau;
  double eps1;
  double eps2;
  int32_t precision;          /* GBA_PRECISION_*                            */
  int32_t loss;               /* GBA_LOSS_*                                 */
  double huber_delta;         /* pixels (whitened)                          */
  int32_t linear_solver;      /* GBA_LINEAR_*                               */
  int32_t pcg_max_iterations;
  double pcg_relative_tolerance;
  int32_t use_cuda_graph;     /* capture each LM iteration once, replay     */
  int32_t profile;            /* record per-stage CUDA events               */
  int32_t device;             /* CUDA device ordinal                        */
  /* 1: other plans may run on the device at the same time (the server sets
   * it); the grid-wide dataflow factorization, which wants every SM, is then
   * not used. */
  int32_t shared_device;
  /* Stop after an accepted step whose cost decrease is at most this
   * fraction of the cost before it (Ceres' function_tolerance,
   * camera_shared_ceres_optimizor.hpp:478); 0 disables the test. */
  double function_tolerance;
  /* Work-item sizes of the two reductions split into per-warp items: key
   * pairs per Schur-assembly item (0: 1024) and keys per image-reduction
   * item (0: 512).  They change the grouping (and so the rounding) of the
   * block sums, not the model; gba_autotune picks them for a batch. */
  int32_t pair_item;
  int32_t image_item;
  /* Keys per key work chunk (0: 1024): the unit of the cost, Jacobian and
   * Z kernels and of the cost's partial sums (so it changes the rounding of
   * the cost sum, not the model); gba_autotune picks it with the others. */
  int32_t key_item;
  /* Layout of the Schur assembly's per-key records (GBA_Z_*): where they
   * lie in memory, not their values or the sums' order (the same bits
   * either way).  0 (auto): image-major planes when a block's key pairs
   * cover a large share of its images' keys (small dense windows), else
   * records in key order; gba_autotune times both. */
  int32_t z_layout;
} gba_options;

/* Autotuning of the work-item sizes (gba_options.pair_item / image_item /
 * key_item) for a batch: every candidate builds a plan of the given
 * problems (initial x0 per problem) with the given options (at most two LM
 * iterations, stopping tests off, graph replay), runs it once to warm up and
 * is timed over three graph replays (CUDA events on the plan's stream);
 * pair_item is searched first over {256, 512, 1024, 2048, 4096} with the
 * default image_item and key_item, then image_item over {256, 512, 1024}
 * with the best pair_item, then key_item over {256, 512, 1024, 2048} with
 * the best two, then (options->z_layout auto) the other Z layout with the
 * best sizes.  out receives the fastest sizes and layout and their time per
 * LM iteration beside that of the defaults.  A status code. */
typedef struct gba_tuning {
  int32_t pair_item;
  int32_t image_item;
  double ms_per_iteration;           /* the chosen item sizes              */
  double default_ms_per_iteration;   /* pair_item 1024, image_item 512,
                                        key_item 1024                      */
  int32_t candidates;                /* configurations timed               */
  int32_t key_item;
  int32_t z_layout;                  /* GBA_Z_RECORDS or GBA_Z_PLANES      */
  int32_t reserved_[1];
} gba_tuning;

GBA_API int gba_autotune(const gba_problem* problems, const double* const* near_ys,
                         const double* const* x0, int32_t n, const gba_options* options,
                         gba_tuning* out);

/* Fills the defaults used by the reference's relative-pair test
 * (test_camera_shared_relative_pair.cpp:976-979): 50 iterations,
 * tau 1e-3, eps1 1e-8, eps2 1e-8, FP64, trivial loss, dense Cholesky. */
GBA_API void gba_default_options(gba_options* options);

#define GBA_STOP_MAX_ITERATIONS 0
#define GBA_STOP_SMALL_GRADIENT 1
#define GBA_STOP_SMALL_STEP     2
#define GBA_STOP_ERROR          3
#define GBA_STOP_SMALL_COST_CHANGE 4

#define GBA_NUM_STAGES 12
/* stage indices of gba_report.stage_ms */
#define GBA_STAGE_LINEARIZE    0   /* per-point Jacobians, V_p, g_p          */
#define GBA_STAGE_POINT_SCHUR  1   /* C_p, Z, h_p                            */
#define GBA_STAGE_ASSEMBLE     2   /* reduced-system block sums              */
#define GBA_STAGE_FACTOR       3   /* Cholesky column steps + forward solve  */
#define GBA_STAGE_BACKSUB      4   /* point back-substitution and update     */
#define GBA_STAGE_COST         5   /* candidate cost                         */
#define GBA_STAGE_CONTROL      6   /* LM decisions                           */
#define GBA_STAGE_OTHER        7   /* dense reduced system from block sums   */
#define GBA_STAGE_SOLVE        8   /* backward triangular solve              */
#define GBA_STAGE_IMAGE_REDUCE 9   /* U_i, g_i                               */
#define GBA_STAGE_IMAGE_PREP  10   /* image rotations                        */
#define GBA_STAGE_RESERVED    11

typedef struct gba_report {
  int32_t status;             /* GBA_OK or an error code                    */
  int32_t stop_reason;        /* GBA_STOP_*                                 */
  int32_t iterations;         /* LM iterations (accepted + rejected)        */
  int32_t accepted;
  int32_t rejected;
  int32_t factor_failures;    /* non-SPD reduced systems (step rejected)    */
  int32_t pcg_iterations;     /* total over the solve                       */
  int32_t pad_;
  double initial_cost;        /* sum r^T Lambda r (Mahalanobis, no 1/2)     */
  double final_cost;
  double final_rmse;          /* sqrt(sum ||r_key||^2 / K), pixels          */
  double final_mu;
  double final_gradient_inf_norm;
  double setup_ms;            /* structure build + upload                   */
  double solve_ms;            /* LM loop, device time                       */
  double stage_ms[GBA_NUM_STAGES];  /* with options.profile                 */
  int64_t h2d_bytes;          /* host->device bytes copied for this solve   */
  int64_t d2h_bytes;          /* device->host bytes copied for this solve   */
  double queue_ms;            /* server: submit -> admitted                 */
  double latency_ms;          /* server: submit -> result ready             */
} gba_report;

/* ---- one-shot solve: the drop-in for
 * CameraSharedLevenbergMarquardtOptimizor::operator()
 * (camera_shared_levenberg_marquardt_optimizor.hpp:43-58).
 * near_y [y_size] is the observed y; x_inout [x_size] holds the initial x on
 * entry and the optimized x on return.  Host buffers. */
GBA_API int gba_solve(const gba_problem* problem, const double* near_y,
              const gba_options* options, double* x_inout,
              gba_report* report);

/* ---- resident plans: one or many problems kept on the device ----------- */
typedef struct gba_plan gba_plan;

GBA_API int gba_plan_create(const gba_problem* problems, const double* const* near_ys,
                    int32_t number_of_problems, const gba_options* options,
                    gba_plan** plan);
GBA_API int gba_plan_destroy(gba_plan* plan);
GBA_API int gba_plan_number_of_problems(const gba_plan* plan);
/* Copies x0 of every problem (host) to the device and remembers it. */
GBA_API int gba_plan_set_initial_x(gba_plan* plan, int32_t problem, const double* x0);
/* Resets every problem to its remembered x0 and runs the LM solve of all
 * problems together (asynchronous on the plan's stream). */
GBA_API int gba_plan_run(gba_plan* plan);
/* Waits for the plan's stream; returns the first device status seen. */
GBA_API int gba_plan_synchronize(gba_plan* plan);
/* Non-blocking: GBA_OK when the last gba_plan_run has finished on the
 * device, GBA_ERR_BUSY while it is still running. */
GBA_API int gba_plan_query(gba_plan* plan);
GBA_API int gba_plan_get_x(gba_plan* plan, int32_t problem, double* x_out);
/* Every problem at once (x0s / xs [number of problems] host pointers; reports
 * may be NULL): one upload, one device gather and one copy instead of one
 * synchronizing call per problem. */
GBA_API int gba_plan_set_initial_x_all(gba_plan* plan, const double* const* x0s);
GBA_API int gba_plan_get_all(gba_plan* plan, double* const* xs, gba_report* reports);

/* Batched form (create once, submit initial x, poll for the results): the
 * asynchronous face of a plan.  submit uploads every problem's x0 and
 * launches the solve without waiting; poll returns GBA_ERR_BUSY while the
 * device is still solving, else fills xs / reports (as gba_plan_get_all) and
 * returns GBA_OK.  A batch may be submitted again after a poll succeeded. */
typedef struct gba_plan gba_batch;
GBA_API int gba_batch_create(const gba_problem* problems, const double* const* near_ys,
                             int32_t number_of_problems, const gba_options* options,
                             gba_batch** batch);
GBA_API int gba_batch_submit(gba_batch* batch, const double* const* x0s);
GBA_API int gba_batch_poll(gba_batch* batch, double* const* xs, gba_report* reports);
GBA_API int gba_batch_destroy(gba_batch* batch);
GBA_API int gba_plan_get_report(gba_plan* plan, int32_t problem, gba_report* report);
/* Device time of the last gba_plan_run in milliseconds (CUDA events on the
 * plan's stream), and the average duration of the named kernel's launches
 * in that run when options.profile was set (0 when not recorded). */
GBA_API int gba_plan_last_run_ms(gba_plan* plan, double* ms);
GBA_API int gba_plan_kernel_stats(gba_plan* plan, int32_t stage, double* total_ms,
                          int32_t* launches);
/* Counts of this library's kernel launches in the last run. */
GBA_API int gba_plan_last_run_launches(gba_plan* plan, int64_t* launches);
/* Device bytes the plan holds (every buffer of its arena). */
GBA_API int gba_plan_device_bytes(gba_plan* plan, int64_t* bytes);
/* Sizes of a plan's work lists (no counterpart in the reference: the
 * structure the device builds once per plan), for cost models and
 * roofline arithmetic. */
typedef struct gba_plan_structure_info {
  int64_t problems, keys, points, images;
  int64_t key_pairs;        /* (key a, key b) pairs of the Schur assembly    */
  int64_t pair_items;       /* work items of the Schur assembly              */
  int64_t blocks;           /* image-pair blocks of the reduced systems      */
  int64_t image_items;      /* work items of the image reduction             */
  int64_t camera_records;   /* per-point camera records (free cameras)       */
  int64_t max_reduced_size; /* largest reduced system (unknowns)             */
  int64_t factor_schedule;  /* dense factorization: 0 one launch per tile
                               column (batches), 1 one dataflow launch,
                               2 one small-system launch (batches of
                               systems of at most 8 tile rows), -1 PCG     */
  int64_t z_layout;         /* the Schur assembly's records: GBA_Z_RECORDS
                               or GBA_Z_PLANES                             */
  int64_t forked;           /* 1: each LM iteration runs on two streams    */
  int64_t reserved_[1];
} gba_plan_structure_info;
GBA_API int gba_plan_structure(gba_plan* plan, gba_plan_structure_info* out);

/* ---- batched one-shot solve (independent problems, one plan) ----------- */
GBA_API int gba_solve_batch(const gba_problem* problems, const double* const* near_ys,
                    int32_t number_of_problems, const gba_options* options,
                    double* const* x_inout, gba_report* reports);
/* The same with the initial x and the result in separate buffers (x_out[q]
 * may be x0[q]): a caller that keeps its x0 needs no copy of it. */
GBA_API int gba_solve_batch_into(const gba_problem* problems, const double* const* near_ys,
                                 int32_t number_of_problems, const gba_options* options,
                                 const double* const* x0, double* const* x_out, gba_report* reports);

/* ---- single-stage entry points (the trait plug-ins of
 * camera_shared_nllso_meta_levenberg_marquardt.hpp:33-106), used for parity
 * checks of each stage.  Host buffers in and out. ------------------------- */

/* CameraSharedVectorFunction::operator() (:412-632): y [y_size]. */
GBA_API int gba_vector_function(const gba_problem* problem, const double* x,
                        double* y, int32_t precision);

/* CameraSharedAnalyticalJacobianMatrixCalculator (:66-332): per key, in key
 * order, the 2x3 point block, the 2x6 image block and the 2xc camera block,
 * row-major; blocks of fixed parameter groups are not written (pass NULL). */
GBA_API int gba_jacobian(const gba_problem* problem, const double* x,
                 double* point_blocks, double* image_blocks,
                 double* camera_blocks, int32_t precision);

/* Mahalanobis distance sum r^T Lambda r of r = f(x) - near_y
 * (camera_shared_mahalanobis_distance_calculator.hpp:28-58); with a Huber
 * loss each key's term s becomes rho(s). */
GBA_API int gba_cost(const gba_problem* problem, const double* x,
             const double* near_y, const gba_options* options, double* cost);

/* One damped Gauss-Newton step: builds the normal equations at x
 * (camera_shared_normal_equation_builder.hpp:92-108), augments them with mu
 * (camera_shared_augmentor.hpp:22-26) and solves (N + mu I) delta = g by the
 * Schur complement (camera_shared_normal_equation_solver.hpp:75-114).
 * delta_x [x_size]; the LM update is x - delta_x. */
GBA_API int gba_schur_step(const gba_problem* problem, const double* x,
                   const double* near_y, double mu,
                   const gba_options* options, double* delta_x);

/* ---- serving: continuous batching of independent solves ---------------
 * A server owns a worker thread.  Submitted requests (deep-copied) wait in a
 * FIFO queue; whenever device memory (the budget) and in-flight slots allow,
 * the worker admits the queued requests that fit, packs them into one plan
 * (a micro-batch) on its own CUDA stream and launches it while earlier
 * micro-batches are still running, so requests that arrive while others are
 * on the GPU overlap with them.  Finished micro-batches are harvested without
 * blocking the device; their memory returns to the budget.  A request's
 * result does not depend on what it was batched with (every reduction has a
 * fixed order).  Requests larger than the whole budget are refused at submit
 * (GBA_ERR_BUSY). */
typedef struct gba_server gba_server;

typedef struct gba_server_config {
  gba_options solve;              /* options of every request's solve        */
  int64_t memory_budget_bytes;    /* 0: 80% of the free device memory        */
  int32_t max_batch;              /* requests packed into one micro-batch    */
  int32_t max_in_flight;          /* micro-batches running concurrently      */
  int32_t reserved_[6];
} gba_server_config;

typedef struct gba_server_stats {
  int64_t submitted, completed, cancelled, refused;
  int64_t queued, in_flight_requests, in_flight_batches, batches_launched;
  int64_t admitted_bytes, budget_bytes;
} gba_server_stats;

GBA_API void gba_default_server_config(gba_server_config* config);
GBA_API int gba_server_create(const gba_server_config* config, gba_server** server);
GBA_API int gba_server_destroy(gba_server* server);
/* Copies the problem, near_y [y_size] and x0 [x_size]; returns a ticket. */
GBA_API int gba_server_submit(gba_server* server, const gba_problem* problem,
                              const double* near_y, const double* x0, int64_t* ticket);
/* Non-blocking.  GBA_OK: the result is ready -- x_out [x_size] and report
 * are filled and the ticket is released; GBA_ERR_BUSY: still queued or
 * running; GBA_ERR_INVALID: unknown ticket; other codes: the solve failed
 * (the ticket is released). */
GBA_API int gba_server_poll(gba_server* server, int64_t ticket, double* x_out,
                            gba_report* report);
/* As poll, waiting up to timeout_ms (negative: without limit). */
GBA_API int gba_server_wait(gba_server* server, int64_t ticket, double timeout_ms,
                            double* x_out, gba_report* report);
/* A queued request is dropped; a running one finishes but its result is
 * discarded.  Later polls return GBA_ERR_CANCELLED. */
GBA_API int gba_server_cancel(gba_server* server, int64_t ticket);
GBA_API int gba_server_get_stats(gba_server* server, gba_server_stats* stats);
/* Device bytes a plan for this problem would hold (host-side estimate used
 * for admission). */
GBA_API int64_t gba_estimate_device_bytes(const gba_problem* problem, int32_t precision);

/* ---- allocation-free cost ------------------------------------------------
 * No counterpart in the reference: an entry point for callers that must not
 * allocate device memory -- a plugin inside an application that owns every
 * device allocation through its own pool, or code that runs where
 * cudaMalloc is not allowed.  It evaluates the same sum as gba_cost (trivial
 * or Huber loss, identity key weights) for a problem whose arrays the caller
 * already holds in device memory, and writes the sum to d_cost (device).
 * It allocates nothing: its temporaries live in a fixed static device array
 * of libgba.so (about 1.6 MB, held on every GPU that loads the library until
 * exit), so problems are limited to GBA_NOALLOC_MAX_IMAGES images (larger
 * ones return GBA_ERR_INVALID).  Every call shares that array: calls whose
 * work overlaps on the GPU race and must be serialized.  Each call looks up
 * the array's device address on the current device; the first call on a
 * device also loads the library's kernels there, so make it before any
 * stream capture.  Null arrays that a launch would read return
 * GBA_ERR_INVALID before anything is launched.  Ids are checked on the
 * device: a key whose image, point or camera id is out of range is skipped
 * and the cost written is NaN.  `stream` is a cudaStream_t (NULL = default
 * stream); the call only enqueues work. */
#define GBA_NOALLOC_MAX_IMAGES 16384

typedef struct gba_device_problem {
  int32_t number_of_points;
  int32_t number_of_images;
  int32_t number_of_cameras;
  int32_t number_of_keys;
  const int32_t* key_image;    /* device [K] image id of each key           */
  const int32_t* key_point;    /* device [K] point id of each key           */
  const double* keys;          /* device [2K] observed keys                 */
  const int32_t* image_camera; /* device [I] camera id of each image        */
  const double* cameras;       /* device [10C] k1 k2 k3 d1 d2 f s cx cy a   */
  const double* points;        /* device [3P]                               */
  const double* images;        /* device [6I] angle-axis r, translation t   */
} gba_device_problem;

GBA_API int gba_cost_noalloc(const gba_device_problem* problem, int32_t loss,
                             double huber_delta, double* d_cost, void* stream);

/* ---- batched multi-view triangulation ----------------------------------
 * MultipleViewMaximumLikelihoodEstimator / MultipleViewLevenbergMarquardtOptimizor
 * (triangulate/multiple_view_maximum_likelihood_estimator.hpp:32-84,
 * multiple_view_levenberg_marquardt_optimizor.hpp:50-99) for many points at
 * once: each point is initialised by the linear DLT of its undistorted keys
 * (multiple_view_dlt.hpp:27-52, sfm_utility/undistortor.hpp:24-80) and
 * refined by Levenberg-Marquardt on its 3 coordinates against its distorted
 * keys with identity key weights (options: max_iterations, tau, eps1, eps2).
 * Views carry CameraIntrinsicParams and CameraExtrinsicParams
 * (sfm_utility/camera_type.hpp): intrinsics [f skew cx cy pixel_ratio k1 k2
 * k3 d1 d2], extrinsics [rotation (angle-axis, world to camera), position
 * (the camera centre)].  Point j is seen by views track_views[t] with keys
 * track_keys[2t], t in [track_offsets[j], track_offsets[j+1]).  One thread
 * per point, FP64. */
typedef struct gba_triangulation {
  int64_t number_of_views;
  const double* intrinsics;       /* [10 V] */
  const double* extrinsics;       /* [6 V]  */
  int64_t number_of_points;
  const int64_t* track_offsets;   /* [n + 1], ascending, track_offsets[0] = 0 */
  const int64_t* track_views;     /* [m] view of each observation            */
  const double* track_keys;       /* [2 m] observed (distorted) keys         */
} gba_triangulation;

/* points [3n] out; point_status [n] out (may be NULL): GBA_OK, or
 * GBA_ERR_INVALID for a track with fewer than 2 views (the reference's -1),
 * GBA_ERR_NAN when the DLT or the refinement produced no finite point.
 * Returns GBA_OK when the call ran (per-point failures are in point_status),
 * else an input error. */
GBA_API int gba_triangulate(const gba_triangulation* problem, const gba_options* options,
                            double* points, int32_t* point_status);
/* Device time of the calling thread's last gba_triangulate kernel (ms), when
 * that call had options->profile set; else 0. */
GBA_API double gba_triangulate_last_kernel_ms(void);

/* FMA throughput of the device at its current clocks (TFLOP/s; precision
 * GBA_PRECISION_MIXED = FP32, GBA_PRECISION_FP64 = FP64): the compute roof
 * of the kernels that run on the CUDA cores. */
GBA_API int gba_fma_peak(int32_t precision, int32_t device, double* tflops);

/* ---- library ------------------------------------------------------------ */
GBA_API const char* gba_status_string(int status);
GBA_API const char* gba_version(void);
/* Number of kernels this library has launched since load (all threads). */
GBA_API int64_t gba_kernel_launch_count(void);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* GBA_H_ */
