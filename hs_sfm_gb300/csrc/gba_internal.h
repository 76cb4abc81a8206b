// gba_internal.h -- device data layout of a plan (a batch of bundle-adjustment
// problems resident on one GPU) shared by the kernels and the host planner.
//
// Every problem of a batch is concatenated into global arrays; a single
// problem is a batch of one.  Keys are stored point-major (all keys of a
// point contiguous, sorted by image id), which makes the per-point
// quantities of the Schur complement (V_p, g_p, V_p^-1) register-local.
// Indices on the device are int32 (global key, point, image ids), offsets
// into the dense reduced systems are int64.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include <vector>

#include "../../include/gba.h"

namespace gba {

constexpr int kTile = 32;          // dense Cholesky tile
constexpr int kDfTraceCap = 1024;   // traced tasks per CTA of the dataflow factorization
constexpr int kPcgSlots = 8;        // PCG partial sums per image chunk
constexpr int kImgCamVals = 128;   // per image item: E (6x10), U_c upper (55), g_c (10), pad
constexpr int kKeyChunk = 1024;    // default keys per key work chunk (gba_options.key_item)
constexpr int kPointChunk = 128;   // points per point work chunk
constexpr int kImageChunk = 8;     // images per image work chunk (backsub)
constexpr int kImageItem = 512;    // keys per image-reduce work item (warp each)
constexpr int kPairItem = 1024;    // pairs per Schur-assembly work item
constexpr int kJRStride = 20;      // per key: Jp(6) Ji(12) rw(2)
constexpr int kZStride = 20;       // per key: Z(18) + pad
// Z planes from this mean share of an image's keys in a block's key pairs
constexpr double kZPlanesDensity = 0.2;
// Plans with at least this many keys fork each LM iteration (two streams)
constexpr long long kForkMinKeys = 300000;
constexpr int kItemStride = 44;    // per work item: 36 block + 6 rhs + pad

// Per-problem LM state (device).  Written only by the control kernels.
struct LMState {
  double mu, nu;
  double F, F_new;                 // current / candidate cost
  double dn2, xn2, gd;             // ||delta||^2, ||x||^2, g^T delta
  double er;                       // e^T delta, e = g - (N + mu I) delta (inexact solves)
  double raw;                      // sum of squared plain residuals at the current x
  unsigned long long ginf_bits;    // max |g| as ordered bits (non-negative)
  unsigned long long maxdiag_bits; // max diag(N) as ordered bits
  double initial_cost;
  int iter, accepted, rejected, factor_fail, stop, status;
  int active;     // still iterating
  int parity;     // which x / residual buffer is current
  int relin;      // a linearization is pending
  int evaluate;   // a candidate is pending evaluation
  int factor_ok;  // reduced system factored this iteration
  int first;      // the first linearization (sets mu0)
  int pcg_iters;
  int pad_;
};

// Per-problem constant description (device).
struct ProbInfo {
  int point_begin, num_points;
  int image_begin, num_images;
  int key_begin, num_keys;
  int n;              // reduced system size = 6 * num_ext
  int nt;             // number of kTile tiles of the reduced system
  long long s_off;    // offset of the n x n dense system (row-major)
  int item_begin, num_items;
  int block_begin, num_blocks;
  // reduced-system "images": the real images, then, with free cameras, nc
  // 6-wide parts of each camera's parameters (zero-padded past cps)
  int ext_begin, num_ext;
  int cam_begin, num_cams, cps, nc;
  // fixed groups: bit 0 points, bit 1 images.  A fixed group keeps its
  // values: its Jacobian columns are zero, so its normal blocks are mu I,
  // its gradient and step zero, and it is left out of ||x||
  // (camera_shared_normal_equation_solver.hpp:540-706 solve the same
  // systems without the fixed unknowns).
  int fix;
  int pad_;
};

struct Chunk {       // a contiguous range of one problem's entities
  int prob, begin, end, pad_;
};

struct DevPlan {
  int B;
  int precision;      // GBA_PRECISION_*
  int loss;
  double huber_delta;
  double tau, eps1, eps2;
  double ftol;        // relative cost decrease that stops (0: off)
  int max_iterations;
  int has_key_weights;
  int max_n, max_nt;  // largest reduced system in the batch

  const ProbInfo* prob;
  LMState* state;

  // keys
  int K;
  const int* key_img;        // global image id
  const int* key_pt;         // global point id
  const double2* key_obs;    // observed key
  const double* key_wl;      // [3K] upper factor of the key weight (l00,l10,l11) or null
  // points
  int P;
  const int* pt_key_off;     // [P+1]
  const int* pt_prob;
  // images
  int I;
  const int* img_key_off;    // [I+1]
  const int* img_keys;       // keys of each image, by point
  const int* img_prob;
  const int* img_cam;        // global camera id
  int n_img_items;
  const int4* img_items;     // (image, q begin, q end, prob), <= kImageItem keys
  const int* img_item_off;   // [I+1] items of each image
  double* img_item_partial;  // [items * 28]
  double* cam64[2];          // [C*10]  k1 k2 k3 d1 d2 f s cx cy a, by parity
  float* cam32[2];           // [C*10]  (both parities the same array while cameras are fixed)
  // parameters (double buffered by LMState::parity)
  double* x_pt[2];           // [3P]
  double* x_img[2];          // [6I]
  const double* x0_pt;
  const double* x0_img;
  double* img_rot[2];        // [12I] R (9) + t (3), FP64
  float2* img_rot_ff[2];     // [12I] double-float mirror (mixed path) or null
  float2* x_ff[2];           // [3P] double-float mirror of x_pt (mixed path) or null
  const float2* key_obs_ff;  // [2K] double-float keys (mixed path) or null
  float2* cam_ff[2];         // [10C] double-float cameras, [9] = f * a (mixed path), by parity
  void* img_lin[2];          // [12I] T: r(3) t(3) ct s c a1 a2 pad
  // per key
  void* RW[2];               // [4K] T: rw0 rw1 sqrt(w) pad  (whitened, weighted residual)
  void* JR[2];               // [20K] T, by parity: a candidate's records are formed
                             // with its cost (fuse_lin) and become current if it is accepted
  int fuse_lin;              // 1: the candidate cost kernels write the candidate's records
  void* Z;                   // [20(K+R)] T records, or 9 planes of z_n T pairs (z_planes)
  int z_planes;              // 1: Z as planes, slots image by image (img_keys order)
  long long z_n;             // plane stride in slots (>= K + R)
  // per point
  void* PV;                  // [12P] T: V(6) g(3) pad
  void* PS;                  // [12P] T: Cinv(6) h(3) pad
  // per image (FP64)
  double* U;                 // [36I]
  double* gi;                // [6I]
  // reduced systems
  void* S;                   // T: sum n^2 over problems (lower triangles)
  void* b;                   // T: [6I] rhs -> forward solution -> delta (images)
  void* Linv;                // T: [B * max_nt * kTile^2] inverses of diagonal tiles
  int* factor_flag;          // [B] 0 ok, 1 not positive definite, 2 a bounded wait ran out
  // dataflow factorization (one problem; df_grid == 0: per-column launches)
  int df_grid, df_max_own;
  const int* df_own_off;     // [df_grid + 1] owned tiles of each CTA
  const int2* df_own;        // (i, j) per owned tile, sorted by (j, i) within a CTA
  unsigned* df_flags;        // [nt * nt] epoch at which tile (i, j) was published
  unsigned* df_sync;         // [0] epoch of the last launch, [1] finished CTAs, [2] aborted epoch
  unsigned long long* df_trace; // optional task timeline: [grid][kDfTraceCap][4], or null
  long long df_spin_limit;   // idle polls before a CTA gives up (GBA_ERR_TIMEOUT)
  // cluster backward solve: polls of a step's mbarrier before a warp gives
  // up (GBA_ERR_TIMEOUT), and a step whose delta is never sent (-1: none;
  // set only by tests, through GBA_SOLVE_DROP_STEP)
  long long solve_spin_limit;
  int solve_drop_step;
  // block-Jacobi PCG on the block-sparse reduced system (linear_solver PCG)
  int pcg;                   // 1: PCG instead of the dense factorization
  int pcg_max_iterations;
  double pcg_tol2;           // squared relative residual tolerance
  const int2* blk_gij;       // [n_blocks] global (first, second) image of each block
  const int* img_diag_blk;   // [I] block (i, i) of each image
  const int* adj_off;        // [I + 1] blocks touching each image
  const int2* adj;           // (block, other image << 1 | this image is the block's second)
  void* Sblk;                // T: [n_blocks * 36], row = first image component
  void* Minv;                // T: [I * 36] inverses of the diagonal blocks
  void* pcg_r;               // T: [6I] residual
  void* pcg_z;               // T: [6I] preconditioned residual
  void* pcg_q;               // T: [6I] S p
  void* pcg_p[2];            // T: [6I] search directions (by iteration parity)
  double* pcg_part;          // [kPcgSlots * n_ext_chunks]: p.q, r.z (x2), r.r (x2), b.b, x.r
  int* pcg_done;             // [B] 1 once a problem's inner solve has stopped
  // the PCG iterations as a device-side loop (a CUDA-graph while node) when
  // the plan runs from a graph: pcg_it counts its passes of two iterations;
  // the body is captured on pcg_body_stream.  Null: one launch pair per iteration.
  int* pcg_it;
  unsigned long long* pcg_extra;   // passes run beyond each loop's first (all runs)
  cudaStream_t pcg_body_stream;
  // PCG work chunks over reduced-system images (images, then free cameras'
  // parts; the image chunks when no camera is free) and their problems
  int n_ext_chunks;
  const Chunk* ext_chunks;
  const int* prob_ext_chunk_off;  // [B+1]
  const int* ext_prob;            // [I_ext] problem of each reduced-system image
  // Schur assembly
  const int2* pairs;         // (key_a, key_b) per pair, grouped by block
  const int4* items;         // (block, pair_begin, pair_end, prob)
  const int2* blk_ij;        // (i, j) local image ids per block, i <= j
  const int* blk_prob;       // [n_blocks] problem of each block (plans without free cameras), or null
  long long s_elems;         // elements of S (all problems' dense systems)
  const int* blk_item_off;   // [num_blocks_total + 1] items of each block
  int n_items, n_blocks;
  const int* blk_map;        // per problem I*I dense map (j*I + i), j <= i -> block or -1
  const long long* blk_map_off; // [B]
  double* item_partial;      // [items * kItemStride]
  // work chunks and their partial sums (FP64)
  int n_key_chunks, n_pt_chunks, n_img_chunks;
  int key_z_split;                // CTAs of 256 keys per key chunk in the Z kernel
  const Chunk* key_chunks;
  const Chunk* pt_chunks;
  const Chunk* img_chunks;
  const int* prob_key_chunk_off;  // [B+1]
  const int* prob_pt_chunk_off;   // [B+1]
  const int* prob_img_chunk_off;  // [B+1]
  double* key_chunk_sum;          // [2 * n_key_chunks] cost, sum of squared plain residuals
  // free cameras (camera parameters are unknowns; dense solver).  Camera
  // parameters are kept in the problem's order (the first cps of 10 per
  // camera); Jacobians and the per-image sums use all ten columns
  // [k1 k2 k3 d1 d2 f s cx cy a] and pick the computed ones.
  int free_cams;
  int Ctot;                       // cameras of the plan
  int R;                          // camera records (Z records K .. K+R-1)
  int I_ext;                      // reduced-system images of the plan
  const int* img_ext;             // [I] reduced-system index of each image
  const int4* cam_info;           // [Ctot] (cps if free else 0, mask, problem, ext index of part 0)
  const int* cam_img_off;         // [Ctot + 1] into cam_imgs
  const int* cam_imgs;            // images of each camera, ascending
  const int* prob_cam_off;        // [B + 1] cameras of each problem
  double* x_cam[2];               // [10 * Ctot] by parity
  double* x0_cam;
  void* JC[2];                    // T: [20 K] camera Jacobian, 2 rows x 10 (all parameters), by parity
  const int* pt_rec_off;          // [P + 1] camera records of each point (indices >= K)
  const int2* rec_info;           // [R] (global camera, ext index)
  double* img_item_cam;           // [n_img_items * kImgCamVals] partial sums of image items
  double* img_cam_sum;            // [I * kImgCamVals] the sums of each image's items
  double* Ei;                     // [60 I] J_i^T J_c per image (full columns)
  double* Uc;                     // [100 Ctot] camera normal block, cps x cps, row stride 10
  double* gc;                     // [10 Ctot]
  double* cam_sum;                // [3 Ctot] dn2, xn2, g^T d of the camera step
  // soft constraints on points and images (rows of y after the keys)
  int n_cons;
  const int4* cons;               // (group 0 point / 1 image / 2 camera, global index, parameter, problem)
  const double2* cons_yw;         // (observed value, weight)
  const int* pt_cons_off;         // [P + 1] into cons_by_pt, or null without constraints
  const int* cons_by_pt;
  const int* img_cons_off;        // [I + 1] into cons_by_img
  const int* cons_by_img;
  const int* prob_cons_off;       // [B + 1] rows of each problem
  double* cons_cost;              // [B] constraint and prior terms of the cost at the x of the last cost launch
  // point priors (ground control points): 3 rows each after the constraint rows
  int n_priors;
  const int* pt_prior_off;        // [P + 1] into prior_by_pt, or null without priors
  const int* prior_by_pt;
  const int* prior_pt;            // [n] global point of each prior
  const double* prior_y;          // [3 n] observed coordinates
  const double* prior_info;       // [9 n] inverse covariance, row-major
  const int* prob_prior_off;      // [B + 1] priors of each problem
  double* pt_chunk_sum;           // [3 * n_pt_chunks] dn2, xn2, gd
  double* img_chunk_sum;          // [3 * n_img_chunks]
  unsigned long long* launch_counter; // device-side count (unused: host counts)
  // LM control folded into the producers: the last CTA of a problem to
  // finish k_backsub runs the step decision and the last of the candidate
  // cost the accept decision (no k_ctrl_step / k_ctrl_accept launches).
  // fold_count [2B]: per problem the arrival counters of the two kernels.
  int fold_ctrl;
  unsigned* fold_count;
  // batched dense factorization of small systems (at most 8 tile rows,
  // FP32): one launch of k_chol_small (factor and solve) per iteration
  // instead of the per-column launches
  int chol_small;
};

// A failed CUDA call on the host side of a plan (GBA_ERR_* status).
struct CudaError {
  int status;
};

// Host launchers (gba_kernels.cu).  `T` selects the working precision of
// the Jacobian / Schur stages: float (mixed) or double (plain FP64).
int launch_init(const DevPlan& d, cudaStream_t s);
int launch_image_prep(const DevPlan& d, int which, cudaStream_t s);
int launch_cost(const DevPlan& d, int which, cudaStream_t s);
int launch_ctrl_initial_cost(const DevPlan& d, cudaStream_t s);
// keys = false: the point sums only (the records were formed with the
// accepted candidate's cost)
int launch_linearize(const DevPlan& d, cudaStream_t s, bool keys = true);
int launch_image_reduce(const DevPlan& d, cudaStream_t s);
int launch_ctrl_after_linearize(const DevPlan& d, cudaStream_t s);
int launch_point_schur(const DevPlan& d, cudaStream_t s);
// plan build with Z planes: key_slot [K] = the inverse of img_keys, and the
// assembly's pairs rewritten as slots
int launch_z_slots(const DevPlan& d, int* key_slot, cudaStream_t s);
int launch_assemble(const DevPlan& d, cudaStream_t s);
int launch_assemble_items(const DevPlan& d, cudaStream_t s);
int launch_assemble_S(const DevPlan& d, cudaStream_t s);
int launch_cholesky(const DevPlan& d, cudaStream_t s);
int launch_assemble_blocks(const DevPlan& d, cudaStream_t s);
int launch_pcg_setup(const DevPlan& d, cudaStream_t s);
int launch_pcg_iterations(const DevPlan& d, cudaStream_t s);
int launch_cholesky_factor(const DevPlan& d, cudaStream_t s);
int launch_cholesky_solve(const DevPlan& d, cudaStream_t s);
// Raises the backward solve's shared-memory limit for systems of up to
// max_nt tile rows (before a graph capture); a GBA_* status.
int prepare_cholesky_solve(int max_nt, int precision);
// Readies k_chol_small for systems of up to max_nt tile rows (before a graph
// capture); false when it does not apply (FP64, larger systems).
bool prepare_chol_small(int max_nt, int precision);
// Tile ownership of the dataflow factorization of an nt-tile system for this
// device, or false when it does not fit in shared memory.
bool dataflow_layout(int nt, bool mixed, int device, int* grid, int* max_own,
                     std::vector<int>* own_off, std::vector<int2>* own);
int launch_backsub(const DevPlan& d, cudaStream_t s);
int launch_ctrl_step(const DevPlan& d, cudaStream_t s);
int launch_ctrl_accept(const DevPlan& d, cudaStream_t s);

// Adds kernels launched outside a plan to gba_kernel_launch_count() (gba_plan.cu).
void count_launches(long long n);

// Stage entry points on a plan (gba_kernels.cu): Jacobian blocks in sorted
// key order (T precision), vector function (FP64).
int launch_vector_function(const DevPlan& d, double* y_sorted, cudaStream_t s);
int launch_jacobian_out(const DevPlan& d, double* jp, double* ji, double* jc, cudaStream_t s);
// Key pairs of the reduced system on the device (plans without free
// cameras).  pinfo[q] = (first image, Ie, first code, 0): problem q's image
// pairs (a, c) have the codes first code + a * Ie + c (L codes in all, the
// problems' ranges in order).  count_blocks_on_device counts the pairs per
// code (cnt), numbers the blocks -- the codes with pairs and every
// diagonal, in code order -- into bid [L] (-1 where no block) and returns
// the block list (blk_code = a * Ie + c within the problem, blk_first = its
// first pair; both hold up to the sum of Ie (Ie + 1) / 2), each problem's
// first block (prob_block) and info = (blocks, pairs); qlast is the last
// problem with images, max_ie the largest Ie; off [L] is scratch.
// build_pairs_on_device writes the pairs of every point (pp [P + 1]
// scratch) with their block ids and sorts them stably by block: *out points
// at the sorted pairs (one of the two value buffers).  pairs_sort_scratch
// sizes hist and scratch; scratch for count_blocks_on_device holds
// scan_scratch_ints(L).  Both return the launch count (-1: bad arguments).
long long scan_scratch_ints(long long L);
int count_blocks_on_device(int nprob, int qlast, int max_ie, int P, const int4* d_pinfo, const int* d_pt_key_off,
                           const int* d_key_img, const int* d_pt_prob, long long L, int* d_cnt, int* d_bid,
                           int* d_off, int* d_scratch, int* d_blk_code, int* d_blk_first, int* d_prob_block,
                           int* d_info, cudaStream_t s);
int build_pairs_on_device(int P, int nblocks, const int4* d_pinfo, const int* d_pt_key_off, const int* d_key_img,
                          const int* d_pt_prob, int* d_pp, const int* d_bid, long long n, int* d_keys0,
                          int2* d_vals0, int* d_keys1, int2* d_vals1, int* d_hist, int* d_scratch, int* d_bad,
                          int2** out, cudaStream_t s);
void pairs_sort_scratch(long long n, int P, long long* hist_ints, long long* scratch_ints);
// The observed keys split into double-float pairs (mixed path) on the device.
int launch_split_keys(const DevPlan& d, float2* out, cudaStream_t s);
// Every problem's current x (x0 before a run) into out [3P + 6I + 10 Ctot (free cameras)].
int launch_gather_x(const DevPlan& d, int ran, double* out, cudaStream_t s);

}  // namespace gba
